// Host-side launchers of the device kernels (one declaration per kernel family).
#pragma once

#include "bm_internal.h"

namespace bm {

// Bytes of device scratch the EDT line passes need for a volume.
size_t edt_scratch_bytes(Dims dm);

// First EDT pass (x rows): phase selection from the inputs (mode), the 1-D
// distance to the nearest non-selected voxel of the row, squared (kInfSq when
// the row has none), the row-padded selection bitmask, and the site count.
cudaError_t launch_edt_x(const uint8_t* a, const uint8_t* b, int mode, Dims dm, uint32_t* out,
                         uint32_t* selbits, Counters* ctr, cudaStream_t s, unsigned long long* launches);

// Lower-envelope pass along y (axis 1) or z (axis 2).  The z pass also
// records the maximum squared distance in ctr->rmax.
cudaError_t launch_edt_line(int axis, const uint32_t* in, uint32_t* out, Dims dm, void* scratch,
                            Counters* ctr, cudaStream_t s, unsigned long long* launches);

// Search-template table entries lut[r2] for r2 in [lo, hi]:
// {scan_cube(1,0,0), scan_cube(1,1,0), scan_cube(1,1,1), f32 bits of 2*sqrt(r2)}.
cudaError_t launch_lut(uint4* lut, uint32_t lo, uint32_t hi, cudaStream_t s, unsigned long long* launches);

// Distance-ridge extraction: appends {linear index, r2} records.
cudaError_t launch_ridges(const uint32_t* dist, Dims dm, const uint4* lut, uint2* ridges,
                          Counters* ctr, cudaStream_t s, unsigned long long* launches);

// Sphere fill: atomic max of r2 over every voxel of each ridge ball (any phase).
cudaError_t launch_fill(const uint2* ridges, const Counters* ctr, unsigned long long max_ridges, Dims dm,
                        uint32_t* fillmap, cudaStream_t s, unsigned long long* launches);

// Surface cleanup pass 1 as a bitmask: nonzero voxel with no zero 26-neighbour.
cudaError_t launch_interior_bits(const uint32_t* fillmap, Dims dm, uint32_t* posbits, cudaStream_t s,
                                 unsigned long long* launches);

// Cleanup pass 2, phase mask, optional f32 map, exact statistics.
cudaError_t launch_final(const uint32_t* fillmap, const uint32_t* posbits, const uint32_t* selbits, Dims dm,
                         const uint4* lut, float scale, float* outmap, StatsAccum* acc, cudaStream_t s,
                         unsigned long long* launches);

}  // namespace bm
