// Host-side launchers of the device kernels (one declaration per kernel family).
#pragma once

#include "bm_internal.h"

namespace bm {

// Grid of a persistent (tile-looping) kernel: as many CTAs as the current
// device keeps resident at once, at most one per tile.
template <typename Kernel>
inline unsigned resident_grid(Kernel kernel, int threads, size_t smem, long long tiles) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem);
  long long g = (long long)(per > 0 ? per : 1) * (sms > 0 ? sms : 1);
  if (g > tiles) g = tiles;
  if (g < 1) g = 1;
  return (unsigned)g;
}

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

// Windowed y (axis 1) / z (axis 2) pass; lines it cannot bound are recomputed
// by the lower-envelope kernel (redo: one byte per line, scratch as above).
// wait_cycles: limit of the TMA copy's first bounded wait (< 0: the default,
// about 2 s); a block that gives up sets ctr->status.
cudaError_t launch_edt_window(int axis, const uint32_t* in, uint32_t* out, Dims dm, void* scratch, uint8_t* redo,
                              Counters* ctr, long long wait_cycles, cudaStream_t s, unsigned long long* launches);

// Search-template table entries lut[r2] for r2 in [lo, hi]:
// {scan_cube(1,0,0), scan_cube(1,1,0), scan_cube(1,1,1), f32 bits of 2*sqrt(r2)}.
cudaError_t launch_lut(uint4* lut, uint32_t lo, uint32_t hi, cudaStream_t s, unsigned long long* launches);

// Distance-ridge extraction: appends {linear index, r2} records and, when occ
// is not null, sets occ[r2] = 1 for every ridge r2.  When ridgebits is not null, writes the ridge bitmask
// rows (layout of selbits) of every tile with a selected voxel (the caller
// zeroes it first).
cudaError_t launch_ridges(const uint32_t* dist, const uint32_t* selbits, Dims dm, const uint4* lut, uint2* ridges,
                          Counters* ctr, uint32_t* occ, uint32_t* ridgebits, cudaStream_t s,
                          unsigned long long* launches);

// Site values by reverse chain passes: the non-selected voxels a ridge sphere
// reaches are exactly the nearest sites of the ridge voxel, reached through
// the argmins of the z, y and x passes.  launch_chain_z: for every ridge
// voxel c (ridgebits) and every z' with g(x, y, z') + (z - z')^2 = m(c),
// chain(x, y, z') = max(., m(c)) (chain zeroed by the caller).
// launch_chain_y: for every (x, y, z') with chain > 0 and every y' with
// f(x, y', z') + (y - y')^2 = g(x, y, z'), the x pass's nearest sites x' of
// (x, y', z') get sites(x', y', z') = max(., chain): run on the tile fill's
// map, whose non-selected voxels are 0, it adds what launch_sites would.
// f, g, m: the x, y and z pass outputs.  halo: rows staged on each side, at
// least isqrt(largest ridge r2) + 1; the largest ridge r2 must be below
// kChainMaxR2.
constexpr int kChainMaxR2 = 2048;
constexpr int kChainMaxHalo = 46;  // isqrt(kChainMaxR2 - 1) + 1
cudaError_t launch_chain_z(const uint32_t* g, const uint32_t* m, const uint32_t* ridgebits, uint32_t* chain, Dims dm,
                           int halo, cudaStream_t s, unsigned long long* launches);
cudaError_t launch_chain_y(const uint32_t* f, const uint32_t* g, const uint32_t* chain, const uint32_t* selbits,
                           uint32_t* sites, Dims dm, int halo, cudaStream_t s, unsigned long long* launches);

// Sphere fill: atomic max of r2 over every voxel of each ridge ball (any phase).
cudaError_t launch_fill(const uint2* ridges, const Counters* ctr, unsigned long long max_ridges, Dims dm,
                        uint32_t* fillmap, cudaStream_t s, unsigned long long* launches);

// Fused cleanup passes 1 and 2, phase mask, optional f32 map, exact statistics.
// dia: f32 diameters 2*sqrt(r2) by r2 (launch_dia_table).
// Values whose f32 exponent lies in [e_lo, e_lo + kFixedSpan] are summed in
// fixed point, one FixedPartial per CTA in part[0 .. *grid); the others go to
// acc's per-exponent sums.  At most kCleanupMaxGrid CTAs.
constexpr unsigned kCleanupMaxGrid = 4096;
// tile_next: a zeroed counter the CTAs take tiles from.
cudaError_t launch_cleanup(const uint32_t* fillmap, const uint32_t* selbits, Dims dm, const float* dia, float scale,
                           float* outmap, StatsAccum* acc, FixedPartial* part, int e_lo, unsigned* tile_next,
                           unsigned* grid, cudaStream_t s, unsigned long long* launches);
cudaError_t launch_dia_table(const uint4* lut, uint32_t n, float* dia, cudaStream_t s, unsigned long long* launches);

// Tile-owned fill (fill.cu).
// Rows of y per fill tile: 64 for volumes of at least kFillTallMinVoxels (fewer
// ball entries per voxel), 32 from kFillMidMinVoxels, else 16 (more tiles: a
// small volume's fill is bound by its tiles' serial chains); requested = 16,
// 32 or 64 forces it.
int fill_tile_rows(Dims dm, int requested);
long long fill_tile_count(Dims dm, int ty);
size_t scan_scratch_words(long long n);
// Exclusive scan of n u32 values (out may alias in); scratch of scan_scratch_words(n).
cudaError_t launch_scan(const uint32_t* in, uint32_t* out, long long n, uint32_t* scratch, cudaStream_t s,
                        unsigned long long* launches);
// occ[0..rmax+1] (occ[rmax+1] == 0) -> rank_desc / rvals / info->nR.
// rgeo[rank] = {r2, ceil sqrt, floor sqrt, 0} for every rank.
cudaError_t launch_rank(const uint32_t* occ, uint32_t* rank_desc, uint32_t rmax, uint32_t* rvals, uint4* rgeo,
                        FillInfo* info, uint32_t* scan_scratch, cudaStream_t s, unsigned long long* launches);
// ty: the fill tile's rows of y (fill_tile_rows).
cudaError_t launch_bin(bool count, const uint2* ridges, const Counters* ctr, unsigned long long max_ridges,
                       const uint32_t* rank_desc, FillInfo* info, Dims dm, int ty, uint32_t* counts,
                       const uint32_t* offsets, uint32_t* entries, cudaStream_t s, unsigned long long* launches);
// Sphere lattice-point table: count (surf_cnt[r2]) or fill (surf_pts from surf_off[r2]) for r2 in [lo, hi].
cudaError_t launch_surf(bool count, uint32_t lo, uint32_t hi, uint32_t* surf_cnt, const uint32_t* surf_off,
                        uint32_t* surf_pts, cudaStream_t s, unsigned long long* launches);
// Selected voxels of every tile from the binned balls; non-selected voxels get 0.
// selbits: the phase's row-padded selection bitmask (edt_x output).
// order_scratch: tile_order_words(dm, ty) words (the tiles' processing order).
size_t tile_order_words(Dims dm, int ty);
cudaError_t launch_tile_fill(const uint32_t* entries, const uint32_t* offsets, const uint32_t* rvals,
                             const uint4* rgeo, const FillInfo* info, const uint32_t* selbits, Dims dm, int ty,
                             uint32_t* order_scratch, uint32_t* fillmap, cudaStream_t s, unsigned long long* launches);
// Non-selected voxels on each ridge's sphere: atomic max of r2 (after the tile
// fill).  surf_off / surf_pts: the lattice-point table covering every ridge r2;
// small: 8 lanes per ridge instead of 16 (spheres of about 40 points or fewer).
cudaError_t launch_sites(const uint2* ridges, const Counters* ctr, unsigned long long max_ridges,
                         const uint32_t* selbits, const uint32_t* surf_off, const uint32_t* surf_pts, bool small,
                         Dims dm, uint32_t* fillmap, cudaStream_t s, unsigned long long* launches);

// The sum and the sum of squares of x = f32(raw * scale) as f64 over the finite
// positive raw values of map[0 .. n), each accumulated in index order with one
// f64 rounding per value -- the reference's own sequence (metrics.rs:215-224),
// reproduced exactly (ordered.cu).  out[0] = sum, out[1] = sum of squares.
// maxbits: device pointer to the f32 bits of the largest such value (the
// statistics accumulator's max_bits), which scales the approximate sums.
size_t ordered_sum_scratch_bytes(long long n);
cudaError_t launch_ordered_sums(const float* map, long long n, float scale, const uint32_t* maxbits, void* scratch,
                                double* out, cudaStream_t s, unsigned long long* launches);

// Exact moment sums of f32(raw * scale) over the finite positive raw values.
cudaError_t launch_moments(const float* map, long long n, float scale, StatsAccum* acc, cudaStream_t s,
                           unsigned long long* launches);
// Quantiles (quantile.cu): histogram of the high 16 bits of the positive finite
// f32 values, and of the low 16 bits for values whose high bits equal one of
// ntarget (<= 16) targets (hist laid out [target][65536]).
cudaError_t launch_hist_hi(const float* map, long long n, uint32_t* hist, cudaStream_t s, unsigned long long* launches);
cudaError_t launch_hist_lo(const float* map, long long n, const uint32_t* targets, int ntarget, uint32_t* hist,
                           cudaStream_t s, unsigned long long* launches);

}  // namespace bm
