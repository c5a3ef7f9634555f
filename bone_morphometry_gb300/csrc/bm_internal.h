// Internal definitions shared by the CUDA translation units of libbm_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>
#include <vector>

#include "bm.h"

namespace bm {

// "No site on this line" in the EDT passes: larger than any squared distance
// (< 2^31), yet adding a scan offset dp^2 (dp <= 67) to it cannot wrap.
constexpr uint32_t kInfSq = 0xF0000000u;

// Selection of the phase from the inputs, evaluated inside the first EDT pass
// (edt.rs:19-24 and volume.rs:84-105).
enum SelMode : int {
  SEL_FOREGROUND = 0,  // a != 0
  SEL_BACKGROUND = 1,  // a == 0
  SEL_BONE_IN_ROI = 2,    // roi != 0 && bone != 0       (Tb.Th phase)
  SEL_MARROW_IN_ROI = 3,  // roi != 0 && bone == 0       (Tb.Sp phase)
};

struct Dims {
  int w, h, d;
  __host__ __device__ long long n() const { return (long long)w * h * d; }
  __host__ __device__ int nw() const { return (w + 31) >> 5; }  // 32-bit words per x row of a bitmask
};

// Unsigned 32-bit division by a fixed divisor d >= 2 through a multiply
// (the round-up method of Granlund and Montgomery): with l = ceil(log2 d) and
// m = floor(2^32 (2^l - d) / d) + 1, n / d = (t + ((n - t) >> 1)) >> (l - 1)
// where t = mulhi(m, n), for every 32-bit n.
struct FastDiv {
  uint32_t d, m, s;
  static FastDiv of(uint32_t div) {
    FastDiv f;
    f.d = div;
    uint32_t l = 0;
    while ((1ull << l) < div) ++l;
    f.m = (uint32_t)(((1ull << 32) * ((1ull << l) - div)) / div + 1);
    f.s = l - 1;
    return f;
  }
#ifdef __CUDACC__
  __device__ __forceinline__ uint32_t div(uint32_t n) const {
    const uint32_t t = __umulhi(m, n);
    return (t + ((n - t) >> 1)) >> s;
  }
#endif
};

#ifdef __CUDACC__
// floor(sqrt(v)) for v < 2^30 from the hardware reciprocal square root: the
// estimate (float)v * rsqrt((float)v) is within 0.01 of sqrt(v) there (the
// float conversion and the reciprocal root are each within a few ulp), so one
// integer correction step each way makes the floor exact.
__device__ __forceinline__ uint32_t isqrt30(uint32_t v) {
  const float f = (float)v;
  uint32_t r = (uint32_t)(f * rsqrtf(fmaxf(f, 1.0f)));
  r -= (r * r > v) ? 1u : 0u;
  r += ((r + 1) * (r + 1) <= v) ? 1u : 0u;
  return r;
}
#endif

// Linear voxel index -> (x, y, z) without hardware division.
struct VoxelDecoder {
  FastDiv w, wh;
  static VoxelDecoder of(const Dims& dm) {
    return VoxelDecoder{FastDiv::of((uint32_t)dm.w), FastDiv::of((uint32_t)dm.w * (uint32_t)dm.h)};
  }
#ifdef __CUDACC__
  __device__ __forceinline__ void operator()(uint32_t idx, int& x, int& y, int& z) const {
    const uint32_t zq = wh.div(idx);
    const uint32_t rem = idx - zq * wh.d;
    const uint32_t yq = w.div(rem);
    z = (int)zq;
    y = (int)yq;
    x = (int)(rem - yq * w.d);
  }
#endif
};

// Exact-sum accumulator for the statistics: per f32 exponent the sum of the
// 24-bit mantissas and of the 48-bit squared mantissas (split into two 24-bit
// halves), plus count and maximum.  Exact for < 2^34 values.
struct StatsAccum {
  unsigned long long sum_m[256];
  unsigned long long sq_hi[256];
  unsigned long long sq_lo[256];
  unsigned long long count;
  unsigned int max_bits;
  unsigned int pad;
  // Fixed-point totals (filled on the host from FixedPartial records):
  // sum of m * 2^(e - e_lo) and of m^2 * 2^(2 (e - e_lo)) over the values
  // whose exponent e lies in [e_lo, e_lo + kFixedSpan]; fx_elo = 0: none.
  unsigned long long fx_s1[2];
  unsigned long long fx_s2[3];
  int fx_elo;
  int fx_pad;
};

// Exponent span of the fixed-point statistics path (values of one map lie
// within 2^16 of their smallest possible value).
constexpr int kFixedSpan = 20;

// One CTA's fixed-point statistics: s1 (sum of shifted mantissas) and the
// 128-bit sum of their squares.
struct FixedPartial {
  unsigned long long s1;
  unsigned long long s2lo, s2hi;
  unsigned long long pad;
};

// Tile of the tile-owned sphere fill: 32 x (16, 32 or 64) x 16 voxels (x, y, z).
constexpr int kFillTX = 32;
constexpr int kFillTZ = 16;
// Volumes of at least kFillTallMinVoxels fill 64-row tiles by default, those
// of at least kFillMidMinVoxels 32-row tiles, smaller ones 16-row tiles.
// Measured on the 512^3 generator's specimens at other edges (ms per fill
// launch, 16 / 32 / 64 rows): 192^3 0.65 / 0.85 / 1.36, 256^3 1.06 / 1.08 /
// 1.51, 320^3 1.83 / 1.57 / 1.66, 384^3 3.15 / 2.65 / 2.40, 512^3 - / 5.6 / 5.1.
constexpr long long kFillTallMinVoxels = 3ll << 24;
constexpr long long kFillMidMinVoxels = 1ll << 24;

// Largest r^2 whose sphere lattice points the tile fill tabulates (radius 256);
// volumes with larger distances use the per-ball atomic fill.
constexpr uint32_t kSurfMaxR2 = 65536;
// Largest volume whose Tb.Th and Tb.Sp phases run side by side (bm_tbth_tbsp).
constexpr long long kSplitMaxVoxels = 1ll << 28;

// Device-side sizes of one phase's fill binning.
struct FillInfo {
  uint32_t nR;                         // distinct ridge r^2 values
  uint32_t pad;
  unsigned long long total_entries;    // (ball, tile) pairs
  unsigned long long site_steps;       // sum over ridges of ceil(2 pi ceil(sqrt(r^2)) / 16): half-warp steps of
                                       // the site kernel over the spheres' lattice points (about 2 pi r each)
  unsigned long long ridges;           // ridge count
};

// Device scratch owned by a context, grown on demand and reused across calls.
struct Buffer {
  void* ptr = nullptr;
  size_t bytes = 0;
};

struct Counters {  // device-side counters of one phase
  unsigned long long sites;     // non-selected voxels
  unsigned long long selected;  // selected voxels
  unsigned long long ridges;
  unsigned int rmax;
  unsigned int status;          // nonzero: a bounded wait gave up / capacity exceeded
  unsigned int tile_next[2];    // next tile to take: ridge pass, cleanup pass (dynamic tile scheduling)
};

// Kernel families timed by the context's profiler (bm_profile_*).
enum KernelFamily : int {
  KF_COUNT_ROI = 0,
  KF_EDT_X,
  KF_EDT_Y,
  KF_EDT_Z,
  KF_TEMPLATES,
  KF_RIDGE,
  KF_FILL,
  KF_FILL_RANK,
  KF_FILL_BIN,
  KF_FILL_SITES,
  KF_CLEAN_FINAL,
  KF_QUANTILE,
  KF_STATS_ORDER,
  KF_COUNT
};

struct ProfRec {
  int family;
  cudaEvent_t start, stop;
};

class Pool;  // worker pool of the batched / served forms (serve.cpp)
void pool_destroy(Pool* p);

}  // namespace bm

struct bm_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  // second context (own stream and buffers) that runs the marrow phase of
  // bm_tbth_tbsp while this one runs the bone phase; created on first use
  bm_ctx* twin = nullptr;
  cudaEvent_t inputs_ready = nullptr;
  bool split_phases = true;  // false: both phases on this context, one after the other
  int fill_rows = 0;         // rows of y per fill tile: 0 = by volume size, or 16 / 32 / 64
  int site_method = 0;       // BM_SITES_*
  long long wait_cycles = -1;  // first-wait limit of the bounded device waits (< 0: default)
  std::mutex mu;
  std::string last_error;
  unsigned long long launches = 0;
  int num_sms = 0;

  // cached search-template table: lut[r2] = {t100, t110, t111, 0}
  bm::Buffer lut;
  uint32_t lut_max = 0;  // entries 0..lut_max are valid
  bm::Buffer lutf;       // f32 diameters 2*sqrt(r2), r2 = 0..lut_max

  bm::Buffer in_a, in_b;       // staged host inputs
  bm::Buffer dist, dist2;      // u32 EDT ping/pong
  bm::Buffer edtmap, chainmap; // u32 z-pass output kept apart from the x pass's, and the site-chain map
  bm::Buffer stack;            // EDT line scratch
  bm::Buffer fillmap;          // u32 propagated r^2
  bm::Buffer selbits, ridgebits; // row-padded bitmasks: selected voxels, ridge voxels
  bm::Buffer ridges;           // ridge records
  bm::Buffer counters;         // bm::Counters
  bm::Buffer roicount;         // ROI and bone-in-ROI voxel counts (the bails of bm_tbth_tbsp)
  bm::Buffer accum;            // bm::StatsAccum
  bm::Buffer cpart;            // bm::FixedPartial per cleanup CTA
  bm::Buffer outmap;           // f32 output staging
  bm::Buffer outmap2;
  bm::Buffer host_pinned;      // pinned staging for small readbacks
  bm::Buffer occ, rank, rvals; // per-r^2 flags, ranks, rank -> r^2
  bm::Buffer rgeo;             // rank -> {r^2, ceil sqrt, floor sqrt, 0}
  bm::Buffer fillinfo;         // bm::FillInfo
  bm::Buffer bincounts, binoffsets, binentries, scanscratch;
  // cached sphere lattice-point table for r2 in [0, surf_max]
  bm::Buffer surf_off, surf_pts;
  bm::Buffer redo;             // per-line flags of the windowed EDT passes
  bm::Buffer qhist, qtargets, qmap;  // quantile histograms, targets, map scratch
  bm::Buffer ordmap, ordscratch, ordout;  // f32 map for the ordered sums, their scratch, their two results
  bm::Buffer tileorder;        // the fill's tile order (heaviest first) and its bucket counts
  uint32_t surf_max = 0;

  // profiler: CUDA events around every library launch while enabled
  // bm_tbth_tbsp's upload pipeline: a copy stream and one event per slab of
  // planes (created on first use)
  cudaStream_t upload_stream = nullptr;
  std::vector<cudaEvent_t> slab_ready;

  bool profiling = false;
  std::vector<bm::ProfRec> prof;
  std::vector<cudaEvent_t> event_pool;
  double prof_ms[bm::KF_COUNT] = {};
  unsigned long long prof_n[bm::KF_COUNT] = {};

  // worker pool used by bm_batch_tbth_tbsp (created on first use)
  std::mutex pool_mu;
  bm::Pool* pool = nullptr;
  int workers = 4;
};

namespace bm {
// Device bytes currently cached by a context's buffers.
size_t cached_bytes(const bm_ctx* ctx);
}  // namespace bm
