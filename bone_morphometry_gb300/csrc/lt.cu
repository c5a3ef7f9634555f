// Local thickness on sm_103a (local_thickness.rs:16-358): search templates,
// distance ridge, sphere fill, surface cleanup, phase mask and the exact
// statistics of the scaled map (metrics.rs:204-241).
#include "kernels.h"

namespace bm {

namespace {

// floor(sqrt(v)) exactly: float estimate, then integer fix-up (same contract
// as integer_sqrt, local_thickness.rs:339-348).
__device__ __forceinline__ uint32_t isqrt_u32(uint32_t v) {
  uint32_t r = (uint32_t)sqrtf((float)v);
  while ((unsigned long long)(r + 1) * (r + 1) <= v) ++r;
  while ((unsigned long long)r * r > v) --r;
  return r;
}

__device__ __forceinline__ uint32_t csqrt_u32(uint32_t v) {  // ceiling_sqrt, :351-358
  const uint32_t f = isqrt_u32(v);
  return f * f == v ? f : f + 1;
}

// One warp per r^2: lanes split k, loop j; the three offsets of
// create_templates (local_thickness.rs:67-73) share one integer sqrt.
__global__ void __launch_bounds__(256) lut_kernel(uint4* __restrict__ lut, uint32_t lo, uint32_t hi) {
  const int lane = threadIdx.x & 31;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long rr = (long long)lo + wid; rr <= (long long)hi; rr += nwarps) {
    const uint32_t R = (uint32_t)rr;
    const uint32_t rad = isqrt_u32(R) + 1;
    uint32_t m0 = 0, m1 = 0, m2 = 0;
    for (uint32_t k = lane; k <= rad; k += 32) {
      const uint32_t kk = k * k;
      if (kk > R) break;
      const uint32_t k1 = (k + 1) * (k + 1);
      for (uint32_t j = 0; j <= rad; ++j) {
        const uint32_t kj = kk + j * j;
        if (kj > R) break;
        const uint32_t i1 = isqrt_u32(R - kj) + 1;
        const uint32_t ii = i1 * i1;
        const uint32_t j1 = (j + 1) * (j + 1);
        m0 = max(m0, kk + j * j + ii);
        m1 = max(m1, kk + j1 + ii);
        m2 = max(m2, k1 + j1 + ii);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      m0 = max(m0, __shfl_xor_sync(0xffffffffu, m0, o));
      m1 = max(m1, __shfl_xor_sync(0xffffffffu, m1, o));
      m2 = max(m2, __shfl_xor_sync(0xffffffffu, m2, o));
    }
    if (lane == 0) {
      // (2.0_f64 * sqrt(r2 as f64)) as f32, local_thickness.rs:206
      const float dia = __double2float_rn(2.0 * sqrt((double)R));
      lut[R] = make_uint4(m0, m1, m2, __float_as_uint(dia));
    }
  }
}

// One warp per ridge ball; lanes take the (z, y) rows of the clipped box and
// walk their chord |dx| <= isqrt(r2 - dy^2 - dz^2) (local_thickness.rs:172-202).
__global__ void __launch_bounds__(256)
fill_kernel(const uint2* __restrict__ ridges, const Counters* __restrict__ ctr, Dims dm,
            uint32_t* __restrict__ fillmap) {
  const unsigned long long nr = ctr->ridges;
  const int lane = threadIdx.x & 31;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long sl = (long long)dm.w * dm.h;
  for (long long i = wid; i < (long long)nr; i += nwarps) {
    const uint2 rec = ridges[i];
    const long long idx = rec.x;
    const uint32_t R = rec.y;
    const int z = (int)(idx / sl);
    const long long rem = idx - (long long)z * sl;
    const int y = (int)(rem / dm.w);
    const int x = (int)(rem - (long long)y * dm.w);
    const int rad = (int)csqrt_u32(R);
    const int zs = max(z - rad, 0), ze = min(z + rad, dm.d - 1);
    const int ys = max(y - rad, 0), ye = min(y + rad, dm.h - 1);
    const int ny = ye - ys + 1;
    const int rows = (ze - zs + 1) * ny;
    for (int r = lane; r < rows; r += 32) {
      const int zz = zs + r / ny;
      const int yy = ys + r % ny;
      const uint32_t dz = (uint32_t)abs(zz - z), dy = (uint32_t)abs(yy - y);
      const uint32_t dyz = dz * dz + dy * dy;
      if (dyz > R) continue;
      const int half = (int)isqrt_u32(R - dyz);
      const int x0 = max(x - half, 0), x1 = min(x + half, dm.w - 1);
      uint32_t* rowp = fillmap + ((long long)zz * dm.h + yy) * dm.w;
      for (int xx = x0; xx <= x1; ++xx) atomicMax(rowp + xx, R);
    }
  }
}



// NEIGHBORS_26 of local_thickness.rs:285-312 (Fiji's visitation order), which
// fixes the order of the f32 sum in cleanup pass 2; constant so that the
// unrolled loop addresses shared memory with immediate offsets.
__device__ constexpr signed char kN26c[26][3] = {
    {0, 0, -1}, {0, 0, 1},  {0, -1, 0}, {0, 1, 0},   {-1, 0, 0},  {1, 0, 0},  {0, 1, -1},
    {0, 1, 1},  {1, -1, 0}, {1, 1, 0},  {-1, 0, 1},  {1, 0, 1},   {0, -1, -1}, {0, -1, 1},
    {-1, -1, 0}, {-1, 1, 0}, {-1, 0, -1}, {1, 0, -1}, {1, 1, 1},   {1, -1, 1}, {-1, 1, 1},
    {-1, -1, 1}, {1, 1, -1}, {1, -1, -1}, {-1, 1, -1}, {-1, -1, -1}};

// Fused surface cleanup (local_thickness.rs:210-281), phase mask (:31-43),
// f32 calibration and exact moment sums (metrics.rs:215-226) on a tile of
// 32 x 16 x 8 voxels (the staged halo is 2.1 times the tile; 2.5 times at
// 32 x 8 x 8).  The r^2 map is staged with a halo of 2 (out-of-volume
// voxels hold kOob, which is neither zero nor interior -- look() returns -1
// there).  Pass 1 ("nonzero and no zero 26-neighbour") is a 3x3x3 erosion of
// the nonzero mask, done on 64-bit row masks (x, then y, then z); pass 2 sums
// the diameters of interior neighbours in NEIGHBORS_26 order with IEEE f32
// adds and one IEEE division, exactly as the reference.
constexpr int kCTX = 32, kCTY = 16, kCTZ = 8;
constexpr int kCH = 2;                       // halo
constexpr int kCSX = kCTX + 2 * kCH;         // 36
constexpr int kCSY = kCTY + 2 * kCH;         // 20
constexpr int kCSZ = kCTZ + 2 * kCH;         // 12
constexpr uint32_t kOob = 0xffffffffu;
constexpr int kCleanThreads = 256;
static_assert(kCTZ * kCTY <= kCleanThreads, "the empty-tile check reads one selection word per thread");

__device__ __forceinline__ void flush_run(StatsAccum& sacc, uint32_t e, unsigned long long& s1,
                                          unsigned long long& sh, unsigned long long& sl) {
  if (s1) {
    atomicAdd(&sacc.sum_m[e], s1);
    atomicAdd(&sacc.sq_hi[e], sh);
    atomicAdd(&sacc.sq_lo[e], sl);
    s1 = sh = sl = 0;
  }
}

// One value of the calibrated map into this thread's statistics: in fixed
// point when its exponent is within kFixedSpan of e_lo (no atomics), else into
// the per-exponent run.
__device__ __forceinline__ void add_value(float val, float scale, int e_lo, unsigned long long& cnt, uint32_t& mx,
                                          unsigned long long& fx1, unsigned __int128& fx2, uint32_t& run_e,
                                          unsigned long long& run_s1, unsigned long long& run_sh,
                                          unsigned long long& run_sl, StatsAccum& sacc) {
  const uint32_t bits = __float_as_uint(__fmul_rn(val, scale));
  ++cnt;
  mx = max(mx, bits);
  uint32_t e = bits >> 23, m = bits & 0x7fffffu;
  if (e) m |= 0x800000u;
  else e = 1;
  const uint32_t sh = e - (uint32_t)e_lo;
  if (sh <= (uint32_t)kFixedSpan) {
    const unsigned long long m64 = m;
    fx1 += m64 << sh;
    fx2 += (unsigned __int128)(m64 * m64) << (2 * sh);
    return;
  }
  if (e != run_e) {  // a new exponent: flush this thread's run
    flush_run(sacc, run_e, run_s1, run_sh, run_sl);
    run_e = e;
  }
  const unsigned long long sq = (unsigned long long)m * m;
  run_s1 += m;
  run_sh += sq >> 24;
  run_sl += sq & 0xffffffu;
}

__global__ void __launch_bounds__(kCleanThreads, 3)
cleanup_tile_kernel(const uint32_t* __restrict__ fm, const uint32_t* __restrict__ selbits, Dims dm,
                    const float* __restrict__ dia, float scale, float* __restrict__ outmap,
                    StatsAccum* __restrict__ acc, FixedPartial* __restrict__ part, int e_lo, int ntx, int nty,
                    int ntz, unsigned* __restrict__ tile_next) {
  __shared__ uint32_t T[kCSZ * kCSY * kCSX];         // f32 diameter bits of the r^2 map
  __shared__ uint32_t s_tile;
  __shared__ unsigned long long nz[kCSZ * kCSY];     // bit x: T != 0 (or out of volume)
  __shared__ unsigned long long inr[kCSZ * kCSY];    // bit x: interior (pass-1 value kept)
  __shared__ unsigned long long own[kCSZ * kCSY];    // bit x: T != 0 inside the volume
  __shared__ StatsAccum sacc;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < 256; i += kCleanThreads) {
    sacc.sum_m[i] = 0;
    sacc.sq_hi[i] = 0;
    sacc.sq_lo[i] = 0;
  }
  if (tid == 0) {
    sacc.count = 0;
    sacc.max_bits = 0;
  }
  const int nw = dm.nw();
  unsigned long long cnt = 0;
  uint32_t mx = 0;
  // this thread's run of values with one f32 exponent: sums of the mantissas
  // and of the two 24-bit halves of their squares (flushed when the exponent
  // changes, so a thread's values are added once, without warp votes)
  uint32_t run_e = 0;
  unsigned long long run_s1 = 0, run_sh = 0, run_sl = 0;
  // fixed-point sums of the values with exponent in [e_lo, e_lo + kFixedSpan]
  unsigned long long fx1 = 0;
  unsigned __int128 fx2 = 0;
  const long long ntiles = (long long)ntx * nty * ntz;
  // tiles are taken from a counter as CTAs free up (their costs vary widely)
  for (;;) {
    __syncthreads();  // every thread has read s_tile
    if (tid == 0) s_tile = atomicAdd(tile_next, 1u);
    __syncthreads();
    const long long tile = s_tile;
    if (tile >= ntiles) break;
    const int tx = (int)(tile % ntx), ty = (int)((tile / ntx) % nty), tz = (int)(tile / ((long long)ntx * nty));
    const int x0 = tx * kCTX, y0 = ty * kCTY, z0 = tz * kCTZ;
    // a tile without selected voxels (outside the ROI, say) has a zero output and
    // no statistics: skip its staging
    bool any_sel = false;
    if (tid < kCTZ * kCTY) {
      const int z = z0 + tid / kCTY, y = y0 + tid % kCTY;
      if (z < dm.d && y < dm.h) any_sel = selbits[((long long)z * dm.h + y) * nw + tx] != 0u;
    }
    if (!__syncthreads_or(any_sel)) {
      if (outmap) {
        for (int r = warp; r < kCTZ * kCTY; r += kCleanThreads / 32) {
          const int z = z0 + r / kCTY, y = y0 + r % kCTY, x = x0 + lane;
          if (z < dm.d && y < dm.h && x < dm.w) outmap[((long long)z * dm.h + y) * dm.w + x] = 0.0f;
        }
      }
      continue;
    }
    // stage the r^2 map with halo 2: one row of 36 per warp step.  Each warp
    // has 18 rows; their loads are issued in batches of 3 before any use, so
    // the latencies overlap.
    constexpr int kRowsPerWarp = kCSZ * kCSY / (kCleanThreads / 32);  // 30
    constexpr int kBatch = 3;
    static_assert(kCSZ * kCSY % (kCleanThreads / 32) == 0 && kRowsPerWarp % kBatch == 0, "staging split");
#pragma unroll
    for (int b = 0; b < kRowsPerWarp; b += kBatch) {
      uint32_t v[kBatch], v2[kBatch];
#pragma unroll
      for (int j = 0; j < kBatch; ++j) {
        const int r = warp + (kCleanThreads / 32) * (b + j);
        const int z = z0 - kCH + r / kCSY, y = y0 - kCH + r % kCSY;
        const bool rin = z >= 0 && z < dm.d && y >= 0 && y < dm.h;
        const uint32_t* row = fm + ((long long)z * dm.h + y) * dm.w;
        const int x = x0 - kCH + lane, xb = x0 - kCH + 32 + lane;
        v[j] = (rin && x >= 0 && x < dm.w) ? row[x] : kOob;
        v2[j] = (lane < kCSX - 32 && rin && xb < dm.w) ? row[xb] : kOob;
      }
#pragma unroll
      for (int j = 0; j < kBatch; ++j) {
        const int r = warp + (kCleanThreads / 32) * (b + j);
        uint32_t* srow = T + r * kCSX;
        // staged as the f32 diameter bits (2*sqrt(r^2)), 0 staying 0; pass 2
        // reads diameters only within one voxel of the tile, so the outer
        // ring keeps just its nonzero flags
        const int rz = r / kCSY, ry = r % kCSY;
        const bool ring = rz == 0 || rz == kCSZ - 1 || ry == 0 || ry == kCSY - 1;
        if (!ring) {
          srow[lane] = (lane == 0 || v[j] == 0u || v[j] == kOob) ? 0u : __float_as_uint(dia[v[j]]);
          if (lane < kCSX - 32)
            srow[32 + lane] =
                (lane == kCSX - 33 || v2[j] == 0u || v2[j] == kOob) ? 0u : __float_as_uint(dia[v2[j]]);
        }
        const unsigned b1 = __ballot_sync(0xffffffffu, v[j] != 0u);
        const unsigned b2 = __ballot_sync(0xffffffffu, lane < kCSX - 32 && v2[j] != 0u);
        const unsigned o1 = __ballot_sync(0xffffffffu, v[j] != 0u && v[j] != kOob);
        const unsigned o2 = __ballot_sync(0xffffffffu, lane < kCSX - 32 && v2[j] != 0u && v2[j] != kOob);
        if (lane == 0) {
          nz[r] = (unsigned long long)b1 | ((unsigned long long)b2 << 32);
          own[r] = (unsigned long long)o1 | ((unsigned long long)o2 << 32);
        }
      }
    }
    __syncthreads();
    // pass 1: erosion of nz over x, y, z for the halo-1 region (rows z,y in [1, kCS-2])
    for (int r = tid; r < kCSZ * kCSY; r += kCleanThreads) {
      const int zz = r / kCSY, yy = r % kCSY;
      unsigned long long m = 0;
      if (zz >= 1 && zz <= kCSZ - 2 && yy >= 1 && yy <= kCSY - 2) {
        m = ~0ull;
        for (int dz = -1; dz <= 1; ++dz)
          for (int dy = -1; dy <= 1; ++dy) {
            const unsigned long long q = nz[(zz + dz) * kCSY + yy + dy];
            m &= q & (q << 1) & (q >> 1);
          }
        // interior also needs the voxel itself nonzero and inside the volume
        m &= own[r];
      }
      inr[r] = m;
    }
    __syncthreads();
    // pass 2 + mask + stats, one output row (32 voxels) per warp step
    for (int r = warp; r < kCTZ * kCTY; r += kCleanThreads / 32) {
      const int oz = r / kCTY, oy = r % kCTY;
      const int z = z0 + oz, y = y0 + oy, x = x0 + lane;
      if (z >= dm.d || y >= dm.h) continue;
      const uint32_t selw = selbits[((long long)z * dm.h + y) * nw + tx];
      float* orow = outmap ? outmap + ((long long)z * dm.h + y) * dm.w : nullptr;
      if (selw == 0u) {  // nothing selected in this row: the masked map is 0
        if (orow && x < dm.w) orow[x] = 0.0f;
        continue;
      }
      const int sz = oz + kCH, sy = oy + kCH, sx = lane + kCH;
      float val = 0.0f;
      if (x < dm.w && ((selw >> lane) & 1u)) {
        const uint32_t t = T[(sz * kCSY + sy) * kCSX + sx];
        if (t != 0u) {
          const float own = __uint_as_float(t);
          if ((inr[sz * kCSY + sy] >> sx) & 1ull) {
            val = own;
          } else {
            // interior flags of the 3x3x3 neighbourhood, bit (dz+1)*9 + (dy+1)*3 + (dx+1)
            uint32_t cube = 0;
#pragma unroll
            for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
              for (int dy = -1; dy <= 1; ++dy)
                cube |= (uint32_t)((inr[(sz + dz) * kCSY + sy + dy] >> (sx - 1)) & 7ull)
                        << ((dz + 1) * 9 + (dy + 1) * 3);
            const uint32_t* tc = T + (sz * kCSY + sy) * kCSX + sx;
            int count = 0;
            float sum = 0.0f;
#pragma unroll
            for (int k = 0; k < 26; ++k) {  // NEIGHBORS_26 order (compile-time offsets)
              const int ci = (kN26c[k][2] + 1) * 9 + (kN26c[k][1] + 1) * 3 + (kN26c[k][0] + 1);
              if (cube & (1u << ci)) {
                sum = __fadd_rn(sum, __uint_as_float(tc[(kN26c[k][2] * kCSY + kN26c[k][1]) * kCSX + kN26c[k][0]]));
                ++count;
              }
            }
            val = count > 0 ? __fdiv_rn(sum, (float)count) : own;
          }
        }
      }
      if (orow && x < dm.w) orow[x] = val;
      if (val > 0.0f) add_value(val, scale, e_lo, cnt, mx, fx1, fx2, run_e, run_s1, run_sh, run_sl, sacc);
    }
  }
  flush_run(sacc, run_e, run_s1, run_sh, run_sl);
  if (cnt) atomicAdd(&sacc.count, cnt);
  if (mx) atomicMax(&sacc.max_bits, mx);
  // this CTA's fixed-point sums: warp reduction, then one record per CTA
  unsigned long long f2lo = (unsigned long long)fx2, f2hi = (unsigned long long)(fx2 >> 64);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    fx1 += __shfl_xor_sync(0xffffffffu, fx1, o);
    const unsigned long long olo = __shfl_xor_sync(0xffffffffu, f2lo, o);
    const unsigned long long ohi = __shfl_xor_sync(0xffffffffu, f2hi, o);
    const unsigned long long lo = f2lo + olo;
    f2hi += ohi + (lo < f2lo ? 1u : 0u);
    f2lo = lo;
  }
  __shared__ unsigned long long s_fx[kCleanThreads / 32][3];
  if (lane == 0) {
    s_fx[warp][0] = fx1;
    s_fx[warp][1] = f2lo;
    s_fx[warp][2] = f2hi;
  }
  __syncthreads();
  if (tid == 0) {
    FixedPartial r{0ull, 0ull, 0ull, 0ull};
    for (int w = 0; w < kCleanThreads / 32; ++w) {
      r.s1 += s_fx[w][0];
      const unsigned long long lo = r.s2lo + s_fx[w][1];
      r.s2hi += s_fx[w][2] + (lo < r.s2lo ? 1u : 0u);
      r.s2lo = lo;
    }
    part[blockIdx.x] = r;
  }
  for (int i = tid; i < 256; i += kCleanThreads) {
    if (sacc.sum_m[i]) atomicAdd(&acc->sum_m[i], sacc.sum_m[i]);
    if (sacc.sq_hi[i]) atomicAdd(&acc->sq_hi[i], sacc.sq_hi[i]);
    if (sacc.sq_lo[i]) atomicAdd(&acc->sq_lo[i], sacc.sq_lo[i]);
  }
  if (tid == 0) {
    if (sacc.count) atomicAdd(&acc->count, sacc.count);
    if (sacc.max_bits) atomicMax(&acc->max_bits, sacc.max_bits);
  }
}

// Distance ridge (local_thickness.rs:104-167) on 32 x 8 x 8 tiles with the
// distance map staged with a halo of 1 (out-of-volume neighbours are skipped,
// as in the reference's bounds checks).  A selected voxel (d > 0) is a ridge
// unless some 26-neighbour's d reaches the search template of its own r^2
// (offset class = number of nonzero components).
constexpr int kRTX = 32, kRTY = 8, kRTZ = 8;
constexpr int kRSX = kRTX + 2, kRSY = kRTY + 2, kRSZ = kRTZ + 2;

__global__ void __launch_bounds__(256)
ridge_tile_kernel(const uint32_t* __restrict__ dist, const uint32_t* __restrict__ selbits, Dims dm,
                  const uint4* __restrict__ lut, uint2* __restrict__ ridges, Counters* __restrict__ ctr,
                  uint32_t* __restrict__ occ, uint32_t* __restrict__ ridgebits, int ntx, int nty, int ntz) {
  __shared__ uint32_t D[kRSZ * kRSY * kRSX];
  __shared__ uint32_t s_wcnt[8];
  __shared__ unsigned long long s_base;
  __shared__ uint32_t s_tile;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long ntiles = (long long)ntx * nty * ntz;
  const int nw = dm.nw();
  // tiles are taken from a counter as CTAs free up (their costs vary widely)
  for (;;) {
    __syncthreads();  // every thread has read s_tile
    if (tid == 0) s_tile = atomicAdd(&ctr->tile_next[0], 1u);
    __syncthreads();
    const long long tile = s_tile;
    if (tile >= ntiles) break;
    const int tx = (int)(tile % ntx), ty = (int)((tile / ntx) % nty), tz = (int)(tile / ((long long)ntx * nty));
    const int x0 = tx * kRTX, y0 = ty * kRTY, z0 = tz * kRTZ;
    // ridges are selected voxels: a tile without any has none
    bool any_sel = false;
    if (tid < kRTZ * kRTY) {
      const int z = z0 + tid / kRTY, y = y0 + tid % kRTY;
      if (z < dm.d && y < dm.h) any_sel = selbits[((long long)z * dm.h + y) * nw + tx] != 0u;
    }
    if (!__syncthreads_or(any_sel)) continue;
    // stage the distance map with halo 1: one row of 34 per warp step, loads
    // of all the warp's rows issued before the stores
    constexpr int kRidgeRows = (kRSZ * kRSY + 7) / 8;  // 13 (the last step covers 4 rows)
    constexpr int kRBatch = 5;
#pragma unroll
    for (int b = 0; b < kRidgeRows; b += kRBatch) {
      uint32_t v[kRBatch], v2[kRBatch];
#pragma unroll
      for (int j = 0; j < kRBatch; ++j) {
        const int r = warp + 8 * (b + j);
        const int z = z0 - 1 + r / kRSY, y = y0 - 1 + r % kRSY;
        const bool rin = b + j < kRidgeRows && r < kRSZ * kRSY && z >= 0 && z < dm.d && y >= 0 && y < dm.h;
        const uint32_t* row = dist + ((long long)z * dm.h + y) * dm.w;
        const int x = x0 - 1 + lane, xb = x0 + 31 + lane;
        v[j] = (rin && x >= 0 && x < dm.w) ? row[x] : 0u;
        v2[j] = (lane < 2 && rin && xb < dm.w) ? row[xb] : 0u;
      }
#pragma unroll
      for (int j = 0; j < kRBatch; ++j) {
        const int r = warp + 8 * (b + j);
        if (b + j < kRidgeRows && r < kRSZ * kRSY) {
          uint32_t* srow = D + r * kRSX;
          srow[lane] = v[j];
          if (lane < 2) srow[32 + lane] = v2[j];
        }
      }
    }
    __syncthreads();
    // ridge masks of this warp's 8 rows, then one global slot reservation per tile
    unsigned mk[kRTZ * kRTY / 8];
    int wcount = 0;
#pragma unroll
    for (int k = 0; k < kRTZ * kRTY / 8; ++k) {
      const int r = warp + 8 * k;
      const int oz = r / kRTY, oy = r % kRTY;
      const int z = z0 + oz, y = y0 + oy, x = x0 + lane;
      bool ridge = false;
      if (z < dm.d && y < dm.h && x < dm.w) {
        const int sx = lane + 1, sy = oy + 1, sz = oz + 1;
        const uint32_t R = D[(sz * kRSY + sy) * kRSX + sx];
        if (R > 0u) {
          const uint4 t = lut[R];
          ridge = true;
          // neighbours outside the volume hold 0 and never reach a template (>= 4)
#pragma unroll
          for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
              for (int dx = -1; dx <= 1; ++dx) {
                if (dx == 0 && dy == 0 && dz == 0) continue;
                const int c = (dx != 0) + (dy != 0) + (dz != 0);
                const uint32_t thr = c == 1 ? t.x : (c == 2 ? t.y : t.z);
                if (D[((sz + dz) * kRSY + sy + dy) * kRSX + sx + dx] >= thr) ridge = false;
              }
        }
      }
      mk[k] = __ballot_sync(0xffffffffu, ridge);
      wcount += __popc(mk[k]);
      if (ridgebits && lane == 0 && z < dm.d && y < dm.h) ridgebits[((long long)z * dm.h + y) * nw + tx] = mk[k];
    }
    if (lane == 0) s_wcnt[warp] = (uint32_t)wcount;
    __syncthreads();
    if (tid == 0) {
      uint32_t tot = 0;
      for (int w = 0; w < 8; ++w) {
        const uint32_t c = s_wcnt[w];
        s_wcnt[w] = tot;
        tot += c;
      }
      s_base = tot ? atomicAdd(&ctr->ridges, (unsigned long long)tot) : 0ull;
    }
    __syncthreads();
    unsigned long long slot = s_base + s_wcnt[warp];
#pragma unroll
    for (int k = 0; k < kRTZ * kRTY / 8; ++k) {
      const unsigned m = mk[k];
      if ((m >> lane) & 1u) {
        const int r = warp + 8 * k;
        const int oz = r / kRTY, oy = r % kRTY;
        const int z = z0 + oz, y = y0 + oy, x = x0 + lane;
        const uint32_t R = D[((oz + 1) * kRSY + oy + 1) * kRSX + lane + 1];
        ridges[slot + __popc(m & ((1u << lane) - 1u))] =
            make_uint2((uint32_t)(((long long)z * dm.h + y) * dm.w + x), R);
        if (occ && occ[R] == 0u) occ[R] = 1u;
      }
      slot += __popc(m);
    }
  }
}

__global__ void dia_extract_kernel(const uint4* __restrict__ lut, uint32_t n, float* __restrict__ dia) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    dia[i] = __uint_as_float(lut[i].w);
}

inline unsigned grid_for(long long work, int per_block, int cap) {
  long long b = (work + per_block - 1) / per_block;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (unsigned)b;
}

}  // namespace

cudaError_t launch_lut(uint4* lut, uint32_t lo, uint32_t hi, cudaStream_t s, unsigned long long* launches) {
  if (hi < lo) return cudaSuccess;
  const long long count = (long long)hi - lo + 1;
  lut_kernel<<<grid_for(count, 8, 152 * 16), 256, 0, s>>>(lut, lo, hi);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_dia_table(const uint4* lut, uint32_t n, float* dia, cudaStream_t s, unsigned long long* launches) {
  dia_extract_kernel<<<grid_for(n, 256, 1024), 256, 0, s>>>(lut, n, dia);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_ridges(const uint32_t* dist, const uint32_t* selbits, Dims dm, const uint4* lut, uint2* ridges,
                          Counters* ctr, uint32_t* occ, uint32_t* ridgebits, cudaStream_t s,
                          unsigned long long* launches) {
  const int ntx = (dm.w + kRTX - 1) / kRTX, nty = (dm.h + kRTY - 1) / kRTY, ntz = (dm.d + kRTZ - 1) / kRTZ;
  const long long tiles = (long long)ntx * nty * ntz;
  ridge_tile_kernel<<<resident_grid(ridge_tile_kernel, 256, 0, tiles), 256, 0, s>>>(dist, selbits, dm, lut, ridges,
                                                                                    ctr, occ, ridgebits, ntx, nty, ntz);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_fill(const uint2* ridges, const Counters* ctr, unsigned long long max_ridges, Dims dm,
                        uint32_t* fillmap, cudaStream_t s, unsigned long long* launches) {
  fill_kernel<<<grid_for((long long)max_ridges, 8, 152 * 32), 256, 0, s>>>(ridges, ctr, dm, fillmap);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_cleanup(const uint32_t* fillmap, const uint32_t* selbits, Dims dm, const float* dia, float scale,
                           float* outmap, StatsAccum* acc, FixedPartial* part, int e_lo, unsigned* tile_next,
                           unsigned* grid, cudaStream_t s, unsigned long long* launches) {
  const int ntx = (dm.w + kCTX - 1) / kCTX, nty = (dm.h + kCTY - 1) / kCTY, ntz = (dm.d + kCTZ - 1) / kCTZ;
  const long long tiles = (long long)ntx * nty * ntz;
  unsigned g = resident_grid(cleanup_tile_kernel, kCleanThreads, 0, tiles);
  if (g > kCleanupMaxGrid) g = kCleanupMaxGrid;
  *grid = g;
  cleanup_tile_kernel<<<g, kCleanThreads, 0, s>>>(fillmap, selbits, dm, dia, scale, outmap, acc, part, e_lo, ntx, nty,
                                                  ntz, tile_next);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace bm
