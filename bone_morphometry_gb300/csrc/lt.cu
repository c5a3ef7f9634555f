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

// Thread per voxel.  A voxel is selected exactly when its squared distance is
// positive (non-selected voxels are sites, distance 0), so the ridge test of
// local_thickness.rs:104-167 needs only the distance map.
__global__ void __launch_bounds__(256)
ridge_kernel(const uint32_t* __restrict__ dist, Dims dm, const uint4* __restrict__ lut, uint2* __restrict__ ridges,
             Counters* __restrict__ ctr, uint32_t* __restrict__ occ) {
  const long long N = dm.n();
  const long long sl = (long long)dm.w * dm.h;
  const int lane = threadIdx.x & 31;
  for (long long base = (long long)blockIdx.x * blockDim.x; base < N; base += (long long)gridDim.x * blockDim.x) {
    const long long idx = base + threadIdx.x;
    bool ridge = false;
    uint32_t R = 0;
    if (idx < N) {
      R = dist[idx];
      if (R > 0) {
        const int z = (int)(idx / sl);
        const long long rem = idx - (long long)z * sl;
        const int y = (int)(rem / dm.w);
        const int x = (int)(rem - (long long)y * dm.w);
        const uint4 t = lut[R];
        ridge = true;
        for (int dz = -1; dz <= 1 && ridge; ++dz) {
          const int nz = z + dz;
          if (nz < 0 || nz >= dm.d) continue;
          for (int dy = -1; dy <= 1 && ridge; ++dy) {
            const int ny = y + dy;
            if (ny < 0 || ny >= dm.h) continue;
            const uint32_t* rowp = dist + ((long long)nz * dm.h + ny) * dm.w;
            for (int dx = -1; dx <= 1; ++dx) {
              if (dx == 0 && dy == 0 && dz == 0) continue;
              const int nx = x + dx;
              if (nx < 0 || nx >= dm.w) continue;
              const int c = (dx != 0) + (dy != 0) + (dz != 0);
              const uint32_t thr = c == 1 ? t.x : (c == 2 ? t.y : t.z);
              if (rowp[nx] >= thr) {
                ridge = false;
                break;
              }
            }
          }
        }
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, ridge);
    if (m) {
      unsigned long long slot = 0;
      const int leader = __ffs(m) - 1;
      if (lane == leader) slot = atomicAdd(&ctr->ridges, (unsigned long long)__popc(m));
      slot = __shfl_sync(0xffffffffu, slot, leader);
      if (ridge) {
        ridges[slot + __popc(m & ((1u << lane) - 1u))] = make_uint2((uint32_t)idx, R);
        if (occ && occ[R] == 0u) occ[R] = 1u;  // read first: most ridges share few r2 values
      }
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

// Pass 1 of clean_up_surface_jaggies (local_thickness.rs:214-238) as a bit:
// set for a nonzero voxel none of whose in-bounds 26-neighbours is zero (such a
// voxel keeps its value; the others become -1).  One warp per 32-voxel word.
__global__ void __launch_bounds__(256)
interior_kernel(const uint32_t* __restrict__ fm, Dims dm, uint32_t* __restrict__ posbits) {
  const int nw = dm.nw();
  const long long words = (long long)nw * dm.h * dm.d;
  const int lane = threadIdx.x & 31;
  const long long wid0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long wi = wid0; wi < words; wi += nwarps) {
    const long long row = wi / nw;
    const int c = (int)(wi - row * nw);
    const int y = (int)(row % dm.h);
    const int z = (int)(row / dm.h);
    const int x = c * 32 + lane;
    bool pos = false;
    if (x < dm.w) {
      const long long idx = row * dm.w + x;
      if (fm[idx] != 0u) {
        pos = true;
        for (int dz = -1; dz <= 1 && pos; ++dz) {
          const int nz = z + dz;
          if (nz < 0 || nz >= dm.d) continue;
          for (int dy = -1; dy <= 1 && pos; ++dy) {
            const int nyy = y + dy;
            if (nyy < 0 || nyy >= dm.h) continue;
            const uint32_t* rowp = fm + ((long long)nz * dm.h + nyy) * dm.w;
            for (int dx = -1; dx <= 1; ++dx) {
              const int nx = x + dx;
              if (nx < 0 || nx >= dm.w) continue;
              if (rowp[nx] == 0u) {
                pos = false;
                break;
              }
            }
          }
        }
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, pos);
    if (lane == 0) posbits[wi] = m;
  }
}

// NEIGHBORS_26 of local_thickness.rs:285-312 (Fiji's visitation order), which
// fixes the order of the f32 sum in pass 2.
__constant__ signed char kN26[26][3] = {
    {0, 0, -1}, {0, 0, 1},  {0, -1, 0}, {0, 1, 0},   {-1, 0, 0},  {1, 0, 0},  {0, 1, -1},
    {0, 1, 1},  {1, -1, 0}, {1, 1, 0},  {-1, 0, 1},  {1, 0, 1},   {0, -1, -1}, {0, -1, 1},
    {-1, -1, 0}, {-1, 1, 0}, {-1, 0, -1}, {1, 0, -1}, {1, 1, 1},   {1, -1, 1}, {-1, 1, 1},
    {-1, -1, 1}, {1, 1, -1}, {1, -1, -1}, {-1, 1, -1}, {-1, -1, -1}};

__device__ __forceinline__ bool bit_at(const uint32_t* __restrict__ bits, int nw, long long row, int x) {
  return (bits[row * nw + (x >> 5)] >> (x & 31)) & 1u;
}

__device__ __forceinline__ void accum_value(StatsAccum* s, float v) {
  const uint32_t b = __float_as_uint(v);
  uint32_t e = b >> 23;
  uint32_t m = b & 0x7fffffu;
  if (e) m |= 0x800000u;
  else e = 1;
  const unsigned long long sq = (unsigned long long)m * m;
  atomicAdd(&s->sum_m[e], (unsigned long long)m);
  atomicAdd(&s->sq_hi[e], sq >> 24);
  atomicAdd(&s->sq_lo[e], sq & 0xffffffull);
}

// Pass 2 (local_thickness.rs:243-277), the final abs (:279), the phase mask
// (:31-43), the f32 calibration multiply and the exact moment sums of
// nonzero_stats (metrics.rs:215-226).  One warp per 32-voxel word.
__global__ void __launch_bounds__(256)
final_kernel(const uint32_t* __restrict__ fm, const uint32_t* __restrict__ posbits,
             const uint32_t* __restrict__ selbits, Dims dm, const uint4* __restrict__ lut, float scale,
             float* __restrict__ outmap, StatsAccum* __restrict__ acc) {
  __shared__ StatsAccum sacc;
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    sacc.sum_m[i] = 0;
    sacc.sq_hi[i] = 0;
    sacc.sq_lo[i] = 0;
  }
  if (threadIdx.x == 0) {
    sacc.count = 0;
    sacc.max_bits = 0;
  }
  __syncthreads();
  const int nw = dm.nw();
  const long long words = (long long)nw * dm.h * dm.d;
  const int lane = threadIdx.x & 31;
  const long long wid0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  unsigned long long cnt = 0;
  uint32_t mx = 0;
  for (long long wi = wid0; wi < words; wi += nwarps) {
    const long long row = wi / nw;
    const int c = (int)(wi - row * nw);
    const int y = (int)(row % dm.h);
    const int z = (int)(row / dm.h);
    const int x = c * 32 + lane;
    if (x >= dm.w) continue;
    const long long idx = row * dm.w + x;
    float val = 0.0f;
    const bool sel = (selbits[wi] >> lane) & 1u;
    if (sel) {
      const uint32_t T = fm[idx];
      if (T != 0u) {
        const float own = __uint_as_float(lut[T].w);
        if ((posbits[wi] >> lane) & 1u) {
          val = own;
        } else {
          int count = 0;
          float sum = 0.0f;
          for (int k = 0; k < 26; ++k) {
            const int nx = x + kN26[k][0], nyy = y + kN26[k][1], nz = z + kN26[k][2];
            if (nx < 0 || nyy < 0 || nz < 0 || nx >= dm.w || nyy >= dm.h || nz >= dm.d) continue;
            const long long nrow = (long long)nz * dm.h + nyy;
            if (!bit_at(posbits, nw, nrow, nx)) continue;
            sum = __fadd_rn(sum, __uint_as_float(lut[fm[nrow * dm.w + nx]].w));
            ++count;
          }
          val = count > 0 ? __fdiv_rn(sum, (float)count) : own;
        }
      }
    }
    if (outmap) outmap[idx] = val;
    if (val > 0.0f) {
      const float v = __fmul_rn(val, scale);
      accum_value(&sacc, v);
      ++cnt;
      mx = max(mx, __float_as_uint(v));
    }
  }
  if (cnt) atomicAdd(&sacc.count, cnt);
  if (mx) atomicMax(&sacc.max_bits, mx);
  __syncthreads();
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    if (sacc.sum_m[i]) atomicAdd(&acc->sum_m[i], sacc.sum_m[i]);
    if (sacc.sq_hi[i]) atomicAdd(&acc->sq_hi[i], sacc.sq_hi[i]);
    if (sacc.sq_lo[i]) atomicAdd(&acc->sq_lo[i], sacc.sq_lo[i]);
  }
  if (threadIdx.x == 0) {
    if (sacc.count) atomicAdd(&acc->count, sacc.count);
    if (sacc.max_bits) atomicMax(&acc->max_bits, sacc.max_bits);
  }
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

cudaError_t launch_ridges(const uint32_t* dist, Dims dm, const uint4* lut, uint2* ridges, Counters* ctr,
                          uint32_t* occ, cudaStream_t s, unsigned long long* launches) {
  ridge_kernel<<<grid_for(dm.n(), 256, 152 * 32), 256, 0, s>>>(dist, dm, lut, ridges, ctr, occ);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_fill(const uint2* ridges, const Counters* ctr, unsigned long long max_ridges, Dims dm,
                        uint32_t* fillmap, cudaStream_t s, unsigned long long* launches) {
  fill_kernel<<<grid_for((long long)max_ridges, 8, 152 * 32), 256, 0, s>>>(ridges, ctr, dm, fillmap);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_interior_bits(const uint32_t* fillmap, Dims dm, uint32_t* posbits, cudaStream_t s,
                                 unsigned long long* launches) {
  const long long words = (long long)dm.nw() * dm.h * dm.d;
  interior_kernel<<<grid_for(words, 8, 152 * 32), 256, 0, s>>>(fillmap, dm, posbits);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_final(const uint32_t* fillmap, const uint32_t* posbits, const uint32_t* selbits, Dims dm,
                         const uint4* lut, float scale, float* outmap, StatsAccum* acc, cudaStream_t s,
                         unsigned long long* launches) {
  const long long words = (long long)dm.nw() * dm.h * dm.d;
  final_kernel<<<grid_for(words, 8, 152 * 16), 256, 0, s>>>(fillmap, posbits, selbits, dm, lut, scale, outmap,
                                                            acc);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace bm
