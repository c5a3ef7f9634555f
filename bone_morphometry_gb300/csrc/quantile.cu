// Exact order statistics of a thickness map (metrics.rs:242-298).
//
// The reference keeps the finite positive f32 values and selects the k-th
// smallest with select_nth_unstable (total order on floats).  Positive finite
// floats order like their bit patterns, so the k-th value is found by a
// two-level radix select on the 32-bit pattern: a histogram of the high 16
// bits over the whole map, then, for the bins that hold the wanted ranks, a
// histogram of the low 16 bits.  The host walks the histograms; the values are
// exact, so the interpolation that follows (in f64, then f32 calibration) is
// the reference's arithmetic on the reference's operands.
#include "kernels.h"

namespace bm {

namespace {

__device__ __forceinline__ bool positive_finite(uint32_t b) { return b != 0u && b < 0x7f800000u; }

// hist[hi16] += 1 for every positive finite value; lanes with the same key
// add once.
__global__ void __launch_bounds__(256)
hist_hi_kernel(const uint32_t* __restrict__ map, long long n, uint32_t* __restrict__ hist) {
  for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += (long long)gridDim.x * blockDim.x) {
    const long long i = base + threadIdx.x;
    const uint32_t b = i < n ? map[i] : 0u;
    const bool ok = positive_finite(b);
    const unsigned act = __ballot_sync(0xffffffffu, ok);
    if (ok) {
      const uint32_t key = b >> 16;
      const unsigned grp = __match_any_sync(act, key);
      if ((int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicAdd(&hist[key], (uint32_t)__popc(grp));
    }
  }
}

// For target j (hi16 value targets[j]), hist[j * 65536 + lo16] += 1.
__global__ void __launch_bounds__(256)
hist_lo_kernel(const uint32_t* __restrict__ map, long long n, const uint32_t* __restrict__ targets, int ntarget,
               uint32_t* __restrict__ hist) {
  __shared__ uint32_t t[16];
  if (threadIdx.x < 16) t[threadIdx.x] = threadIdx.x < (unsigned)ntarget ? targets[threadIdx.x] : 0xffffffffu;
  __syncthreads();
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const uint32_t b = map[i];
    if (!positive_finite(b)) continue;
    const uint32_t hi = b >> 16;
    for (int j = 0; j < ntarget; ++j)
      if (t[j] == hi) atomicAdd(&hist[(size_t)j * 65536 + (b & 0xffffu)], 1u);
  }
}

// Exact moment sums of f32(raw * scale) over the finite positive raw values
// (metrics.rs:215-226), same accumulator as the cleanup kernel.
__global__ void __launch_bounds__(256)
moments_kernel(const uint32_t* __restrict__ map, long long n, float scale, StatsAccum* __restrict__ acc) {
  __shared__ unsigned long long s1[256], sh[256], sl[256];
  __shared__ unsigned long long scount;
  __shared__ uint32_t smax;
  for (int i = threadIdx.x; i < 256; i += blockDim.x) s1[i] = sh[i] = sl[i] = 0;
  if (threadIdx.x == 0) {
    scount = 0;
    smax = 0;
  }
  __syncthreads();
  unsigned long long cnt = 0;
  uint32_t mx = 0;
  const int lane = threadIdx.x & 31;
  for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += (long long)gridDim.x * blockDim.x) {
    const long long i = base + threadIdx.x;
    const uint32_t b = i < n ? map[i] : 0u;
    const bool ok = positive_finite(b);
    const unsigned act = __ballot_sync(0xffffffffu, ok);
    if (ok) {
      const float v = __fmul_rn(__uint_as_float(b), scale);
      const uint32_t vb = __float_as_uint(v);
      ++cnt;
      mx = max(mx, vb);
      uint32_t e = vb >> 23, m = vb & 0x7fffffu;
      if (e) m |= 0x800000u;
      else e = 1;
      const unsigned long long sq = (unsigned long long)m * m;
      const unsigned grp = __match_any_sync(act, e);
      const uint32_t a1 = __reduce_add_sync(grp, m);
      const uint32_t a2 = __reduce_add_sync(grp, (uint32_t)(sq >> 24));
      const uint32_t a3 = __reduce_add_sync(grp, (uint32_t)(sq & 0xffffffu));
      if (lane == __ffs(grp) - 1) {
        atomicAdd(&s1[e], (unsigned long long)a1);
        atomicAdd(&sh[e], (unsigned long long)a2);
        atomicAdd(&sl[e], (unsigned long long)a3);
      }
    }
  }
  if (cnt) atomicAdd(&scount, cnt);
  if (mx) atomicMax(&smax, mx);
  __syncthreads();
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    if (s1[i]) atomicAdd(&acc->sum_m[i], s1[i]);
    if (sh[i]) atomicAdd(&acc->sq_hi[i], sh[i]);
    if (sl[i]) atomicAdd(&acc->sq_lo[i], sl[i]);
  }
  if (threadIdx.x == 0) {
    if (scount) atomicAdd(&acc->count, scount);
    if (smax) atomicMax(&acc->max_bits, smax);
  }
}

}  // namespace

cudaError_t launch_moments(const float* map, long long n, float scale, StatsAccum* acc, cudaStream_t s,
                           unsigned long long* launches) {
  long long blocks = (n + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (blocks < 1) blocks = 1;
  moments_kernel<<<(unsigned)blocks, 256, 0, s>>>(reinterpret_cast<const uint32_t*>(map), n, scale, acc);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_hist_hi(const float* map, long long n, uint32_t* hist, cudaStream_t s,
                           unsigned long long* launches) {
  long long blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  hist_hi_kernel<<<(unsigned)blocks, 256, 0, s>>>(reinterpret_cast<const uint32_t*>(map), n, hist);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_hist_lo(const float* map, long long n, const uint32_t* targets, int ntarget, uint32_t* hist,
                           cudaStream_t s, unsigned long long* launches) {
  long long blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  hist_lo_kernel<<<(unsigned)blocks, 256, 0, s>>>(reinterpret_cast<const uint32_t*>(map), n, targets, ntarget, hist);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace bm
