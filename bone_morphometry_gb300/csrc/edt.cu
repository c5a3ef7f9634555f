// Exact squared Euclidean distance transform on sm_103a (edt.rs:57-156).
//
// The reference computes the Felzenszwalb-Huttenlocher lower envelope in f64
// with INF = 1e30 and rounds; on integer inputs every comparison it makes is
// exact and INF parabolas never reach the envelope inside a line that has a
// finite one, so its output is the mathematically exact squared EDT.  The GPU
// computes the same values with integers only:
//   pass x : distance to the nearest non-selected voxel of the row, from a
//            bitmask of the row (ballot + clz/ffs), squared;
//   pass y, z : lower envelope of the parabolas (q - p)^2 + f(p) with the
//            intersection test done by int64 cross-multiplication; lines
//            whose every entry is "no site" (kInfSq) stay kInfSq.
#include <climits>
#include <cstdint>

#include "kernels.h"

namespace bm {

namespace {

template <int MODE>
__device__ __forceinline__ bool selected_at(const uint8_t* __restrict__ a, const uint8_t* __restrict__ b,
                                            long long i) {
  if (MODE == SEL_FOREGROUND) return a[i] != 0;
  if (MODE == SEL_BACKGROUND) return a[i] == 0;
  if (MODE == SEL_BONE_IN_ROI) return b[i] != 0 && a[i] != 0;
  return b[i] != 0 && a[i] == 0;
}

constexpr int kXWarps = 8;

// One warp per x row.  Shared memory per warp: site bitmask of the row and, per
// word, the nearest non-empty word at-or-before / at-or-after it.
template <int MODE>
__global__ void __launch_bounds__(kXWarps * 32)
edt_x_kernel(const uint8_t* __restrict__ a, const uint8_t* __restrict__ b, Dims dm, uint32_t* __restrict__ out,
             uint32_t* __restrict__ selbits, Counters* __restrict__ ctr) {
  extern __shared__ uint32_t smem[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nw = dm.nw();
  uint32_t* mask = smem + (size_t)warp * 3 * nw;
  int* prevnz = reinterpret_cast<int*>(mask + nw);
  int* nextnz = prevnz + nw;
  const long long rows = (long long)dm.h * dm.d;
  unsigned long long sites = 0;

  for (long long row = (long long)blockIdx.x * kXWarps + warp; row < rows;
       row += (long long)gridDim.x * kXWarps) {
    const long long base = row * dm.w;
    for (int c = 0; c < nw; ++c) {
      const int x = c * 32 + lane;
      const bool in = x < dm.w;
      const bool s = in && selected_at<MODE>(a, b, base + x);
      const unsigned site = __ballot_sync(0xffffffffu, in && !s);
      const unsigned selw = __ballot_sync(0xffffffffu, s);
      if (lane == 0) {
        mask[c] = site;
        selbits[row * nw + c] = selw;
        sites += __popc(site);
      }
    }
    __syncwarp();
    int carry = -1;
    for (int c0 = 0; c0 < nw; c0 += 32) {
      const int c = c0 + lane;
      int v = (c < nw && mask[c] != 0u) ? c : -1;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v = max(v, t);
      }
      v = max(v, carry);
      if (c < nw) prevnz[c] = v;
      carry = __shfl_sync(0xffffffffu, v, 31);
    }
    carry = INT_MAX;
    for (int c0 = ((nw - 1) >> 5) << 5; c0 >= 0; c0 -= 32) {
      const int c = c0 + lane;
      int v = (c < nw && mask[c] != 0u) ? c : INT_MAX;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_down_sync(0xffffffffu, v, o);
        if (lane + o < 32) v = min(v, t);
      }
      v = min(v, carry);
      if (c < nw) nextnz[c] = v;
      carry = __shfl_sync(0xffffffffu, v, 0);
    }
    __syncwarp();
    for (int c = 0; c < nw; ++c) {
      const int x = c * 32 + lane;
      if (x < dm.w) {
        const uint32_t m = mask[c];
        uint32_t val = 0;
        if (!((m >> lane) & 1u)) {
          int left = -1, right = -1;
          const uint32_t lo = m & ((1u << lane) - 1u);
          if (lo) {
            left = c * 32 + 31 - __clz(lo);
          } else if (c > 0) {
            const int p = prevnz[c - 1];
            if (p >= 0) left = p * 32 + 31 - __clz(mask[p]);
          }
          const uint32_t hi = (lane == 31) ? 0u : (m & ~((2u << lane) - 1u));
          if (hi) {
            right = c * 32 + __ffs(hi) - 1;
          } else if (c + 1 < nw) {
            const int p = nextnz[c + 1];
            if (p != INT_MAX) right = p * 32 + __ffs(mask[p]) - 1;
          }
          int g = INT_MAX;
          if (left >= 0) g = x - left;
          if (right >= 0) g = min(g, right - x);
          val = (g == INT_MAX) ? kInfSq : (uint32_t)g * (uint32_t)g;
        }
        out[base + x] = val;
      }
    }
    __syncwarp();
  }
  if (lane == 0 && sites) atomicAdd(&ctr->sites, sites);
}

// 4-bit selection mask of the 4 voxels in a (bone) and b (roi) words:
// per byte, the MODE predicate, packed to bits 0..3.
template <int MODE>
__device__ __forceinline__ uint32_t sel4(uint32_t a, uint32_t b) {
  const uint32_t nza = __vcmpne4(a, 0u), nzb = __vcmpne4(b, 0u);  // 0xff per nonzero byte
  uint32_t m;
  if (MODE == SEL_FOREGROUND) m = nza;
  else if (MODE == SEL_BACKGROUND) m = ~nza;
  else if (MODE == SEL_BONE_IN_ROI) m = nzb & nza;
  else m = nzb & ~nza;
  m &= 0x01010101u;
  return (m * 0x01020408u) >> 24 & 0xfu;  // bytes 0..3 -> bits 0..3
}

// The x pass for rows whose bytes are 16-byte aligned (w a multiple of 16 and
// aligned inputs): each lane loads 16 voxels of bone and roi at once and the
// lanes' 16-bit masks pair up into the row's 32-bit words; the distances are
// then computed as in edt_x_kernel, one x per lane (coalesced stores).
template <int MODE>
__global__ void __launch_bounds__(kXWarps * 32)
edt_x_vec_kernel(const uint8_t* __restrict__ a, const uint8_t* __restrict__ b, Dims dm, uint32_t* __restrict__ out,
                 uint32_t* __restrict__ selbits, Counters* __restrict__ ctr) {
  extern __shared__ uint32_t smem[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nw = dm.nw();
  uint32_t* mask = smem + (size_t)warp * 3 * nw;
  int* prevnz = reinterpret_cast<int*>(mask + nw);
  int* nextnz = prevnz + nw;
  const long long rows = (long long)dm.h * dm.d;
  const bool two = MODE == SEL_BONE_IN_ROI || MODE == SEL_MARROW_IN_ROI;
  unsigned long long sites = 0;

  for (long long row = (long long)blockIdx.x * kXWarps + warp; row < rows;
       row += (long long)gridDim.x * kXWarps) {
    const long long base = row * dm.w;
    const uint4* av = reinterpret_cast<const uint4*>(a + base);
    const uint4* bv = two ? reinterpret_cast<const uint4*>(b + base) : nullptr;
    const int nvec = dm.w >> 4;  // 16 voxels per uint4
    for (int v0 = 0; v0 < nvec; v0 += 32) {
      const int v = v0 + lane;
      uint32_t s16 = 0, t16 = 0;
      if (v < nvec) {
        const uint4 A = av[v];
        const uint4 B = two ? bv[v] : make_uint4(0u, 0u, 0u, 0u);
        s16 = sel4<MODE>(A.x, B.x) | (sel4<MODE>(A.y, B.y) << 4) | (sel4<MODE>(A.z, B.z) << 8) |
              (sel4<MODE>(A.w, B.w) << 12);
        t16 = ~s16 & 0xffffu;  // all 16 voxels lie inside the row
      }
      const uint32_t s_hi = __shfl_down_sync(0xffffffffu, s16, 1);
      const uint32_t t_hi = __shfl_down_sync(0xffffffffu, t16, 1);
      if (!(lane & 1) && v < nvec) {
        const int c = v >> 1;  // word index: voxels 32c .. 32c + 31
        // a row of 16k voxels with k odd ends on a half word: its upper half is empty
        const bool full = v + 1 < nvec;
        const uint32_t sw = s16 | (full ? s_hi << 16 : 0u);
        const uint32_t tw = t16 | (full ? t_hi << 16 : 0u);
        mask[c] = tw;
        selbits[row * nw + c] = sw;
        sites += __popc(tw);
      }
    }
    __syncwarp();
    int carry = -1;
    for (int c0 = 0; c0 < nw; c0 += 32) {
      const int c = c0 + lane;
      int v = (c < nw && mask[c] != 0u) ? c : -1;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v = max(v, t);
      }
      v = max(v, carry);
      if (c < nw) prevnz[c] = v;
      carry = __shfl_sync(0xffffffffu, v, 31);
    }
    carry = INT_MAX;
    for (int c0 = ((nw - 1) >> 5) << 5; c0 >= 0; c0 -= 32) {
      const int c = c0 + lane;
      int v = (c < nw && mask[c] != 0u) ? c : INT_MAX;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_down_sync(0xffffffffu, v, o);
        if (lane + o < 32) v = min(v, t);
      }
      v = min(v, carry);
      if (c < nw) nextnz[c] = v;
      carry = __shfl_sync(0xffffffffu, v, 0);
    }
    __syncwarp();
    for (int c = 0; c < nw; ++c) {
      const int x = c * 32 + lane;
      if (x < dm.w) {
        const uint32_t m = mask[c];
        uint32_t val = 0;
        if (!((m >> lane) & 1u)) {
          int left = -1, right = -1;
          const uint32_t lo = m & ((1u << lane) - 1u);
          if (lo) {
            left = c * 32 + 31 - __clz(lo);
          } else if (c > 0) {
            const int p = prevnz[c - 1];
            if (p >= 0) left = p * 32 + 31 - __clz(mask[p]);
          }
          const uint32_t hi = (lane == 31) ? 0u : (m & ~((2u << lane) - 1u));
          if (hi) {
            right = c * 32 + __ffs(hi) - 1;
          } else if (c + 1 < nw) {
            const int p = nextnz[c + 1];
            if (p != INT_MAX) right = p * 32 + __ffs(mask[p]) - 1;
          }
          int g = INT_MAX;
          if (left >= 0) g = x - left;
          if (right >= 0) g = min(g, right - x);
          val = (g == INT_MAX) ? kInfSq : (uint32_t)g * (uint32_t)g;
        }
        out[base + x] = val;
      }
    }
    __syncwarp();
  }
  if (lane == 0 && sites) atomicAdd(&ctr->sites, sites);
}

// One thread per line; consecutive threads take consecutive x so that every
// load and store of the line data is a coalesced row.  The envelope stack
// (position, f) lives in global scratch, k-major, and is cached by L1/L2.
__global__ void __launch_bounds__(256)
edt_line_kernel(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, int n, long long stride, int w,
                long long outer, long long nlines, uint32_t* __restrict__ spos, uint32_t* __restrict__ sf,
                Counters* __restrict__ ctr, int track_max, const uint8_t* __restrict__ only) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t localmax = 0;
  if (t < nlines && (only == nullptr || only[t])) {
    const long long base = (t / w) * outer + (t % w);
    int k = -1;
    long long p1 = 0, F1 = 0;  // stack top
    long long p0 = 0, F0 = 0;  // entry below the top (valid when k >= 1)
    for (int q = 0; q < n; ++q) {
      const uint32_t fq = in[base + (long long)q * stride];
      if (fq == kInfSq) continue;
      const long long Fq = (long long)fq + (long long)q * q;
      while (k >= 1 && (Fq - F1) * (p1 - p0) <= (F1 - F0) * ((long long)q - p1)) {
        --k;
        p1 = p0;
        F1 = F0;
        if (k >= 1) {
          p0 = spos[(long long)(k - 1) * nlines + t];
          F0 = (long long)sf[(long long)(k - 1) * nlines + t] + p0 * p0;
        }
      }
      ++k;
      spos[(long long)k * nlines + t] = (uint32_t)q;
      sf[(long long)k * nlines + t] = fq;
      p0 = p1;
      F0 = F1;
      p1 = q;
      F1 = Fq;
    }
    if (k < 0) {
      for (int q = 0; q < n; ++q) out[base + (long long)q * stride] = kInfSq;
    } else {
      int j = 0;
      long long pj = spos[t];
      uint32_t fj = sf[t];
      long long Fj = (long long)fj + pj * pj;
      long long pn = 0, Fn = 0;
      uint32_t fn = 0;
      if (k >= 1) {
        pn = spos[nlines + t];
        fn = sf[nlines + t];
        Fn = (long long)fn + pn * pn;
      }
      for (int q = 0; q < n; ++q) {
        while (j < k && (Fn - Fj) < 2LL * q * (pn - pj)) {
          ++j;
          pj = pn;
          fj = fn;
          Fj = Fn;
          if (j < k) {
            pn = spos[(long long)(j + 1) * nlines + t];
            fn = sf[(long long)(j + 1) * nlines + t];
            Fn = (long long)fn + pn * pn;
          }
        }
        const long long dq = q - pj;
        const uint32_t v = (uint32_t)(dq * dq) + fj;
        out[base + (long long)q * stride] = v;
        localmax = max(localmax, v);
      }
    }
  }
  if (track_max) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) localmax = max(localmax, __shfl_xor_sync(0xffffffffu, localmax, o));
    if ((threadIdx.x & 31) == 0 && localmax) atomicMax(&ctr->rmax, localmax);
  }
}

// Windowed y / z pass.  d(q) = min_p (q - p)^2 + f(p), and p = q already gives
// f(q), so only |q - p| <= isqrt(f(q) - 1) can improve it: every output is an
// exact minimum over a window whose width is bounded by its own input value.
// A CTA owns 32 consecutive x of one line-row and kWinTL consecutive outputs
// along the axis; it stages those inputs in shared memory as 128-byte rows,
// then a halo on each side as wide as the largest window it needs (at most
// kWinHalo).  Each lane scans outwards from its output and stops once dp^2
// reaches the best value found.  Lines with an output whose window exceeds the
// halo (or that has no site at all, f = kInfSq) are marked in `redo`; the
// lower-envelope kernel recomputes exactly those lines afterwards.
constexpr int kWinTL = 128;
constexpr int kWinHalo = 64;
constexpr int kWinThreads = 256;
constexpr int kWinWarps = kWinThreads / 32;
static_assert(kInfSq + (kWinHalo + 3u) * (kWinHalo + 3u) > kInfSq, "the window scan adds dp^2 to kInfSq");

// floor(sqrt(f)) + 2 >= isqrt(f - 1) + 1 for f >= 1: the halo that f needs,
// from the hardware reciprocal square root (error far below one).
__device__ __forceinline__ uint32_t halo_need(uint32_t f) {
  const float ff = (float)f;
  return (uint32_t)(ff * rsqrtf(ff)) + 2u;
}

__global__ void __launch_bounds__(kWinThreads)
edt_window_kernel(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, int n, long long stride, int w,
                  long long outer_stride, int nxt, int nchunk, uint8_t* __restrict__ redo, Counters* __restrict__ ctr,
                  int track_max) {
  __shared__ uint32_t buf[(kWinTL + 2 * kWinHalo) * 32];
  __shared__ uint32_t s_need;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long bid = blockIdx.x;
  const int xt = (int)(bid % nxt);
  const int chunk = (int)((bid / nxt) % nchunk);
  const long long orow = bid / ((long long)nxt * nchunk);
  const int x = xt * 32 + lane;
  const bool xin = x < w;
  const long long base = orow * outer_stride + x;
  const int q0 = chunk * kWinTL;
  if (threadIdx.x == 0) s_need = 0u;
  __syncthreads();
  // centre rows (loads of the warp's 16 rows issued before their use)
  uint32_t need = 0;  // halo rows this block needs: from its largest finite value
  constexpr int kPer = kWinTL / kWinWarps;  // 16
  uint32_t f[kPer];
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    const int q = q0 + warp + kWinWarps * j;
    f[j] = (xin && q < n) ? in[base + (long long)q * stride] : kInfSq;
  }
  uint32_t fmax = 0;  // largest finite value (the halo bound grows with it)
  bool inf = false;
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    const uint32_t v = f[j];
    inf = inf || v == kInfSq;
    fmax = max(fmax, v == kInfSq ? 0u : v);
    buf[(kWinHalo + warp + kWinWarps * j) * 32 + lane] = v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) fmax = max(fmax, __shfl_xor_sync(0xffffffffu, fmax, o));
  inf = __any_sync(0xffffffffu, inf);
  if (lane == 0) {
    need = inf ? 0xffffu : (fmax ? halo_need(fmax) : 0u);
    atomicMax(&s_need, need);
  }
  __syncthreads();
  const int halo = (int)min(s_need, (uint32_t)kWinHalo);
  for (int i = warp; i < halo; i += kWinWarps) {
    const int ql = q0 - 1 - i, qr = q0 + kWinTL + i;
    const uint32_t l = (xin && ql >= 0) ? in[base + (long long)ql * stride] : kInfSq;
    const uint32_t r = (xin && qr < n) ? in[base + (long long)qr * stride] : kInfSq;
    buf[(kWinHalo - 1 - i) * 32 + lane] = l;
    buf[(kWinHalo + kWinTL + i) * 32 + lane] = r;
  }
  __syncthreads();
  uint32_t localmax = 0;
  bool bad = false;
  uint32_t* op = out + base + (long long)(q0 + warp) * stride;  // output of row j, advanced per j
  const long long ostep = (long long)kWinWarps * stride;
#pragma unroll 1
  for (int j = 0; j < kPer; ++j, op += ostep) {
    const int i = warp + kWinWarps * j;
    const int q = q0 + i;
    if (!xin || q >= n) continue;
    const uint32_t* col = buf + (kWinHalo + i) * 32 + lane;
    uint32_t best = col[0];
    if (best == 0u) {
      *op = 0u;
      continue;
    }
    // every p with |q - p| < dp has been tried once dp^2 >= best (a step
    // with dp^2 >= best cannot lower it, so four steps run at a time); if the
    // scan would have to pass the staged halo, the line is redone exactly
    bool done = true;
    int dp = 1;
    while ((uint32_t)(dp * dp) < best) {
      if (dp + 3 <= halo) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int d = dp + u;
          best = min(best, min(col[-d * 32], col[d * 32]) + (uint32_t)(d * d));
        }
        dp += 4;
      } else {
        if (dp > halo) {
          done = false;
          break;
        }
        best = min(best, min(col[-dp * 32], col[dp * 32]) + (uint32_t)(dp * dp));
        ++dp;
      }
    }
    if (!done) {
      bad = true;
      continue;
    }
    *op = best;
    localmax = max(localmax, best);
  }
  if (bad) redo[orow * (long long)w + x] = 1u;
  if (track_max) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) localmax = max(localmax, __shfl_xor_sync(0xffffffffu, localmax, o));
    if (lane == 0 && localmax) atomicMax(&ctr->rmax, localmax);
  }
}

}  // namespace

size_t edt_scratch_bytes(Dims dm) {
  // two u32 arrays (position, f) of line-length x line-count for the larger pass
  const long long y_pass = (long long)dm.h * dm.w * dm.d;
  return (size_t)y_pass * 2 * sizeof(uint32_t);
}

template <int MODE>
cudaError_t launch_edt_x_mode(const uint8_t* a, const uint8_t* b, Dims dm, uint32_t* out, uint32_t* selbits,
                              Counters* ctr, unsigned blocks, size_t smem, cudaStream_t s) {
  const bool two = MODE == SEL_BONE_IN_ROI || MODE == SEL_MARROW_IN_ROI;
  const bool vec = dm.w % 16 == 0 && (reinterpret_cast<uintptr_t>(a) & 15u) == 0 &&
                   (!two || (reinterpret_cast<uintptr_t>(b) & 15u) == 0);
  if (vec) {
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(edt_x_vec_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    edt_x_vec_kernel<MODE><<<blocks, kXWarps * 32, smem, s>>>(a, b, dm, out, selbits, ctr);
  } else {
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(edt_x_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    edt_x_kernel<MODE><<<blocks, kXWarps * 32, smem, s>>>(a, b, dm, out, selbits, ctr);
  }
  return cudaGetLastError();
}

cudaError_t launch_edt_x(const uint8_t* a, const uint8_t* b, int mode, Dims dm, uint32_t* out,
                         uint32_t* selbits, Counters* ctr, cudaStream_t s, unsigned long long* launches) {
  const long long rows = (long long)dm.h * dm.d;
  long long blocks = (rows + kXWarps - 1) / kXWarps;
  if (blocks > 152 * 64) blocks = 152 * 64;
  const size_t smem = (size_t)kXWarps * 3 * dm.nw() * sizeof(uint32_t);
  cudaError_t e;
  switch (mode) {
    case SEL_FOREGROUND:
      e = launch_edt_x_mode<SEL_FOREGROUND>(a, b, dm, out, selbits, ctr, (unsigned)blocks, smem, s);
      break;
    case SEL_BACKGROUND:
      e = launch_edt_x_mode<SEL_BACKGROUND>(a, b, dm, out, selbits, ctr, (unsigned)blocks, smem, s);
      break;
    case SEL_BONE_IN_ROI:
      e = launch_edt_x_mode<SEL_BONE_IN_ROI>(a, b, dm, out, selbits, ctr, (unsigned)blocks, smem, s);
      break;
    default:
      e = launch_edt_x_mode<SEL_MARROW_IN_ROI>(a, b, dm, out, selbits, ctr, (unsigned)blocks, smem, s);
      break;
  }
  ++*launches;
  return e;
}

cudaError_t launch_edt_line(int axis, const uint32_t* in, uint32_t* out, Dims dm, void* scratch, Counters* ctr,
                            cudaStream_t s, unsigned long long* launches) {
  int n;
  long long stride, outer, nlines;
  if (axis == 1) {
    n = dm.h;
    stride = dm.w;
    outer = (long long)dm.w * dm.h;
    nlines = (long long)dm.w * dm.d;
  } else {
    n = dm.d;
    stride = (long long)dm.w * dm.h;
    outer = dm.w;
    nlines = (long long)dm.w * dm.h;
  }
  uint32_t* spos = static_cast<uint32_t*>(scratch);
  uint32_t* sf = spos + (size_t)nlines * n;
  const long long blocks = (nlines + 255) / 256;
  edt_line_kernel<<<(unsigned)blocks, 256, 0, s>>>(in, out, n, stride, dm.w, outer, nlines, spos, sf, ctr,
                                                   axis == 2 ? 1 : 0, nullptr);
  ++*launches;
  return cudaGetLastError();
}

cudaError_t launch_edt_window(int axis, const uint32_t* in, uint32_t* out, Dims dm, void* scratch, uint8_t* redo,
                              Counters* ctr, cudaStream_t s, unsigned long long* launches) {
  int n;
  long long stride, outer, nlines, orows;
  if (axis == 1) {
    n = dm.h;
    stride = dm.w;
    outer = (long long)dm.w * dm.h;
    nlines = (long long)dm.w * dm.d;
    orows = dm.d;
  } else {
    n = dm.d;
    stride = (long long)dm.w * dm.h;
    outer = dm.w;
    nlines = (long long)dm.w * dm.h;
    orows = dm.h;
  }
  cudaError_t e = cudaMemsetAsync(redo, 0, (size_t)nlines, s);
  if (e != cudaSuccess) return e;
  const int nxt = (dm.w + 31) / 32;
  const int nchunk = (n + kWinTL - 1) / kWinTL;
  const long long blocks = (long long)nxt * nchunk * orows;
  edt_window_kernel<<<(unsigned)blocks, kWinThreads, 0, s>>>(in, out, n, stride, dm.w, outer, nxt, nchunk, redo, ctr,
                                                             axis == 2 ? 1 : 0);
  ++*launches;
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // exact lower envelope for the lines the window could not cover
  uint32_t* spos = static_cast<uint32_t*>(scratch);
  uint32_t* sf = spos + (size_t)nlines * n;
  edt_line_kernel<<<(unsigned)((nlines + 255) / 256), 256, 0, s>>>(in, out, n, stride, dm.w,
                                                                  axis == 1 ? (long long)dm.w * dm.h : dm.w, nlines,
                                                                  spos, sf, ctr, axis == 2 ? 1 : 0, redo);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace bm
