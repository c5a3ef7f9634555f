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
#include <cuda.h>  // CUtensorMap and its enums (types only; the encoder comes from the runtime)
#include <cudaTypedefs.h>

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
constexpr int kNoLeft = -(1 << 20);  // sentinels: no site on that side (w <= 32768)
constexpr int kNoRight = 1 << 21;

// Second half of the x pass for one row whose site bitmask (1 = non-selected
// voxel) is in mask[0 .. nw): two warp scans give lastpos[c], the highest
// site position in words <= c, and firstpos[c], the lowest in words >= c, so
// that every voxel finds its nearest site on each side without branching:
// inside its own word from the bits below / above it, else from the neighbour
// word's entry.
__device__ __forceinline__ void x_row_scans(const uint32_t* mask, int* lastpos, int* firstpos, int nw, int lane) {
  int carry = kNoLeft;
  for (int c0 = 0; c0 < nw; c0 += 32) {
    const int c = c0 + lane;
    const uint32_t m = c < nw ? mask[c] : 0u;
    int v = m ? c * 32 + 31 - __clz(m) : kNoLeft;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v = max(v, t);
    }
    v = max(v, carry);
    if (c < nw) lastpos[c] = v;
    carry = __shfl_sync(0xffffffffu, v, 31);
  }
  carry = kNoRight;
  for (int c0 = ((nw - 1) >> 5) << 5; c0 >= 0; c0 -= 32) {
    const int c = c0 + lane;
    const uint32_t m = c < nw ? mask[c] : 0u;
    int v = m ? c * 32 + __ffs(m) - 1 : kNoRight;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_down_sync(0xffffffffu, v, o);
      if (lane + o < 32) v = min(v, t);
    }
    v = min(v, carry);
    if (c < nw) firstpos[c] = v;
    carry = __shfl_sync(0xffffffffu, v, 0);
  }
  __syncwarp();
}

// Squared distance of voxel x to the nearer of its sites left / right
// (kInfSq when neither exists; 0 when x is a site).
__device__ __forceinline__ uint32_t x_dist(bool site, int x, int left, int right) {
  const int g = min(x - left, right - x);
  return site ? 0u : (g >= (1 << 20) ? kInfSq : (uint32_t)g * (uint32_t)g);
}

// One voxel per lane per word: one coalesced 128-byte store per word.
__device__ __forceinline__ void x_row_distances(const uint32_t* mask, int* lastpos, int* firstpos, int nw, int w,
                                                int lane, uint32_t* __restrict__ orow) {
  x_row_scans(mask, lastpos, firstpos, nw, lane);
  const uint32_t below = (1u << lane) - 1u, above = ~((2u << lane) - 1u);  // lane 31: above = 0
#pragma unroll 1
  for (int c = 0; c < nw; ++c) {
    const int x = c * 32 + lane;
    const uint32_t m = mask[c];
    const int lprev = c > 0 ? lastpos[c - 1] : kNoLeft;
    const int rnext = c + 1 < nw ? firstpos[c + 1] : kNoRight;
    const uint32_t lo = m & below, hi = m & above;
    const int left = lo ? c * 32 + 31 - __clz(lo) : lprev;
    const int right = hi ? c * 32 + __ffs(hi) - 1 : rnext;
    if (x < w) orow[x] = x_dist((m >> lane) & 1u, x, left, right);
  }
  __syncwarp();
}

// Four adjacent voxels per lane (rows whose length is a multiple of 16 and
// whose start is 16-byte aligned): the nearest site left of the first voxel
// and right of the last come from the word and scan entries as above, the
// others follow from the three bits between them; one 16-byte store per lane,
// 512 bytes per warp.
__device__ __forceinline__ void x_row_distances4(const uint32_t* mask, int* lastpos, int* firstpos, int nw, int w,
                                                 int lane, uint32_t* __restrict__ orow) {
  x_row_scans(mask, lastpos, firstpos, nw, lane);
  const int b = (lane & 7) * 4;  // first bit of this lane's voxels in their word
  const uint32_t below = (1u << b) - 1u, above = ~((2u << (b + 3)) - 1u);  // b + 3 = 31: above = 0
#pragma unroll 1
  for (int x0 = 0; x0 < w; x0 += 128) {
    const int x = x0 + 4 * lane;
    if (x < w) {
      const int c = x >> 5;
      const uint32_t m = mask[c];
      const int cb = c * 32 + b;
      const uint32_t lo = m & below, hi = m & above;
      const int l0 = lo ? c * 32 + 31 - __clz(lo) : (c > 0 ? lastpos[c - 1] : kNoLeft);
      const int r3 = hi ? c * 32 + __ffs(hi) - 1 : (c + 1 < nw ? firstpos[c + 1] : kNoRight);
      const uint32_t bits = m >> b;  // this lane's 4 voxels in bits 0..3
      const int l1 = (bits & 1u) ? cb : l0;
      const int l2 = (bits & 2u) ? cb + 1 : l1;
      const int l3 = (bits & 4u) ? cb + 2 : l2;
      const int r2 = (bits & 8u) ? cb + 3 : r3;
      const int r1 = (bits & 4u) ? cb + 2 : r2;
      const int r0 = (bits & 2u) ? cb + 1 : r1;
      uint4 v;
      v.x = x_dist(bits & 1u, x, l0, r0);
      v.y = x_dist(bits & 2u, x + 1, l1, r1);
      v.z = x_dist(bits & 4u, x + 2, l2, r2);
      v.w = x_dist(bits & 8u, x + 3, l3, r3);
      *reinterpret_cast<uint4*>(orow + x) = v;
    }
  }
  __syncwarp();
}

// One warp per x row.  Shared memory per warp: site bitmask of the row and, per
// word, the nearest site position at-or-before / at-or-after it.
template <int MODE>
__global__ void __launch_bounds__(kXWarps * 32)
edt_x_kernel(const uint8_t* __restrict__ a, const uint8_t* __restrict__ b, Dims dm, uint32_t* __restrict__ out,
             uint32_t* __restrict__ selbits, Counters* __restrict__ ctr) {
  extern __shared__ uint32_t smem[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nw = dm.nw();
  uint32_t* mask = smem + (size_t)warp * 3 * nw;
  int* lastpos = reinterpret_cast<int*>(mask + nw);
  int* firstpos = lastpos + nw;
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
    x_row_distances(mask, lastpos, firstpos, nw, dm.w, lane, out + base);
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
// then computed four adjacent voxels per lane (16-byte stores).
template <int MODE>
__global__ void __launch_bounds__(kXWarps * 32, 5)
edt_x_vec_kernel(const uint8_t* __restrict__ a, const uint8_t* __restrict__ b, Dims dm, uint32_t* __restrict__ out,
                 uint32_t* __restrict__ selbits, Counters* __restrict__ ctr) {
  extern __shared__ uint32_t smem[];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nw = dm.nw();
  uint32_t* mask = smem + (size_t)warp * 3 * nw;
  int* lastpos = reinterpret_cast<int*>(mask + nw);
  int* firstpos = lastpos + nw;
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
    x_row_distances4(mask, lastpos, firstpos, nw, dm.w, lane, out + base);
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
// kWinHalo).  Each lane computes four adjacent outputs q .. q+3 of its column
// at once: the loads at q - e and q + 3 + e serve all four (at distances
// k + e and 3 - k + e for output q + k), so a scan step costs two shared loads
// for four outputs.  The scan runs outwards until e^2 reaches the largest of
// the four minima.  Lines with an output whose window exceeds the halo (or
// that have no site at all, f = kInfSq) are marked in `redo`; the
// lower-envelope kernel recomputes exactly those lines afterwards.
constexpr int kWinTL = 128;
constexpr int kWinHalo = 64;
constexpr int kWinThreads = 256;
constexpr int kWinWarps = kWinThreads / 32;
constexpr int kWinGroup = 4;  // adjacent outputs per lane
static_assert(kWinTL == kWinWarps * kWinGroup * 4, "four groups of four outputs per warp");
static_assert(kInfSq + (kWinHalo + 6u) * (kWinHalo + 6u) > kInfSq, "the window scan adds distance^2 to kInfSq");

// floor(sqrt(f)) + 2 >= isqrt(f - 1) + 1 for f >= 1: the halo that f needs,
// from the hardware reciprocal square root (error far below one).
__device__ __forceinline__ uint32_t halo_need(uint32_t f) {
  const float ff = (float)f;
  return (uint32_t)(ff * rsqrtf(ff)) + 2u;
}

// One scan step at offset e: left candidate L = f(q - e), right R = f(q + 3 + e).
__device__ __forceinline__ void win_step(uint32_t L, uint32_t R, uint32_t e, uint32_t& b0, uint32_t& b1,
                                         uint32_t& b2, uint32_t& b3) {
  const uint32_t s0 = e * e, s1 = s0 + 2u * e + 1u, s2 = s1 + 2u * e + 3u, s3 = s2 + 2u * e + 5u;
  b0 = __viaddmin_u32(L, s0, __viaddmin_u32(R, s3, b0));
  b1 = __viaddmin_u32(L, s1, __viaddmin_u32(R, s2, b1));
  b2 = __viaddmin_u32(L, s2, __viaddmin_u32(R, s1, b2));
  b3 = __viaddmin_u32(L, s3, __viaddmin_u32(R, s0, b3));
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
#pragma unroll 1
  for (int j = 0; j < kPer / kWinGroup; ++j) {
    const int i = kWinGroup * (warp + kWinWarps * j);  // first of the group's rows (warp-uniform)
    const int q = q0 + i;
    if (!xin || q >= n) continue;
    const int m = min(kWinGroup, n - q);  // outputs inside the line
    const uint32_t* col = buf + (kWinHalo + i) * 32 + lane;
    const uint32_t c0 = col[0], c1 = col[32], c2 = col[64], c3 = col[96];
    // the group's own values (rows past the line end hold kInfSq)
    uint32_t b0 = __viaddmin_u32(c1, 1u, __viaddmin_u32(c2, 4u, __viaddmin_u32(c3, 9u, c0)));
    uint32_t b1 = __viaddmin_u32(c0, 1u, __viaddmin_u32(c2, 1u, __viaddmin_u32(c3, 4u, c1)));
    uint32_t b2 = __viaddmin_u32(c0, 4u, __viaddmin_u32(c1, 1u, __viaddmin_u32(c3, 1u, c2)));
    uint32_t b3 = __viaddmin_u32(c0, 9u, __viaddmin_u32(c1, 4u, __viaddmin_u32(c2, 1u, c3)));
    if (m < 4) {  // outputs past the line end take no part in the stopping test
      b3 = 0u;
      if (m < 3) b2 = 0u;
      if (m < 2) b1 = 0u;
    }
    // after offsets 1 .. e-1 every candidate within distance e of every output
    // has been tried, so the scan stops once e^2 reaches the largest minimum
    bool done = true;
    int e = 1;
    uint32_t mx = max(max(b0, b1), max(b2, b3));
    while ((uint32_t)(e * e) < mx) {
      if (e + 3 <= halo) {
#pragma unroll
        for (int u = 0; u < 4; ++u)
          win_step(col[-(e + u) * 32], col[(3 + e + u) * 32], (uint32_t)(e + u), b0, b1, b2, b3);
        e += 4;
      } else {
        if (e > halo) {
          done = false;
          break;
        }
        win_step(col[-e * 32], col[(3 + e) * 32], (uint32_t)e, b0, b1, b2, b3);
        ++e;
      }
      mx = max(max(b0, b1), max(b2, b3));
    }
    if (!done) {
      bad = true;
      continue;
    }
    uint32_t* op = out + base + (long long)q * stride;
    op[0] = b0;
    if (m > 1) op[stride] = b1;
    if (m > 2) op[2 * stride] = b2;
    if (m > 3) op[3 * stride] = b3;
    localmax = max(localmax, mx);
  }
  if (bad) redo[orow * (long long)w + x] = 1u;
  if (track_max) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) localmax = max(localmax, __shfl_xor_sync(0xffffffffu, localmax, o));
    if (lane == 0 && localmax) atomicMax(&ctr->rmax, localmax);
  }
}


// ---- TMA-staged window pass -------------------------------------------------
// Same computation as edt_window_kernel, with the staging done by the tensor
// memory accelerator: one thread issues a single 3-D tiled copy of the block's
// 128 output rows plus a full 64-row halo on each side (256 rows of 32 x,
// 32 KB) into shared memory and every thread waits on the copy's mbarrier.
// Rows outside the line arrive zero-filled and are set to kInfSq ("no site")
// by the blocks at the line ends.  The per-thread load, staging and halo
// sizing work of the plain kernel disappears; the scan may always run to the
// full halo.  Needs w a multiple of 4 (16-byte row pitch) and 16-byte aligned
// buffers; other volumes, and the z pass, take edt_window_kernel.
constexpr int kTmaRows = kWinTL + 2 * kWinHalo;
static_assert(kTmaRows <= 256, "a TMA box dimension is at most 256");
constexpr long long kWaitCycles = 4000000000ll;  // ~2 s at 2 GHz: a copy that has not landed by then never will

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Bounded wait for phase `parity` of the mbarrier at `bar`: false once `limit`
// cycles have passed (limit 0: gives up before the first try).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long limit) {
  const long long t0 = clock64();
  for (;;) {
    if (clock64() - t0 >= limit) return false;
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
  }
}

__global__ void __launch_bounds__(kWinThreads)
edt_window_tma_kernel(const __grid_constant__ CUtensorMap tin, uint32_t* __restrict__ out, int axis, int n,
                      long long stride, int w, long long outer_stride, int nxt, int nchunk,
                      uint8_t* __restrict__ redo, Counters* __restrict__ ctr, int track_max, long long wait_limit) {
  __shared__ alignas(128) uint32_t buf[kTmaRows * 32];
  __shared__ alignas(8) unsigned long long bar;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long bid = blockIdx.x;
  const int xt = (int)(bid % nxt);
  const int chunk = (int)((bid / nxt) % nchunk);
  const int orow = (int)(bid / ((long long)nxt * nchunk));
  const int x = xt * 32 + lane;
  const bool xin = x < w;
  const int q0 = chunk * kWinTL;
  const uint32_t b = smem_u32(&bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int c0 = xt * 32, ql = q0 - kWinHalo;  // x start: 128-byte multiple; rows may start below 0
    const int c1 = axis == 1 ? ql : orow, c2 = axis == 1 ? orow : ql;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(kTmaRows * 32 * 4)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(buf)), "l"(reinterpret_cast<unsigned long long>(&tin)), "r"(c0), "r"(c1), "r"(c2), "r"(b)
        : "memory");
  }
  const bool landed = mbar_wait(b, 0u, wait_limit);
  if (!__syncthreads_and(landed)) {
    // the copy did not complete in time: report it, give the copy in flight a
    // second wait with the full bound (it writes into this block's shared
    // memory) and leave
    if (threadIdx.x == 0) atomicOr(&ctr->status, 1u);
    mbar_wait(b, 0u, kWaitCycles);
    return;
  }
  if (q0 < kWinHalo || q0 + kWinTL + kWinHalo > n) {
    for (int k = threadIdx.x; k < kTmaRows * 32; k += kWinThreads) {
      const int q = q0 - kWinHalo + (k >> 5);
      if (q < 0 || q >= n) buf[k] = kInfSq;
    }
    __syncthreads();
  }
  const long long base = (long long)orow * outer_stride + x;
  uint32_t localmax = 0;
  bool bad = false;
#pragma unroll 1
  for (int j = 0; j < kWinTL / (kWinGroup * kWinWarps); ++j) {
    const int i = kWinGroup * (warp + kWinWarps * j);
    const int q = q0 + i;
    if (!xin || q >= n) continue;
    const int m = min(kWinGroup, n - q);
    const uint32_t* col = buf + (kWinHalo + i) * 32 + lane;
    const uint32_t c0 = col[0], c1 = col[32], c2 = col[64], c3 = col[96];
    uint32_t b0 = __viaddmin_u32(c1, 1u, __viaddmin_u32(c2, 4u, __viaddmin_u32(c3, 9u, c0)));
    uint32_t b1 = __viaddmin_u32(c0, 1u, __viaddmin_u32(c2, 1u, __viaddmin_u32(c3, 4u, c1)));
    uint32_t b2 = __viaddmin_u32(c0, 4u, __viaddmin_u32(c1, 1u, __viaddmin_u32(c3, 1u, c2)));
    uint32_t b3 = __viaddmin_u32(c0, 9u, __viaddmin_u32(c1, 4u, __viaddmin_u32(c2, 1u, c3)));
    if (m < 4) {
      b3 = 0u;
      if (m < 3) b2 = 0u;
      if (m < 2) b1 = 0u;
    }
    bool done = true;
    int e = 1;
    uint32_t mx = max(max(b0, b1), max(b2, b3));
    while ((uint32_t)(e * e) < mx) {
      if (e + 3 <= kWinHalo) {
#pragma unroll
        for (int u = 0; u < 4; ++u)
          win_step(col[-(e + u) * 32], col[(3 + e + u) * 32], (uint32_t)(e + u), b0, b1, b2, b3);
        e += 4;
      } else {
        if (e > kWinHalo) {
          done = false;
          break;
        }
        win_step(col[-e * 32], col[(3 + e) * 32], (uint32_t)e, b0, b1, b2, b3);
        ++e;
      }
      mx = max(max(b0, b1), max(b2, b3));
    }
    if (!done) {
      bad = true;
      continue;
    }
    uint32_t* op = out + base + (long long)q * stride;
    op[0] = b0;
    if (m > 1) op[stride] = b1;
    if (m > 2) op[2 * stride] = b2;
    if (m > 3) op[3 * stride] = b3;
    localmax = max(localmax, mx);
  }
  if (bad) redo[(long long)orow * w + x] = 1u;
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
                   (!two || (reinterpret_cast<uintptr_t>(b) & 15u) == 0) &&
                   (reinterpret_cast<uintptr_t>(out) & 15u) == 0;
  if (vec) {
    if (smem > 48 * 1024) {
      cudaError_t e =
          cudaFuncSetAttribute(edt_x_vec_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
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

namespace {

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

// Tensor map of a u32 volume (x fastest) whose box is 32 x by `rows` along the
// pass axis; false when the volume or buffer does not meet TMA's rules.
bool window_map(CUtensorMap* map, const uint32_t* vol, Dims dm, int axis, unsigned rows) {
  if (dm.w % 4 != 0 || (reinterpret_cast<uintptr_t>(vol) & 15u) != 0) return false;
  const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)dm.w, (cuuint64_t)dm.h, (cuuint64_t)dm.d};
  const cuuint64_t pitch[2] = {(cuuint64_t)dm.w * 4, (cuuint64_t)dm.w * dm.h * 4};
  const cuuint32_t box[3] = {32u, axis == 1 ? rows : 1u, axis == 1 ? 1u : rows};
  const cuuint32_t unit[3] = {1u, 1u, 1u};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, const_cast<uint32_t*>(vol), dims, pitch, box, unit,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

cudaError_t launch_edt_window(int axis, const uint32_t* in, uint32_t* out, Dims dm, void* scratch, uint8_t* redo,
                              Counters* ctr, long long wait_cycles, cudaStream_t s, unsigned long long* launches) {
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
  // TMA staging for the y pass only: a z-pass box spans 256 rows a whole
  // slice apart (a different page each), which the copy engine translates one
  // by one; there the per-thread loads measured faster (2.2 against 3.0 ms on
  // 1024^3 bone).
  CUtensorMap map;
  if (axis == 1 && window_map(&map, in, dm, axis, kTmaRows)) {
    edt_window_tma_kernel<<<(unsigned)blocks, kWinThreads, 0, s>>>(map, out, axis, n, stride, dm.w, outer, nxt,
                                                                   nchunk, redo, ctr, axis == 2 ? 1 : 0,
                                                                   wait_cycles < 0 ? kWaitCycles : wait_cycles);
  } else {
    edt_window_kernel<<<(unsigned)blocks, kWinThreads, 0, s>>>(in, out, n, stride, dm.w, outer, nxt, nchunk, redo,
                                                               ctr, axis == 2 ? 1 : 0);
  }
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
