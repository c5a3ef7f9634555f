// The statistics' f64 sums in the reference's own order (metrics.rs:215-226).
//
// nonzero_stats adds v = (raw * scale_f32) as f64 and v * v, one value after
// the other in index order, into two f64 accumulators.  Its mean and SD are
// functions of those two rounded sums, so reproducing them bit for bit means
// reproducing every rounding of that sequence.  This file does it in parallel.
//
// The idea.  Let s be the running sum.  While s stays inside one binade
// [2^E, 2^(E+1)), every representable value there is a multiple of
// U = 2^(E-52), so s + v rounds to s + (v rounded to a multiple of U) -- an
// integer increment of s/U that depends on v and E only, except when v's
// remainder is exactly U/2: then round-to-nearest-even picks the increment
// that makes s/U even, which depends on the parity of s/U.  So within one
// binade an element is a function of the parity P of s/U:
//     P -> (increment(P), new parity(P)),
// and a run of elements composes into a function of the same shape (two
// 64-bit increments and two parity bits).  Composition is associative, so
// runs reduce in parallel, in order.  A run's function is valid if s/U after
// it is at most 2^53 (every intermediate state then stayed in the binade, or
// reached 2^(E+1) exactly, which both roundings agree on); otherwise the run
// crossed into the next binade and its elements are replayed.
//
// The pipeline.  The map is cut into chunks of kChunk voxels in index order.
//   1. approximate sums of v and v*v per chunk (f32, on values scaled by a
//      power of two) and per block of 32 chunks (fixed point);
//   2. an exclusive scan of the block sums: approximate prefix sums;
//   3. per chunk, the binade the running sum is predicted to stay in (from the
//      approximate prefix, with a relative margin), and the chunk's function
//      for that binade, folded value by value by one thread; per block of 32
//      chunks, the composition when all its chunks share one binade;
//   4. compositions of 32 blocks at each further level;
//   5. a walker (one warp per sum) that follows the sequence from s = 0: it
//      skips empty runs before the first value, applies the largest aligned
//      run whose predicted binade is the one s is in and whose result stays
//      in it (32 entries of a level at a time, composed by a warp
//      reduction), and replays a chunk where no prediction holds -- at the
//      ~30 binade crossings of each sum: lanes fold their values, a warp
//      scan finds the lane whose values leave the binade, and that lane adds
//      them one by one (integer increments of s/U, and a hardware f64
//      addition, the reference's own operation, for the value that crosses).
// Every step the walker takes is checked against the exact state, so a wrong
// prediction costs time, never exactness.  No per-value f64 arithmetic: the
// GB300's f64 rate is a small fraction of its f32 and integer rates.  Not a
// reference function: the reference's loop is serial (metrics.rs:215-226).
#include <climits>
#include <cstdint>

#include "kernels.h"

namespace bm {

namespace {

constexpr int kChunk = 256;                      // voxels per chunk
constexpr unsigned long long kTwo53 = 1ull << 53;
constexpr unsigned long long kSat = 1ull << 54;  // saturated increment: never valid
// Relative margin of the binade prediction.  The approximate prefix sums come
// from f32 chunk sums in fixed point (errors of ~2^-21 of a chunk each,
// shrinking relative to the prefix as it grows); the sequential sum differs
// from the exact prefix by ~sqrt(k) 2^-53.  A miss only sends a chunk to the
// replay.
constexpr double kMargin = 1.0 / 16777216.0;  // 2^-24
// Fixed-point scale of the approximate sums (values scaled into [1, 2)):
// 2^24 units per unit, so a 2^32-voxel map's sums of squares fit 64 bits.
constexpr float kFix = 16777216.0f;
constexpr double kUnfix = 1.0 / 16777216.0;

// meta word of a function: 0 = invalid (no prediction); bit 2 = identity valid
// in every binade; else bits 3.. hold E + 2048; bits 0, 1 = out parity for
// input parity 0, 1.
struct Fn {
  unsigned long long i0, i1;
  uint32_t meta;
};

__device__ __forceinline__ unsigned long long sat_add(unsigned long long a, unsigned long long b) {
  const unsigned long long c = a + b;
  return (c >= kSat || c < a) ? kSat : c;
}

__device__ __forceinline__ Fn fn_identity() { return Fn{0ull, 0ull, 4u | 2u}; }

__device__ __forceinline__ uint32_t meta_of(int E, uint32_t o0, uint32_t o1) {
  return ((uint32_t)(E + 2048) << 3) | o0 | (o1 << 1);
}

// F then G.  Binades: an identity-everywhere side takes the other's; two
// different binades, or an invalid side, give invalid.
__device__ __forceinline__ Fn compose(const Fn& F, const Fn& G) {
  if (F.meta == 0u || G.meta == 0u) return Fn{0ull, 0ull, 0u};
  const uint32_t f0 = F.meta & 1u, f1 = (F.meta >> 1) & 1u;
  Fn H;
  H.i0 = sat_add(F.i0, f0 ? G.i1 : G.i0);
  H.i1 = sat_add(F.i1, f1 ? G.i1 : G.i0);
  const uint32_t h0 = (G.meta >> f0) & 1u, h1 = (G.meta >> f1) & 1u;
  const bool fw = (F.meta & 4u) != 0u, gw = (G.meta & 4u) != 0u;
  uint32_t ebits;
  if (fw && gw) {
    ebits = 4u;
  } else if (fw) {
    ebits = G.meta & ~7u;
  } else if (gw) {
    ebits = F.meta & ~7u;
  } else {
    if ((F.meta >> 3) != (G.meta >> 3)) return Fn{0ull, 0ull, 0u};
    ebits = F.meta & ~7u;
  }
  H.meta = ebits | h0 | (h1 << 1);
  return H;
}

__device__ __forceinline__ Fn shfl_fn(const Fn& f, int src) {
  Fn r;
  r.i0 = __shfl_sync(0xffffffffu, f.i0, src);
  r.i1 = __shfl_sync(0xffffffffu, f.i1, src);
  r.meta = __shfl_sync(0xffffffffu, f.meta, src);
  return r;
}

__device__ __forceinline__ Fn shfl_down_fn(const Fn& f, int o) {
  Fn r;
  r.i0 = __shfl_down_sync(0xffffffffu, f.i0, o);
  r.i1 = __shfl_down_sync(0xffffffffu, f.i1, o);
  r.meta = __shfl_down_sync(0xffffffffu, f.meta, o);
  return r;
}

// In-order reduction of the warp's 32 functions (lane 0 first); result in lane 0.
__device__ __forceinline__ Fn warp_reduce_fn(Fn f, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const Fn g = shfl_down_fn(f, o);
    if ((lane & (2 * o - 1)) == 0 && lane + o < 32) f = compose(f, g);
  }
  return f;
}

// The value nonzero_stats adds for a map entry (metrics.rs:216-224): v =
// raw * scale_f32 in f32, then x = v as f64 (or x * x for the sum of squares,
// exact in f64), as an integer mantissa and a power of two, x = M * 2^k (M = 0
// when the entry is skipped or v is 0; k = INT_MAX marks +inf).
struct Term {
  unsigned long long M;
  int k;
};

__device__ __forceinline__ Term term(float raw, float scale, bool sq) {
  Term t{0ull, 0};
  if (!(raw > 0.0f) || !isfinite(raw)) return t;
  const uint32_t b = __float_as_uint(__fmul_rn(raw, scale));
  const uint32_t ef = (b >> 23) & 0xffu;
  unsigned long long m = b & 0x7fffffu;
  if (ef == 0xffu) {  // the f32 product overflowed: +inf
    t.M = ~0ull;
    t.k = INT_MAX;
    return t;
  }
  if (ef) m |= 1ull << 23;
  if (m == 0) return t;
  const int e = (ef ? (int)ef : 1) - 150;
  t.M = sq ? m * m : m;
  t.k = sq ? 2 * e : e;
  return t;
}

// x itself, for the additions made in f64 (a binade crossing, the first value).
__device__ __forceinline__ double term_value(float raw, float scale, bool sq) {
  const double v = (double)__fmul_rn(raw, scale);
  return sq ? __dmul_rn(v, v) : v;
}

__device__ __forceinline__ int binade_of(double s) {
  return (int)((__double_as_longlong(s) >> 52) & 0x7ff) - 1023;
}

__device__ __forceinline__ unsigned long long units_of(double s) {  // s / 2^(E-52), in [2^52, 2^53)
  return ((unsigned long long)__double_as_longlong(s) & ((1ull << 52) - 1ull)) | (1ull << 52);
}

__device__ __forceinline__ double from_units(unsigned long long u, int E) {  // u in [2^52, 2^53]
  if (u == kTwo53) return __longlong_as_double((long long)(E + 1 + 1023) << 52);
  return __longlong_as_double(((long long)(E + 1023) << 52) | (long long)(u & ((1ull << 52) - 1ull)));
}

// Apply f to s (s > 0, finite); false (s unchanged) when f does not hold there.
__device__ __forceinline__ bool apply_fn(const Fn& f, double& s) {
  if (f.meta == 0u) return false;
  if (f.meta & 4u) return true;  // identity
  const int E = binade_of(s);
  if ((int)(f.meta >> 3) - 2048 != E) return false;
  const unsigned long long u = units_of(s);
  const unsigned long long nu = sat_add(u, (u & 1ull) ? f.i1 : f.i0);
  if (nu > kTwo53) return false;
  s = from_units(nu, E);
  return true;
}

__device__ __forceinline__ void load8(const float* __restrict__ map, long long n, long long base, float (&v)[8]) {
  if (base + 8 <= n && (reinterpret_cast<uintptr_t>(map + base) & 15u) == 0) {
    const float4 a = *reinterpret_cast<const float4*>(map + base);
    const float4 b = *reinterpret_cast<const float4*>(map + base + 4);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  } else {
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = base + j < n ? map[base + j] : 0.0f;
  }
}

// Clamped f32 exponent field of the map's largest value v = raw * scale_f32.
__device__ __forceinline__ int max_exponent_field(uint32_t maxbits) {
  const int ef = (int)((maxbits >> 23) & 0xffu);
  return ef < 1 ? 1 : ef > 253 ? 253 : ef;
}

// Power of two that brings the largest value of the map into [1, 2): the
// approximate sums run in f32 on values scaled by it (no overflow, even for
// their squares).
__device__ __forceinline__ float norm_factor(uint32_t maxbits) {
  return __uint_as_float((uint32_t)(254 - max_exponent_field(maxbits)) << 23);  // 2^(127 - ef)
}

__device__ __forceinline__ unsigned long long to_fixed(float x) {
  return (unsigned long long)__fmul_rn(x, kFix);
}

// 1. Approximate sums per chunk of v and v^2 (scaled by norm_factor, in f32)
// and per block of 32 chunks (fixed point); one warp per block, lane j keeps chunk j.
__global__ void __launch_bounds__(256)
osum_chunk_kernel(const float* __restrict__ map, long long n, float scale, long long nchunks,
                  const uint32_t* __restrict__ maxbits, float* __restrict__ cs, float* __restrict__ cq,
                  unsigned long long* __restrict__ bs, unsigned long long* __restrict__ bq) {
  const int lane = threadIdx.x & 31;
  const long long blk = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long c0 = blk * 32;
  if (c0 >= nchunks) return;
  const float nf = norm_factor(*maxbits);
  float my_s = 0.0f, my_q = 0.0f;
  for (int j = 0; j < 32 && c0 + j < nchunks; ++j) {
    float v[8];
    load8(map, n, (c0 + j) * kChunk + lane * 8, v);
    float s = 0.0f, q = 0.0f;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const float raw = v[t];
      const float x = (raw > 0.0f && isfinite(raw)) ? __fmul_rn(__fmul_rn(raw, scale), nf) : 0.0f;
      s += x;
      q += x * x;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_xor_sync(0xffffffffu, s, o);
      q += __shfl_xor_sync(0xffffffffu, q, o);
    }
    if (lane == j) {
      my_s = s;
      my_q = q;
    }
  }
  if (c0 + lane < nchunks) {
    cs[c0 + lane] = my_s;
    cq[c0 + lane] = my_q;
  }
  unsigned long long ts = c0 + lane < nchunks ? to_fixed(my_s) : 0ull;
  unsigned long long tq = c0 + lane < nchunks ? to_fixed(my_q) : 0ull;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ts += __shfl_xor_sync(0xffffffffu, ts, o);
    tq += __shfl_xor_sync(0xffffffffu, tq, o);
  }
  if (lane == 0) {
    bs[blk] = ts;
    bq[blk] = tq;
  }
}

// 2. Exclusive scan of the block sums in place, fixed point (one CTA of 1024 threads).
__global__ void __launch_bounds__(1024) osum_scan_kernel(unsigned long long* __restrict__ bs,
                                                         unsigned long long* __restrict__ bq, long long nb) {
  __shared__ unsigned long long ws[32], wq[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long per = (nb + 1023) / 1024;
  const long long b0 = (long long)tid * per, b1 = b0 + per < nb ? b0 + per : nb;
  unsigned long long ls = 0, lq = 0;
  for (long long b = b0; b < b1; ++b) {
    ls += bs[b];
    lq += bq[b];
  }
  unsigned long long is = ls, iq = lq;  // inclusive scan of the threads' totals
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long us = __shfl_up_sync(0xffffffffu, is, o), uq = __shfl_up_sync(0xffffffffu, iq, o);
    if (lane >= o) {
      is += us;
      iq += uq;
    }
  }
  if (lane == 31) {
    ws[warp] = is;
    wq[warp] = iq;
  }
  __syncthreads();
  if (warp == 0) {
    unsigned long long a = ws[lane], b = wq[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long ua = __shfl_up_sync(0xffffffffu, a, o), ub = __shfl_up_sync(0xffffffffu, b, o);
      if (lane >= o) {
        a += ua;
        b += ub;
      }
    }
    ws[lane] = a - ws[lane];
    wq[lane] = b - wq[lane];
  }
  __syncthreads();
  unsigned long long rs = ws[warp] + is - ls, rq = wq[warp] + iq - lq;
  for (long long b = b0; b < b1; ++b) {
    const unsigned long long ts = bs[b], tq = bq[b];
    bs[b] = rs;
    bq[b] = rq;
    rs += ts;
    rq += tq;
  }
}

// Binade the running sum is predicted to stay in over [P, P + A] * 2^eshift
// (INT_MIN: none).  P and A are approximate (f32 chunk sums), hence the margin.
__device__ __forceinline__ int predict(double P, double A, int eshift) {
  const double lo = P * (1.0 - kMargin), hi = (P + A) * (1.0 + kMargin);
  if (!(lo > 0.0) || !(hi < 1e300)) return INT_MIN;
  const int e0 = binade_of(lo), e1 = binade_of(hi);
  return e0 == e1 ? e0 + eshift : INT_MIN;
}

struct Level {
  unsigned long long* i0;
  unsigned long long* i1;
  uint32_t* meta;
};

__device__ __forceinline__ void store_fn(const Level& L, long long i, const Fn& f) {
  L.i0[i] = f.i0;
  L.i1[i] = f.i1;
  L.meta[i] = f.meta;
}

__device__ __forceinline__ Fn load_fn(const Level& L, long long i) { return Fn{L.i0[i], L.i1[i], L.meta[i]}; }

// A chunk's function accumulated element by element by one thread: the
// increments and output parities for input parity 0 and 1 (no saturation
// needed inside a chunk: kChunk increments of at most 2^54 fit 64 bits).
struct Acc {
  unsigned long long i0, i1;
  uint32_t o0, o1;
};

// Adds the element M * 2^k to acc for the binade whose ulp is 2^em52; mbits
// bounds M (M < 2^mbits).
__device__ __forceinline__ void acc_elem(Acc& A, unsigned long long M, int k, int em52, int mbits) {
  if (k == INT_MAX) {  // +inf: never within a binade
    A.i0 = A.i1 = kSat;
    return;
  }
  const int sh = em52 - k;
  unsigned long long c;
  if (sh <= 0) {
    c = (sh <= -54 || (M >> (54 + sh)) != 0) ? kSat : (M << -sh);  // M * 2^-sh >= 2^54: saturated
  } else if (sh > mbits) {
    return;  // below half an ulp: lost
  } else {
    const unsigned long long a = M >> sh, rem = M & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
    if (rem == half) {  // a tie: the increment that leaves s/U even, for each input parity
      A.i0 += a + ((A.o0 + a) & 1ull);
      A.i1 += a + ((A.o1 + a) & 1ull);
      A.o0 = 0u;
      A.o1 = 0u;
      return;
    }
    c = a + (rem > half ? 1ull : 0ull);
  }
  A.i0 += c;
  A.i1 += c;
  A.o0 ^= (uint32_t)(c & 1ull);
  A.o1 ^= (uint32_t)(c & 1ull);
}

__device__ __forceinline__ Fn acc_fn(const Acc& A, bool any, int E) {
  if (!any) return fn_identity();
  if (E == INT_MIN) return Fn{0ull, 0ull, 0u};
  return Fn{A.i0 >= kSat ? kSat : A.i0, A.i1 >= kSat ? kSat : A.i1, meta_of(E, A.o0, A.o1)};
}

constexpr int kTileStride = 33;  // words per row of a warp's transpose tile (conflict-free column reads)

// 3. Predicted binade and function of every chunk, for both sums, and the
// first aggregate level.  One warp per block of 32 chunks; lane j owns chunk
// j and folds its 256 values in order.  The values reach the lanes through a
// shared-memory transpose of 32 values of each chunk at a time, so the
// global loads stay coalesced.
__global__ void __launch_bounds__(256)
osum_fn_kernel(const float* __restrict__ map, long long n, float scale, long long nchunks,
               const uint32_t* __restrict__ maxbits, const float* __restrict__ cs, const float* __restrict__ cq,
               const unsigned long long* __restrict__ bps, const unsigned long long* __restrict__ bpq, Level s0,
               Level q0, Level s1, Level q1) {
  __shared__ float tile[8][32 * kTileStride];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long blk = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long c0 = blk * 32;
  if (c0 >= nchunks) return;
  float* T = tile[warp];
  const bool mine = c0 + lane < nchunks;
  const unsigned long long as = mine ? to_fixed(cs[c0 + lane]) : 0ull, aq = mine ? to_fixed(cq[c0 + lane]) : 0ull;
  unsigned long long ps = as, pq = aq;  // inclusive scan within the block
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long us = __shfl_up_sync(0xffffffffu, ps, o), uq = __shfl_up_sync(0xffffffffu, pq, o);
    if (lane >= o) {
      ps += us;
      pq += uq;
    }
  }
  // the approximate sums are of values scaled by 2^(127 - ef): undo it in the binade
  const int shift = max_exponent_field(*maxbits) - 127;
  const int es = predict((double)(bps[blk] + ps - as) * kUnfix, (double)as * kUnfix, shift);
  const int eq = predict((double)(bpq[blk] + pq - aq) * kUnfix, (double)aq * kUnfix, 2 * shift);
  const int ems = es == INT_MIN ? 0 : es - 52, emq = eq == INT_MIN ? 0 : eq - 52;
  Acc A{0ull, 0ull, 0u, 1u}, Q{0ull, 0ull, 0u, 1u};
  bool any = false;
  const long long base0 = c0 * kChunk;
  const bool vec = (reinterpret_cast<uintptr_t>(map) & 15u) == 0 && base0 + 32ll * kChunk <= n;
  for (int t = 0; t < kChunk / 32; ++t) {
    // T[j][x] = value t*32 + x of chunk j
    if (vec) {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int j = 4 * i + (lane >> 3), x = 4 * (lane & 7);
        const float4 v = *reinterpret_cast<const float4*>(map + base0 + (long long)j * kChunk + t * 32 + x);
        float* r = T + j * kTileStride + x;
        r[0] = v.x;
        r[1] = v.y;
        r[2] = v.z;
        r[3] = v.w;
      }
    } else {
      for (int j = 0; j < 32; ++j) {
        const long long idx = base0 + (long long)j * kChunk + t * 32 + lane;
        T[j * kTileStride + lane] = idx < n ? map[idx] : 0.0f;
      }
    }
    __syncwarp();
    if (mine) {
#pragma unroll 4
      for (int x = 0; x < 32; ++x) {
        const Term a = term(T[lane * kTileStride + x], scale, false);
        if (a.M) {
          any = true;
          if (es != INT_MIN) acc_elem(A, a.M, a.k, ems, 24);
          if (eq != INT_MIN)
            acc_elem(Q, a.k == INT_MAX ? a.M : a.M * a.M, a.k == INT_MAX ? INT_MAX : 2 * a.k, emq, 48);
        }
      }
    }
    __syncwarp();
  }
  const Fn my_s = acc_fn(A, any, es), my_q = acc_fn(Q, any, eq);
  if (mine) {
    store_fn(s0, c0 + lane, my_s);
    store_fn(q0, c0 + lane, my_q);
  }
  const Fn as_ = warp_reduce_fn(mine ? my_s : fn_identity(), lane);
  const Fn aq_ = warp_reduce_fn(mine ? my_q : fn_identity(), lane);
  if (lane == 0) {
    store_fn(s1, blk, as_);
    store_fn(q1, blk, aq_);
  }
}

// 4. Next aggregate level: compositions of 32 consecutive entries.
__global__ void __launch_bounds__(256) osum_level_kernel(Level s_in, Level q_in, long long n_in, Level s_out,
                                                         Level q_out) {
  const int lane = threadIdx.x & 31;
  const long long blk = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long i = blk * 32 + lane;
  if (blk * 32 >= n_in) return;
  const Fn fs = warp_reduce_fn(i < n_in ? load_fn(s_in, i) : fn_identity(), lane);
  const Fn fq = warp_reduce_fn(i < n_in ? load_fn(q_in, i) : fn_identity(), lane);
  if (lane == 0) {
    store_fn(s_out, blk, fs);
    store_fn(q_out, blk, fq);
  }
}

constexpr int kMaxLevels = 8;

struct Walk {
  Level lv[kMaxLevels];  // lv[0]: chunks; lv[L]: blocks of 32^L chunks
  long long cnt[kMaxLevels];
  int nlev;
};

// Adds values vals[j0 .. 8) to s one after the other as the reference does
// (one thread): s kept as an integer count of its binade's ulps plus each
// value's rounded increment (round half to even on that count), a hardware
// f64 addition -- the reference's own operation -- for the first value
// (s = 0), for a value that leaves the binade, and for +inf.
__device__ double add_serially(double s, const float (&vals)[8], int j0, float scale, bool sq) {
  bool in_units = isfinite(s) && s > 0.0;
  int E = in_units ? binade_of(s) : 0;
  unsigned long long u = in_units ? units_of(s) : 0ull;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    if (j < j0) continue;
    const Term t = term(vals[j], scale, sq);
    if (!t.M) continue;  // skipped (metrics.rs:216-218) or zero
    if (in_units && t.k != INT_MAX) {
      const int sh = (E - 52) - t.k;
      unsigned long long a = 0;
      bool tie = false, fits = true;
      if (sh <= 0) {
        fits = sh > -54 && (t.M >> (54 + sh)) == 0;
        a = fits ? t.M << -sh : 0;
      } else if (sh < 64) {
        const unsigned long long rem = t.M & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
        a = (t.M >> sh) + (rem > half ? 1ull : 0ull);
        tie = rem == half;
      }
      if (fits && u + a < kTwo53) {  // the exact sum stays below 2^(E+1): the binade's grid
        u += tie ? (a + ((u + a) & 1ull)) : a;
        if (u == kTwo53) {  // a tie rounded up to 2^(E+1): the next binade
          u = 1ull << 52;
          ++E;
        }
        continue;
      }
      s = from_units(u, E);
    }
    s = __dadd_rn(s, term_value(vals[j], scale, sq));  // metrics.rs:223-224
    in_units = isfinite(s) && s > 0.0;
    if (in_units) {
      E = binade_of(s);
      u = units_of(s);
    }
  }
  return in_units ? from_units(u, E) : s;
}

__device__ __forceinline__ Fn shfl_up_fn(const Fn& f, int o) {
  Fn r;
  r.i0 = __shfl_up_sync(0xffffffffu, f.i0, o);
  r.i1 = __shfl_up_sync(0xffffffffu, f.i1, o);
  r.meta = __shfl_up_sync(0xffffffffu, f.meta, o);
  return r;
}

// Inclusive in-order scan: lane j gets the composition of lanes 0 .. j.
__device__ __forceinline__ Fn warp_scan_fn(Fn f, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const Fn g = shfl_up_fn(f, o);
    if (lane >= o) f = compose(g, f);
  }
  return f;
}

// Replays chunk c from state s exactly as the reference adds.  Lane l holds
// values 8l .. 8l+7.  In s's binade every lane folds its values into one
// function and a warp scan composes them in order; the first lane whose
// prefix leaves the binade (or the lane holding the first value, s = 0)
// adds its values serially with add_serially, and the lanes after it are
// folded again in the new binade.  s is broadcast back.
__device__ void replay_chunk(const float* __restrict__ map, long long n, float scale, bool sq, long long c, double& s,
                             int lane) {
  float vals[8];
  load8(map, n, c * kChunk + lane * 8, vals);
  int start = 0;  // first lane not yet added
  const int mbits = sq ? 48 : 24;
  while (start < 32) {
    if (!isfinite(s)) break;  // +inf stays +inf
    int b;                    // the lane that adds serially
    if (s == 0.0) {
      bool any = false;
#pragma unroll
      for (int j = 0; j < 8; ++j) any = any || term(vals[j], scale, sq).M != 0;
      const unsigned m = __ballot_sync(0xffffffffu, lane >= start && any);
      if (!m) break;
      b = __ffs(m) - 1;
    } else {
      const int E = binade_of(s);
      const unsigned long long u0 = units_of(s);
      Acc A{0ull, 0ull, 0u, 1u};
      bool any = false;
      if (lane >= start) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const Term t = term(vals[j], scale, sq);
          if (t.M) {
            any = true;
            acc_elem(A, t.M, t.k, E - 52, mbits);
          }
        }
      }
      const Fn pre = warp_scan_fn(acc_fn(A, any, E), lane);
      const unsigned long long after = sat_add(u0, (u0 & 1ull) ? pre.i1 : pre.i0);
      const unsigned bad = __ballot_sync(0xffffffffu, lane >= start && after > kTwo53);
      if (!bad) {
        s = from_units(__shfl_sync(0xffffffffu, after, 31), E);
        break;
      }
      b = __ffs(bad) - 1;
      // lanes start .. b-1 stay in the binade: s after them
      const unsigned long long ub = __shfl_sync(0xffffffffu, after, b > 0 ? b - 1 : 0);
      if (b > start) s = from_units(ub, E);
    }
    double sb = 0.0;
    if (lane == b) sb = add_serially(s, vals, 0, scale, sq);
    s = __shfl_sync(0xffffffffu, sb, b);
    start = b + 1;
  }
  s = __shfl_sync(0xffffffffu, s, 0);
}

// Largest total of aggregate-level entries the walker keeps in shared memory.
constexpr size_t kWalkSmemBytes = 96 * 1024;
constexpr int kEntryBytes = 20;  // i0, i1, meta

// The lowest level (>= 1) from which all levels fit kWalkSmemBytes.
__host__ __device__ __forceinline__ int cached_from(const long long* cnt, int nlev) {
  long long bytes = 0;
  int L = nlev;
  while (L - 1 >= 1 && bytes + cnt[L - 1] * kEntryBytes <= (long long)kWalkSmemBytes) {
    --L;
    bytes += cnt[L] * kEntryBytes;
  }
  return L;
}

// 5. The walker: block 0 follows the sum of values, block 1 the sum of squares.
// The small aggregate levels are copied to shared memory first, so that the
// walker's level probes near a crossing cost shared-memory latency; level 0
// (and level 1 when large) stay in global memory.
__global__ void __launch_bounds__(32) osum_walk_kernel(const float* __restrict__ map, long long n, float scale,
                                                       Walk ws, Walk wq, double* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char walk_smem[];
  const bool sq = blockIdx.x == 1;
  Walk W = sq ? wq : ws;
  const int lane = threadIdx.x;
  const long long nchunks = W.cnt[0];
  {
    const int Lc = cached_from(W.cnt, W.nlev);
    unsigned char* p = walk_smem;
    for (int L = Lc; L < W.nlev; ++L) {
      const long long c = W.cnt[L];
      unsigned long long* i0 = reinterpret_cast<unsigned long long*>(p);
      unsigned long long* i1 = i0 + c;
      uint32_t* meta = reinterpret_cast<uint32_t*>(i1 + c);
      for (long long i = lane; i < c; i += 32) {
        i0[i] = W.lv[L].i0[i];
        i1[i] = W.lv[L].i1[i];
        meta[i] = W.lv[L].meta[i];
      }
      W.lv[L] = Level{i0, i1, meta};
      p += ((size_t)c * kEntryBytes + 15) & ~(size_t)15;
    }
    __syncwarp();
  }
  double s = 0.0;
  long long c = 0;
  while (c < nchunks) {
    if (!isfinite(s)) break;  // a value overflowed to +inf: the sum stays +inf
    // the highest level whose block starts at c and whose first entry applies:
    // before the first value (s = 0) only empty runs, after it runs in s's binade
    bool moved = false;
    for (int L = W.nlev - 1; L >= 0 && !moved; --L) {
      const int lg = 5 * L;
      const long long span = 1ll << lg;
      if (c & (span - 1)) continue;
      const long long q = c >> lg;
      // up to 32 entries of this level, but not past the next block of level L + 1
      const long long lim = (L + 1 < W.nlev) ? ((q / 32) + 1) * 32 : W.cnt[L];
      const long long qe = lim < W.cnt[L] ? lim : W.cnt[L];
      const long long i = q + lane;
      const Fn f = i < qe ? load_fn(W.lv[L], i) : Fn{0ull, 0ull, 0u};
      const int E = s == 0.0 ? INT_MIN : binade_of(s);
      const bool ok = (f.meta & 4u) || (E != INT_MIN && f.meta != 0u && (int)(f.meta >> 3) - 2048 == E);
      const unsigned okm = __ballot_sync(0xffffffffu, ok);
      const int t = (~okm) ? __ffs(~okm) - 1 : 32;  // entries 0 .. t-1 qualify
      if (t == 0) continue;
      if (E == INT_MIN) {  // empty chunks before the first value
        c = (q + t) * span < nchunks ? (q + t) * span : nchunks;
        moved = true;
        break;
      }
      Fn r = warp_reduce_fn(lane < t ? f : fn_identity(), lane);
      r = shfl_fn(r, 0);
      double s2 = s;
      if (apply_fn(r, s2)) {
        s = s2;
        c = (q + t) * span < nchunks ? (q + t) * span : nchunks;
        moved = true;
      } else if (t > 1) {
        // the run left the binade somewhere: take its first entry alone
        const Fn f0 = shfl_fn(f, 0);
        s2 = s;
        if (apply_fn(f0, s2)) {
          s = s2;
          c = (q + 1) * span < nchunks ? (q + 1) * span : nchunks;
          moved = true;
        }
      }
    }
    if (!moved) {
      replay_chunk(map, n, scale, sq, c, s, lane);
      ++c;
    }
  }
  if (lane == 0) out[sq ? 1 : 0] = s;
}

// Entry counts of the levels: chunks, then blocks of 32 per level up to a
// single entry; at least two levels.
int level_counts(long long nchunks, long long* cnt) {
  int nlev = 0;
  long long c = nchunks;
  for (;;) {
    cnt[nlev++] = c;
    if ((nlev >= 2 && c == 1) || nlev == kMaxLevels) break;
    c = (c + 31) / 32;
  }
  return nlev;
}

}  // namespace

size_t ordered_sum_scratch_bytes(long long n) {
  const long long nchunks = n > 0 ? (n + kChunk - 1) / kChunk : 1;
  const long long nblocks = (nchunks + 31) / 32;
  auto rnd = [](size_t b) { return (b + 255) & ~(size_t)255; };
  size_t bytes = 2 * rnd((size_t)nchunks * 4) + 2 * rnd((size_t)nblocks * 8);
  long long cnt[kMaxLevels];
  const int nlev = level_counts(nchunks, cnt);
  for (int L = 0; L < nlev; ++L) bytes += 2 * (2 * rnd((size_t)cnt[L] * 8) + rnd((size_t)cnt[L] * 4));
  return bytes;
}

cudaError_t launch_ordered_sums(const float* map, long long n, float scale, const uint32_t* maxbits, void* scratch,
                                double* out, cudaStream_t s, unsigned long long* launches) {
  if (n <= 0) return cudaMemsetAsync(out, 0, 2 * sizeof(double), s);
  const long long nchunks = (n + kChunk - 1) / kChunk;
  const long long nblocks = (nchunks + 31) / 32;
  char* p = static_cast<char*>(scratch);
  auto take = [&](size_t bytes) {
    char* r = p;
    p += (bytes + 255) & ~(size_t)255;
    return r;
  };
  float* cs = reinterpret_cast<float*>(take((size_t)nchunks * 4));
  float* cq = reinterpret_cast<float*>(take((size_t)nchunks * 4));
  unsigned long long* bs = reinterpret_cast<unsigned long long*>(take((size_t)nblocks * 8));
  unsigned long long* bq = reinterpret_cast<unsigned long long*>(take((size_t)nblocks * 8));
  Walk ws{}, wq{};
  long long cnt[kMaxLevels];
  const int nlev = level_counts(nchunks, cnt);
  for (int L = 0; L < nlev; ++L) {
    for (Walk* w : {&ws, &wq}) {
      w->lv[L].i0 = reinterpret_cast<unsigned long long*>(take((size_t)cnt[L] * 8));
      w->lv[L].i1 = reinterpret_cast<unsigned long long*>(take((size_t)cnt[L] * 8));
      w->lv[L].meta = reinterpret_cast<uint32_t*>(take((size_t)cnt[L] * 4));
      w->cnt[L] = cnt[L];
    }
  }
  ws.nlev = wq.nlev = nlev;
  const unsigned warps_per_cta = 8;
  const unsigned g1 = (unsigned)((nblocks + warps_per_cta - 1) / warps_per_cta);
  osum_chunk_kernel<<<g1, 32 * warps_per_cta, 0, s>>>(map, n, scale, nchunks, maxbits, cs, cq, bs, bq);
  osum_scan_kernel<<<1, 1024, 0, s>>>(bs, bq, nblocks);
  osum_fn_kernel<<<g1, 32 * warps_per_cta, 0, s>>>(map, n, scale, nchunks, maxbits, cs, cq, bs, bq, ws.lv[0],
                                                   wq.lv[0], ws.lv[1], wq.lv[1]);
  *launches += 3;
  for (int L = 2; L < nlev; ++L) {
    const unsigned g = (unsigned)((cnt[L] + warps_per_cta - 1) / warps_per_cta);
    osum_level_kernel<<<g, 32 * warps_per_cta, 0, s>>>(ws.lv[L - 1], wq.lv[L - 1], cnt[L - 1], ws.lv[L], wq.lv[L]);
    ++*launches;
  }
  const int Lc = cached_from(cnt, nlev);
  size_t wsmem = 0;
  for (int L = Lc; L < nlev; ++L) wsmem += ((size_t)cnt[L] * kEntryBytes + 15) & ~(size_t)15;
  cudaError_t e = cudaFuncSetAttribute(osum_walk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kWalkSmemBytes + 1024);
  if (e != cudaSuccess) return e;
  osum_walk_kernel<<<2, 32, wsmem, s>>>(map, n, scale, ws, wq, out);
  ++*launches;
  return cudaGetLastError();
}

}  // namespace bm
