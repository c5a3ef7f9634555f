// Exact sums of the statistics accumulator, rounded once to f64 (host code).
//
// The device accumulates, per f32 exponent e (value = m * 2^(e-150) with a
// 24-bit integer m), the integer sums of m and of m*m (split as hi*2^24 + lo).
// Values whose exponent lies within kFixedSpan of a known smallest exponent
// e_lo arrive instead as per-CTA sums of m * 2^(e - e_lo) and their squares.
// Here those integers are placed into a wide fixed-point integer and the total
// is rounded to the nearest f64 (ties to even).  The result is the correctly
// rounded exact sum, independent of the order in which the GPU added values.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#include "bm_internal.h"

namespace bm {

struct WideUInt {
  static constexpr int kLimbs = 12;  // 768 bits
  uint64_t limb[kLimbs];
  WideUInt() { std::memset(limb, 0, sizeof limb); }

  // += v * 2^shift
  void add_shifted(uint64_t v, int shift) {
    if (!v) return;
    int li = shift >> 6, sh = shift & 63;
    uint64_t lo = v << sh;
    uint64_t hi = sh ? (v >> (64 - sh)) : 0;
    add_at(li, lo);
    if (hi) add_at(li + 1, hi);
  }

  void add_at(int li, uint64_t v) {
    while (v && li < kLimbs) {
      const uint64_t old = limb[li];
      limb[li] = old + v;
      v = (limb[li] < old) ? 1 : 0;
      ++li;
    }
  }

  bool bit(int i) const { return (limb[i >> 6] >> (i & 63)) & 1u; }

  int top_bit() const {
    for (int li = kLimbs - 1; li >= 0; --li)
      if (limb[li]) return li * 64 + 63 - __builtin_clzll(limb[li]);
    return -1;
  }

  bool any_below(int i) const {  // any set bit at position < i
    if (i <= 0) return false;
    const int li = i >> 6, sh = i & 63;
    for (int k = 0; k < li; ++k)
      if (limb[k]) return true;
    return sh && (limb[li] & ((1ull << sh) - 1));
  }

  // value = this * 2^-lsb_exp, rounded to nearest f64, ties to even
  double to_double(int lsb_exp) const {
    const int p = top_bit();
    if (p < 0) return 0.0;
    uint64_t mant = 0;
    int e;
    if (p < 53) {
      for (int i = p; i >= 0; --i) mant = (mant << 1) | (uint64_t)bit(i);
      e = 0;
    } else {
      for (int i = p; i >= p - 52; --i) mant = (mant << 1) | (uint64_t)bit(i);
      e = p - 52;
      const bool round = bit(p - 53);
      const bool sticky = any_below(p - 53);
      if (round && (sticky || (mant & 1))) {
        ++mant;
        if (mant == (1ull << 53)) {
          mant >>= 1;
          ++e;
        }
      }
    }
    return std::ldexp((double)mant, e - lsb_exp);
  }
};

// Adds the per-CTA fixed-point partials into a's host-side totals.
inline void fold_fixed_partials(StatsAccum& a, const FixedPartial* p, unsigned n, int e_lo) {
  unsigned long long s1[2] = {a.fx_s1[0], a.fx_s1[1]};
  unsigned long long s2[3] = {a.fx_s2[0], a.fx_s2[1], a.fx_s2[2]};
  for (unsigned i = 0; i < n; ++i) {
    s1[0] += p[i].s1;
    s1[1] += (s1[0] < p[i].s1) ? 1u : 0u;
    const unsigned long long lo = s2[0] + p[i].s2lo;
    const unsigned long long c0 = lo < s2[0] ? 1u : 0u;
    s2[0] = lo;
    const unsigned long long mid = s2[1] + p[i].s2hi;
    const unsigned long long c1 = mid < s2[1] ? 1u : 0u;
    s2[1] = mid + c0;
    s2[2] += c1 + ((s2[1] < c0) ? 1u : 0u);
  }
  a.fx_s1[0] = s1[0];
  a.fx_s1[1] = s1[1];
  a.fx_s2[0] = s2[0];
  a.fx_s2[1] = s2[1];
  a.fx_s2[2] = s2[2];
  a.fx_elo = e_lo;
}

inline void exact_sums_to_double(const StatsAccum& a, double* sum, double* sum_sq) {
  WideUInt s, q;
  for (int e = 1; e < 256; ++e) {
    // sum: m * 2^(e-150), fixed point LSB 2^-149  -> shift e-1
    s.add_shifted(a.sum_m[e], e - 1);
    // squares: m^2 * 2^(2e-300), LSB 2^-298 -> shift 2e-2
    q.add_shifted(a.sq_lo[e], 2 * e - 2);
    q.add_shifted(a.sq_hi[e], 2 * e - 2 + 24);
  }
  if (a.fx_elo > 0) {
    // fixed point: units of 2^(e_lo - 150) for the sum, 2^(2 e_lo - 300) for squares
    const int e = a.fx_elo;
    s.add_shifted(a.fx_s1[0], e - 1);
    s.add_shifted(a.fx_s1[1], e - 1 + 64);
    q.add_shifted(a.fx_s2[0], 2 * e - 2);
    q.add_shifted(a.fx_s2[1], 2 * e - 2 + 64);
    q.add_shifted(a.fx_s2[2], 2 * e - 2 + 128);
  }
  *sum = s.to_double(149);
  *sum_sq = q.to_double(298);
}

}  // namespace bm
