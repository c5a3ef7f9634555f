// CPU oracle for the Tb.Th / Tb.Sp hot path of bone-morphometry v0.7.0-rc.3.
//
// TEST INFRASTRUCTURE ONLY.  The GPU library's results are compared against
// this file's, and bench.py times it as the CPU baseline.  It is
// never linked into, loaded by, or called from the product library
// (bone_morphometry_gb300/csrc), which has no CPU fallback.
//
// It restates, in plain C++ with OpenMP standing in for rayon, the reference's
// arithmetic step by step:
//   volume.rs:84-105            phase_inside
//   edt.rs:6, 57-156, 167-223   euclidean_distance_transform_squared, transform_1d
//   local_thickness.rs:16-358   local_thickness and its helpers
//   metrics.rs:204-298          nonzero_stats, linear_quantile_unstable
// The reference keeps f64 with INF = 1e30 inside the EDT, f32 in the surface
// cleanup and a sequential f64 accumulation in the statistics; so does this
// file.  It must be compiled with -ffp-contract=off: Rust never fuses a*b+c,
// and GCC on aarch64 would otherwise emit fmadd and change rounding.
//
// Pins: the reference's own known-answer tests (edt.rs:240-274,
// local_thickness.rs:364-401, metrics.rs:304-326, volume.rs:123-136) and an
// independent EDT (scipy.ndimage.distance_transform_edt) are checked against
// this file by tests/test_oracle.py.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kInf = 1.0e30;  // edt.rs:6

inline bool is_selected(int phase, uint8_t v) {  // edt.rs:19-24
  return phase == 0 ? v != 0 : v == 0;            // 0 = Foreground, 1 = Background
}

inline double intersection(const double* f, size_t p, size_t q, double qf) {  // edt.rs:220-223
  double pf = static_cast<double>(p);
  return ((f[q] + qf * qf) - (f[p] + pf * pf)) / (2.0 * (qf - pf));
}

// Felzenszwalb-Huttenlocher lower envelope, edt.rs:168-217.  v has n slots,
// z has n + 1 slots.
void transform_1d(const double* f, double* d, size_t n, size_t* v, double* z) {
  size_t k = 0;
  v[0] = 0;
  z[0] = -std::numeric_limits<double>::infinity();
  z[1] = std::numeric_limits<double>::infinity();
  for (size_t q = 1; q < n; ++q) {
    double qf = static_cast<double>(q);
    size_t p = v[k];
    double s = intersection(f, p, q, qf);
    while (s <= z[k]) {
      if (k == 0) break;
      k -= 1;
      p = v[k];
      s = intersection(f, p, q, qf);
    }
    if (k == 0 && s <= z[0]) {
      v[0] = q;
      z[0] = -std::numeric_limits<double>::infinity();
      z[1] = std::numeric_limits<double>::infinity();
    } else {
      k += 1;
      v[k] = q;
      z[k] = s;
      z[k + 1] = std::numeric_limits<double>::infinity();
    }
  }
  size_t env = 0;
  for (size_t q = 0; q < n; ++q) {
    double qf = static_cast<double>(q);
    while (z[env + 1] < qf) env += 1;
    size_t p = v[env];
    double delta = qf - static_cast<double>(p);
    d[q] = delta * delta + f[p];
  }
}

struct Scratch {  // edt.rs:34-49
  std::vector<double> in, out, z;
  std::vector<size_t> v;
  void resize(size_t n) {
    in.resize(n);
    out.resize(n);
    v.resize(n);
    z.resize(n + 1);
  }
};

inline size_t index3(size_t x, size_t y, size_t z, size_t w, size_t h) {  // local_thickness.rs:334-336
  return (z * h + y) * w + x;
}

// NEIGHBORS_26 in the visitation order of Fiji's Clean_Up_Local_Thickness,
// local_thickness.rs:285-312.  The order fixes the f32 summation order.
const int kN26[26][3] = {
    {0, 0, -1}, {0, 0, 1},  {0, -1, 0}, {0, 1, 0},   {-1, 0, 0},  {1, 0, 0},  {0, 1, -1},
    {0, 1, 1},  {1, -1, 0}, {1, 1, 0},  {-1, 0, 1},  {1, 0, 1},   {0, -1, -1}, {0, -1, 1},
    {-1, -1, 0}, {-1, 1, 0}, {-1, 0, -1}, {1, 0, -1}, {1, 1, 1},   {1, -1, 1}, {-1, 1, 1},
    {-1, -1, 1}, {1, 1, -1}, {1, -1, -1}, {-1, 1, -1}, {-1, -1, -1}};

inline float look(const float* vals, long x, long y, long z, size_t w, size_t h, size_t d) {  // :316-331
  if (x < 0 || y < 0 || z < 0 || x >= (long)w || y >= (long)h || z >= (long)d) return -1.0f;
  return vals[index3((size_t)x, (size_t)y, (size_t)z, w, h)];
}

inline uint32_t integer_sqrt(uint32_t value) {  // local_thickness.rs:339-348
  uint32_t root = static_cast<uint32_t>(std::sqrt(static_cast<double>(value)));
  while ((uint64_t)(root + 1) * (uint64_t)(root + 1) <= (uint64_t)value) root += 1;
  while ((uint64_t)root * (uint64_t)root > (uint64_t)value) root -= 1;
  return root;
}

inline uint32_t ceiling_sqrt(uint32_t value) {  // local_thickness.rs:351-358
  uint32_t f = integer_sqrt(value);
  return f * f == value ? f : f + 1;
}

uint32_t scan_cube_one(uint32_t dx, uint32_t dy, uint32_t dz, uint32_t r2) {  // :76-102
  uint32_t radius = integer_sqrt(r2) + 1;
  uint32_t best = 0;
  for (uint32_t k = 0; k <= radius; ++k) {
    uint32_t scan_k = k * k;
    uint32_t dk = (k + dz) * (k + dz);
    for (uint32_t j = 0; j <= radius; ++j) {
      uint32_t scan_kj = scan_k + j * j;
      if (scan_kj > r2) continue;
      uint32_t ip = integer_sqrt(r2 - scan_kj) + dx;
      uint32_t cand = dk + (j + dy) * (j + dy) + ip * ip;
      best = std::max(best, cand);
    }
  }
  return best;
}

}  // namespace

extern "C" {

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// volume.rs:84-105: u8(roi != 0 && ((bone != 0) == select_bone)).
void orc_phase_inside(const uint8_t* bone, const uint8_t* roi, size_t n, int select_bone,
                      uint8_t* out) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)n; ++i)
    out[i] = (uint8_t)(roi[i] != 0 && ((bone[i] != 0) == (select_bone != 0)));
}

// edt.rs:57-156.  Returns 0, or 1 when every voxel is selected (edt.rs:61-66).
int orc_edt_sq(const uint8_t* vol, size_t w, size_t h, size_t d, int phase, uint32_t* out) {
  const size_t n = w * h * d;
  const size_t sl = w * h;
  bool all = true;
  for (size_t i = 0; i < n; ++i)
    if (!is_selected(phase, vol[i])) {
      all = false;
      break;
    }
  if (all) return 1;

  std::vector<double> data(n);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)n; ++i) data[i] = is_selected(phase, vol[i]) ? kInf : 0.0;

  // X pass: rows are contiguous (edt.rs:80-90).
#pragma omp parallel
  {
    Scratch s;
    s.resize(w);
#pragma omp for schedule(static)
    for (long r = 0; r < (long)(h * d); ++r) {
      double* row = &data[(size_t)r * w];
      std::memcpy(s.in.data(), row, w * sizeof(double));
      transform_1d(s.in.data(), row, w, s.v.data(), s.z.data());
    }
  }
  // Y pass: one z-slice per task, columns serial inside (edt.rs:93-113).
#pragma omp parallel
  {
    Scratch s;
    s.resize(h);
#pragma omp for schedule(static)
    for (long zz = 0; zz < (long)d; ++zz) {
      double* slice = &data[(size_t)zz * sl];
      for (size_t x = 0; x < w; ++x) {
        for (size_t y = 0; y < h; ++y) s.in[y] = slice[y * w + x];
        transform_1d(s.in.data(), s.out.data(), h, s.v.data(), s.z.data());
        for (size_t y = 0; y < h; ++y) slice[y * w + x] = s.out[y];
      }
    }
  }
  // Z pass into a transposed line buffer (edt.rs:116-133).
  std::vector<double> zl(n);
#pragma omp parallel
  {
    Scratch s;
    s.resize(d);
#pragma omp for schedule(static)
    for (long line = 0; line < (long)sl; ++line) {
      for (size_t zz = 0; zz < d; ++zz) s.in[zz] = data[zz * sl + (size_t)line];
      transform_1d(s.in.data(), &zl[(size_t)line * d], d, s.v.data(), s.z.data());
    }
  }
  // Transpose back; round() only on selected voxels (edt.rs:139-153).
#pragma omp parallel for schedule(static)
  for (long zz = 0; zz < (long)d; ++zz) {
    for (size_t line = 0; line < sl; ++line) {
      size_t idx = (size_t)zz * sl + line;
      uint32_t v = 0;
      if (is_selected(phase, vol[idx])) v = (uint32_t)std::round(zl[line * d + (size_t)zz]);
      out[idx] = v;
    }
  }
  return 0;
}

// create_templates / scan_cube (local_thickness.rs:67-102) for a list of r^2.
void orc_create_templates(const uint32_t* values, size_t count, uint32_t* t0, uint32_t* t1,
                          uint32_t* t2) {
#pragma omp parallel for schedule(dynamic, 16)
  for (long i = 0; i < (long)count; ++i) {
    t0[i] = scan_cube_one(1, 0, 0, values[i]);
    t1[i] = scan_cube_one(1, 1, 0, values[i]);
    t2[i] = scan_cube_one(1, 1, 1, values[i]);
  }
}

uint32_t orc_integer_sqrt(uint32_t v) { return integer_sqrt(v); }
uint32_t orc_ceiling_sqrt(uint32_t v) { return ceiling_sqrt(v); }

// distance_index (local_thickness.rs:46-65) + create_templates + distance_ridges
// (:104-167).  Writes ridge records (linear index, r^2) in ascending index
// order, the order the reference's par_iter().filter_map().collect() keeps.
// Returns the ridge count; ridge_idx / ridge_r2 may be null to only count.
// The caller sizes the ridge arrays with cap entries; entries beyond cap are
// counted but not written.
size_t orc_distance_ridges(const uint8_t* vol, size_t w, size_t h, size_t d, int phase,
                           const uint32_t* sq, uint64_t* ridge_idx, uint32_t* ridge_r2,
                           size_t cap) {
  const size_t n = w * h * d;
  const size_t sl = w * h;
  uint32_t maximum = 0;
  for (size_t i = 0; i < n; ++i) maximum = std::max(maximum, sq[i]);
  std::vector<uint8_t> occurs((size_t)maximum + 1, 0);
  for (size_t i = 0; i < n; ++i) occurs[sq[i]] = 1;
  std::vector<uint32_t> values;
  for (size_t v = 0; v <= maximum; ++v)
    if (occurs[v]) values.push_back((uint32_t)v);
  std::vector<size_t> rank((size_t)maximum + 1, SIZE_MAX);
  for (size_t i = 0; i < values.size(); ++i) rank[values[i]] = i;
  std::vector<uint32_t> t[3];
  for (auto& tt : t) tt.resize(values.size());
  orc_create_templates(values.data(), values.size(), t[0].data(), t[1].data(), t[2].data());

  // Ridge flags in parallel, then an in-order compaction.
  std::vector<uint8_t> flag(n, 0);
#pragma omp parallel for schedule(static)
  for (long ii = 0; ii < (long)n; ++ii) {
    size_t index = (size_t)ii;
    if (!is_selected(phase, vol[index])) continue;
    uint32_t r2 = sq[index];
    if (r2 == 0) continue;
    size_t z = index / sl;
    size_t rem = index - z * sl;
    size_t y = rem / w;
    size_t x = rem - y * w;
    size_t ri = rank[r2];
    bool ridge = true;
    for (long dz = -1; dz <= 1 && ridge; ++dz) {
      long nz = (long)z + dz;
      if (nz < 0 || nz >= (long)d) continue;
      for (long dy = -1; dy <= 1 && ridge; ++dy) {
        long ny = (long)y + dy;
        if (ny < 0 || ny >= (long)h) continue;
        for (long dx = -1; dx <= 1; ++dx) {
          if (dx == 0 && dy == 0 && dz == 0) continue;
          long nx = (long)x + dx;
          if (nx < 0 || nx >= (long)w) continue;
          int comps = (dx != 0) + (dy != 0) + (dz != 0);
          size_t nb = index3((size_t)nx, (size_t)ny, (size_t)nz, w, h);
          if (sq[nb] >= t[comps - 1][ri]) {
            ridge = false;
            break;
          }
        }
      }
    }
    flag[index] = ridge ? 1 : 0;
  }
  size_t count = 0;
  for (size_t i = 0; i < n; ++i) {
    if (!flag[i]) continue;
    if (count < cap) {
      if (ridge_idx) ridge_idx[count] = i;
      if (ridge_r2) ridge_r2[count] = sq[i];
    }
    ++count;
  }
  return count;
}

// propagate_ridges (local_thickness.rs:169-202) on a zeroed u32 map; relaxed
// atomic max exactly as fetch_max(Relaxed).
void orc_propagate(size_t w, size_t h, size_t d, const uint64_t* ridge_idx, const uint32_t* ridge_r2,
                   size_t count, uint32_t* out) {
  const size_t n = w * h * d;
  const size_t sl = w * h;
  std::memset(out, 0, n * sizeof(uint32_t));
#pragma omp parallel for schedule(dynamic, 64)
  for (long i = 0; i < (long)count; ++i) {
    size_t index = (size_t)ridge_idx[i];
    uint32_t r2 = ridge_r2[i];
    size_t z = index / sl;
    size_t rem = index - z * sl;
    size_t y = rem / w;
    size_t x = rem - y * w;
    size_t radius = ceiling_sqrt(r2);
    size_t xs = x >= radius ? x - radius : 0, ys = y >= radius ? y - radius : 0,
           zs = z >= radius ? z - radius : 0;
    size_t xe = std::min(x + radius, w - 1), ye = std::min(y + radius, h - 1),
           ze = std::min(z + radius, d - 1);
    uint64_t r2u = r2;
    for (size_t nz = zs; nz <= ze; ++nz) {
      uint64_t dzz = (uint64_t)(nz > z ? nz - z : z - nz);
      uint64_t dz2 = dzz * dzz;
      for (size_t ny = ys; ny <= ye; ++ny) {
        uint64_t dyy = (uint64_t)(ny > y ? ny - y : y - ny);
        uint64_t dyz2 = dz2 + dyy * dyy;
        if (dyz2 > r2u) continue;
        for (size_t nx = xs; nx <= xe; ++nx) {
          uint64_t dxx = (uint64_t)(nx > x ? nx - x : x - nx);
          if (dyz2 + dxx * dxx <= r2u) {
            uint32_t* p = &out[index3(nx, ny, nz, w, h)];
            uint32_t cur = __atomic_load_n(p, __ATOMIC_RELAXED);
            while (cur < r2 &&
                   !__atomic_compare_exchange_n(p, &cur, r2, true, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
            }
          }
        }
      }
    }
  }
}

// propagated u32 r^2 -> f32 diameter: (2.0_f64 * sqrt(r2 as f64)) as f32
// (local_thickness.rs:204-207).
void orc_r2_to_diameter(const uint32_t* r2, size_t n, float* out) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)n; ++i) out[i] = (float)(2.0 * std::sqrt((double)r2[i]));
}

// clean_up_surface_jaggies (local_thickness.rs:211-281), serial as in the
// reference, followed by the final abs pass.
void orc_cleanup(const float* input, size_t w, size_t h, size_t d, float* output) {
  const size_t n = w * h * d;
  for (size_t i = 0; i < n; ++i) output[i] = 0.0f;
  for (size_t z = 0; z < d; ++z)
    for (size_t y = 0; y < h; ++y)
      for (size_t x = 0; x < w; ++x) {
        size_t index = index3(x, y, z, w, h);
        float value = input[index];
        if (value == 0.0f) continue;
        bool border = false;
        for (int k = 0; k < 26; ++k) {
          if (look(input, (long)x + kN26[k][0], (long)y + kN26[k][1], (long)z + kN26[k][2], w, h, d) ==
              0.0f) {
            border = true;
            break;
          }
        }
        output[index] = border ? -1.0f : value;
      }
  for (size_t z = 0; z < d; ++z)
    for (size_t y = 0; y < h; ++y)
      for (size_t x = 0; x < w; ++x) {
        size_t index = index3(x, y, z, w, h);
        if (output[index] != -1.0f) continue;
        size_t count = 0;
        float sum = 0.0f;
        for (int k = 0; k < 26; ++k) {
          float v = look(output, (long)x + kN26[k][0], (long)y + kN26[k][1], (long)z + kN26[k][2], w, h, d);
          if (v > 0.0f) {
            count += 1;
            sum += v;
          }
        }
        float corrected = count > 0 ? sum / (float)count : input[index];
        output[index] = -corrected;
      }
  for (size_t i = 0; i < n; ++i) output[i] = std::fabs(output[i]);
}

// local_thickness (local_thickness.rs:16-44).  Optional intermediates:
// edt_out (u32 squared EDT), prop_out (u32 propagated r^2 map, unmasked),
// n_ridges_out.  Returns 0, or 1 for an all-selected volume.
int orc_local_thickness(const uint8_t* vol, size_t w, size_t h, size_t d, int phase, float* out,
                        uint32_t* edt_out, uint32_t* prop_out, size_t* n_ridges_out) {
  const size_t n = w * h * d;
  std::vector<uint32_t> sq(n);
  int rc = orc_edt_sq(vol, w, h, d, phase, sq.data());
  if (rc) return rc;
  size_t nr = orc_distance_ridges(vol, w, h, d, phase, sq.data(), nullptr, nullptr, 0);
  std::vector<uint64_t> ri(nr);
  std::vector<uint32_t> rr(nr);
  orc_distance_ridges(vol, w, h, d, phase, sq.data(), ri.data(), rr.data(), nr);
  std::vector<uint32_t> prop(n);
  orc_propagate(w, h, d, ri.data(), rr.data(), nr, prop.data());
  std::vector<float> dia(n);
  orc_r2_to_diameter(prop.data(), n, dia.data());
  orc_cleanup(dia.data(), w, h, d, out);
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)n; ++i)
    if (!is_selected(phase, vol[i])) out[i] = 0.0f;
  if (edt_out) std::memcpy(edt_out, sq.data(), n * sizeof(uint32_t));
  if (prop_out) std::memcpy(prop_out, prop.data(), n * sizeof(uint32_t));
  if (n_ridges_out) *n_ridges_out = nr;
  return 0;
}

// nonzero_stats mean / SD / max (metrics.rs:204-241), sequential f64 in index
// order.  out = {count, mean, sd, max, sum, sum_of_squares}.  Returns 1 when
// no value is finite and positive (metrics.rs:228-230).
int orc_nonzero_stats(const float* values, size_t n, double scale, double* out) {
  uint64_t count = 0;
  double sum = 0.0, ss = 0.0, mx = 0.0;
  const float sf = (float)scale;
  for (size_t i = 0; i < n; ++i) {
    float raw = values[i];
    if (!std::isfinite(raw) || raw <= 0.0f) continue;
    double v = (double)(raw * sf);
    count += 1;
    sum += v;
    ss += v * v;
    mx = std::max(mx, v);
  }
  if (count == 0) return 1;
  double c = (double)count;
  double mean = sum / c;
  double centered = (c * ss - sum * sum) / c;
  double sd = (count > 1 && centered > 0.0) ? std::sqrt(centered / (c - 1.0)) : 0.0;
  out[0] = c;
  out[1] = mean;
  out[2] = sd;
  out[3] = mx;
  out[4] = sum;
  out[5] = ss;
  return 0;
}

// Exact moment sums of v = f32(raw * f32(scale)) over the finite positive raw
// values (the terms nonzero_stats adds, metrics.rs:215-226), kept per f32
// exponent so that no rounding happens: v = m * 2^(e - 150) with an integer
// m < 2^24, so v*v = m*m * 2^(2e - 300).  s1[e] = sum of m (u64: < 2^24 *
// 2^38 terms), s2[2e], s2[2e+1] = low and high 64 bits of the 128-bit sum of
// m*m.  Returns the count of values; max_out = the largest v.  The caller
// combines the bins with exact integer arithmetic.  Not a reference function:
// a checker of the GPU's exactly rounded sums.
uint64_t orc_exact_moment_sums(const float* values, size_t n, double scale, uint64_t* s1, uint64_t* s2,
                               double* max_out) {
  const float sf = (float)scale;
  uint64_t count = 0;
  float mx = 0.0f;
  for (int e = 0; e < 256; ++e) {
    s1[e] = 0;
    s2[2 * e] = s2[2 * e + 1] = 0;
  }
#pragma omp parallel
  {
    uint64_t a1[256] = {};
    unsigned __int128 a2[256] = {};
    uint64_t c = 0;
    float m = 0.0f;
#pragma omp for schedule(static) nowait
    for (long i = 0; i < (long)n; ++i) {
      const float raw = values[i];
      if (!std::isfinite(raw) || raw <= 0.0f) continue;
      const float v = raw * sf;
      uint32_t bits;
      std::memcpy(&bits, &v, 4);
      uint32_t e = (bits >> 23) & 0xFFu;
      uint64_t mant = bits & 0x7FFFFFu;
      if (e) mant |= 1u << 23;
      else e = 1;
      a1[e] += mant;
      a2[e] += (unsigned __int128)(mant * mant);
      ++c;
      m = std::max(m, v);
    }
#pragma omp critical
    {
      for (int e = 0; e < 256; ++e) {
        s1[e] += a1[e];
        unsigned __int128 t = ((unsigned __int128)s2[2 * e + 1] << 64) | s2[2 * e];
        t += a2[e];
        s2[2 * e] = (uint64_t)t;
        s2[2 * e + 1] = (uint64_t)(t >> 64);
      }
      count += c;
      mx = std::max(mx, m);
    }
  }
  *max_out = (double)mx;
  return count;
}

// linear_quantile_unstable over the finite positive values (metrics.rs:242-298).
// quantiles[i] in [0, 1]; out[i] = ((lower + frac*(upper-lower)) as f32 * scale_f32) as f64.
int orc_quantiles(const float* values, size_t n, double scale, const double* quantiles, size_t nq,
                  double* out) {
  std::vector<float> kept;
  kept.reserve(n / 4);
  for (size_t i = 0; i < n; ++i)
    if (std::isfinite(values[i]) && values[i] > 0.0f) kept.push_back(values[i]);
  if (kept.empty()) return 1;
  const float sf = (float)scale;
  for (size_t i = 0; i < nq; ++i) {
    double position = quantiles[i] * (double)(kept.size() - 1);
    size_t lower = (size_t)std::floor(position);
    size_t upper = (size_t)std::ceil(position);
    double fraction = position - (double)lower;
    std::nth_element(kept.begin(), kept.begin() + (long)lower, kept.end());
    double lv = (double)kept[lower];
    double uv = lv;
    if (upper != lower) {
      std::nth_element(kept.begin(), kept.begin() + (long)upper, kept.end());
      uv = (double)kept[upper];
    }
    double qv = lv + fraction * (uv - lv);
    out[i] = (double)((float)qv * sf);
  }
  return 0;
}

}  // extern "C"
