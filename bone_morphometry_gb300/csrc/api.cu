// C ABI of libbm_gb300 (include/bm.h): context, buffer cache, the per-phase
// pipeline and the drop-in entry points for edt.rs / local_thickness.rs /
// metrics.rs.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "exact_sum.h"
#include "kernels.h"

using namespace bm;

namespace {

thread_local std::string g_create_error;

struct CallError {
  int status;
};

void set_err(bm_ctx* ctx, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (ctx) ctx->last_error = buf;
  else g_create_error = buf;
}

[[noreturn]] void fail(bm_ctx* ctx, int status, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  ctx->last_error = buf;
  throw CallError{status};
}

void check(bm_ctx* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return;
  const int st = (e == cudaErrorMemoryAllocation) ? BM_ERR_OOM : BM_ERR_CUDA;
  cudaGetLastError();  // clear a sticky-free error so the context stays usable
  fail(ctx, st, "%s: %s", what, cudaGetErrorString(e));
}

void* ensure(bm_ctx* ctx, Buffer& b, size_t bytes, const char* what) {
  if (bytes == 0) bytes = 16;
  if (b.bytes >= bytes) return b.ptr;
  if (b.ptr) {
    cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
  }
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    fail(ctx, BM_ERR_OOM, "device allocation of %zu bytes for %s failed: %s", bytes, what, cudaGetErrorString(e));
  }
  b.ptr = p;
  b.bytes = bytes;
  return p;
}

void release(Buffer& b) {
  if (b.ptr) cudaFree(b.ptr);
  b.ptr = nullptr;
  b.bytes = 0;
}

const char* const kFamilyName[KF_COUNT] = {"count_roi", "edt_x",     "edt_y",           "edt_z",
                                            "templates", "ridge",     "fill",            "fill_rank",
                                            "fill_bin",  "fill_sites",      "cleanup_final",
                                            "quantile",  "stats_order"};

cudaEvent_t pooled_event(bm_ctx* ctx) {
  if (!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  check(ctx, cudaEventCreate(&e), "event create");
  return e;
}

// Launch through `launch` (a callable returning cudaError_t); while profiling,
// bracket it with events on the launching stream.
template <class L>
void timed(bm_ctx* ctx, int family, cudaStream_t s, const char* what, L&& launch) {
  if (!ctx->profiling) {
    check(ctx, launch(), what);
    return;
  }
  cudaEvent_t a = pooled_event(ctx), b = pooled_event(ctx);
  check(ctx, cudaEventRecord(a, s), "event record");
  check(ctx, launch(), what);
  check(ctx, cudaEventRecord(b, s), "event record");
  ctx->prof.push_back(ProfRec{family, a, b});
}

void fold_profile(bm_ctx* ctx) {
  for (const ProfRec& r : ctx->prof) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.stop) == cudaSuccess && cudaEventElapsedTime(&ms, r.start, r.stop) == cudaSuccess) {
      ctx->prof_ms[r.family] += ms;
      ctx->prof_n[r.family] += 1;
    }
    cudaGetLastError();
    ctx->event_pool.push_back(r.start);
    ctx->event_pool.push_back(r.stop);
  }
  ctx->prof.clear();
}

// volume.rs:12-34 plus the library's own limits (u32 linear ridge index, u32
// squared distances whose search templates cannot overflow u32).
Dims check_dims(bm_ctx* ctx, size_t w, size_t h, size_t d) {
  if (w < 2 || h < 2 || d < 2)
    fail(ctx, BM_ERR_DIMS, "all dimensions must be at least 2 for 3-D morphometry; got %zux%zux%zu", w, h, d);
  if (w > 32768 || h > 32768 || d > 32768)
    fail(ctx, BM_ERR_DIMS, "dimension above 32768 is not supported; got %zux%zux%zu", w, h, d);
  const unsigned long long n = (unsigned long long)w * h * d;
  if (n >= 0xFFFFFFFFull)
    fail(ctx, BM_ERR_DIMS, "volume of %llu voxels exceeds the 2^32-1 voxel limit", n);
  const unsigned long long r2 =
      (unsigned long long)(w - 1) * (w - 1) + (unsigned long long)(h - 1) * (h - 1) +
      (unsigned long long)(d - 1) * (d - 1);
  if (r2 >= (1ull << 30)) fail(ctx, BM_ERR_DIMS, "largest squared distance %llu exceeds 2^30", r2);
  return Dims{(int)w, (int)h, (int)d};
}

const char* phase_name(int phase) { return phase == BM_PHASE_BACKGROUND ? "background" : "foreground"; }

void ensure_lut(bm_ctx* ctx, uint32_t rmax) {
  if (ctx->lut_max >= rmax && ctx->lut.ptr) return;
  // grow to at least twice the current size so repeated growth stays amortised
  uint32_t target = rmax;
  if (ctx->lut.ptr && target < ctx->lut_max * 2u) target = ctx->lut_max * 2u;
  if (target < 1024) target = 1024;
  const size_t bytes = ((size_t)target + 1) * sizeof(uint4);
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    fail(ctx, BM_ERR_OOM, "device allocation of %zu bytes for the template table failed", bytes);
  }
  uint32_t lo = 0;
  if (ctx->lut.ptr) {
    check(ctx, cudaMemcpyAsync(p, ctx->lut.ptr, ((size_t)ctx->lut_max + 1) * sizeof(uint4), cudaMemcpyDeviceToDevice,
                               ctx->stream),
          "template table copy");
    lo = ctx->lut_max + 1;
  }
  timed(ctx, KF_TEMPLATES, ctx->stream, "template kernel",
        [&] { return launch_lut(static_cast<uint4*>(p), lo, target, ctx->stream, &ctx->launches); });
  check(ctx, cudaStreamSynchronize(ctx->stream), "template kernel");
  release(ctx->lut);
  ctx->lut.ptr = p;
  ctx->lut.bytes = bytes;
  ctx->lut_max = target;
  float* dia = static_cast<float*>(ensure(ctx, ctx->lutf, ((size_t)target + 1) * sizeof(float), "diameter table"));
  check(ctx, launch_dia_table(static_cast<const uint4*>(p), target + 1, dia, ctx->stream, &ctx->launches),
        "diameter table");
}

void ensure_surf(bm_ctx* ctx, uint32_t rmax);

// Sphere fill of one phase into F (u32 r^2 map): tile-owned fill, or the
// per-ball atomic scatter when the (ball, tile) entry count would not fit u32.
// f, g, m: the x, y and z pass outputs (kept for the chain passes); ridgebits:
// the ridge bitmask; m is free for reuse once the chain_z pass has read it.
// Returns the map the fill wrote: F, or m's buffer when F is g's (g is still
// needed by the chain_y pass that follows the fill).
uint32_t* fill_phase(bm_ctx* ctx, Dims dm, const uint2* ridges, Counters* ctr, unsigned long long max_ridges,
                     uint32_t rmax, const uint32_t* occ, const uint32_t* selbits, const uint32_t* f,
                     const uint32_t* g, uint32_t* m, const uint32_t* ridgebits, uint32_t* F, cudaStream_t s) {
  const size_t rwords = (size_t)rmax + 2;
  uint32_t* rank = static_cast<uint32_t*>(ensure(ctx, ctx->rank, rwords * 4, "r2 ranks"));
  uint32_t* rvals = static_cast<uint32_t*>(ensure(ctx, ctx->rvals, rwords * 4, "r2 values"));
  uint4* rgeo = static_cast<uint4*>(ensure(ctx, ctx->rgeo, rwords * sizeof(uint4), "r2 geometry"));
  FillInfo* info = static_cast<FillInfo*>(ensure(ctx, ctx->fillinfo, sizeof(FillInfo), "fill info"));
  uint32_t* scratch = static_cast<uint32_t*>(ensure(ctx, ctx->scanscratch, scan_scratch_words((long long)rwords) * 4,
                                                    "scan scratch"));
  check(ctx, cudaMemsetAsync(info, 0, sizeof(FillInfo), s), "memset");
  timed(ctx, KF_FILL_RANK, s, "rank kernel",
        [&] { return launch_rank(occ, rank, rmax, rvals, rgeo, info, scratch, s, &ctx->launches); });
  FillInfo hi;
  check(ctx, cudaMemcpyAsync(&hi, info, sizeof hi, cudaMemcpyDeviceToHost, s), "fill info readback");
  check(ctx, cudaStreamSynchronize(s), "rank kernel");
  const int ty = fill_tile_rows(dm, ctx->fill_rows);
  const long long tiles = fill_tile_count(dm, ty);
  const long long nbins = tiles * (long long)hi.nR;
  uint32_t* counts = static_cast<uint32_t*>(ensure(ctx, ctx->bincounts, ((size_t)nbins + 1) * 4, "bin counts"));
  uint32_t* offsets = static_cast<uint32_t*>(ensure(ctx, ctx->binoffsets, ((size_t)nbins + 1) * 4, "bin offsets"));
  scratch = static_cast<uint32_t*>(ensure(ctx, ctx->scanscratch, scan_scratch_words(nbins + 1) * 4, "scan scratch"));
  check(ctx, cudaMemsetAsync(counts, 0, ((size_t)nbins + 1) * 4, s), "memset");
  if (hi.nR > 0) {
    timed(ctx, KF_FILL_BIN, s, "bin count kernel", [&] {
      return launch_bin(true, ridges, ctr, max_ridges, rank, info, dm, ty, counts, nullptr, nullptr, s,
                        &ctx->launches);
    });
  }
  timed(ctx, KF_FILL_BIN, s, "bin scan",
        [&] { return launch_scan(counts, offsets, nbins + 1, scratch, s, &ctx->launches); });
  check(ctx, cudaMemcpyAsync(&hi, info, sizeof hi, cudaMemcpyDeviceToHost, s), "fill info readback");
  check(ctx, cudaStreamSynchronize(s), "bin kernels");
  if (hi.total_entries >= 0xFFFFFFFFull || rmax > kSurfMaxR2 || hi.nR >= 0xFFFFu) {
    check(ctx, cudaMemsetAsync(F, 0, (size_t)dm.n() * 4, s), "memset");
    timed(ctx, KF_FILL, s, "fill kernel",
          [&] { return launch_fill(ridges, ctr, max_ridges, dm, F, s, &ctx->launches); });
    return F;
  }
  uint32_t* entries = static_cast<uint32_t*>(
      ensure(ctx, ctx->binentries, ((size_t)hi.total_entries + 1) * 4, "bin entries"));
  if (hi.nR > 0) {
    timed(ctx, KF_FILL_BIN, s, "bin scatter kernel", [&] {
      return launch_bin(false, ridges, ctr, max_ridges, rank, info, dm, ty, counts, offsets, entries, s,
                        &ctx->launches);
    });
  }
  // Sites: the site kernel's half-warp steps over the ridge spheres' lattice
  // points (35-55 ps each, measured), or the two chain passes (9-17 ps a
  // voxel, bounded halo): chains above 0.2 steps per voxel.  The 512^3
  // workload's phases sit at 0.07 (bone) and 0.62 (marrow), the 1024^3
  // plate generator's at 0.10 and 0.28.
  const int halo = (int)std::sqrt((double)rmax) + 1;
  const bool chains_fit = f && g && m && ridgebits && rmax < (uint32_t)kChainMaxR2;
  const bool auto_chains = (double)hi.site_steps > 0.2 * (double)dm.n();
  const bool chains = chains_fit && (ctx->site_method == BM_SITES_CHAINS ||
                                     (ctx->site_method == BM_SITES_AUTO && auto_chains));
  uint32_t* chain = nullptr;
  if (chains) {
    const size_t nbytes = (size_t)dm.n() * 4;
    chain = static_cast<uint32_t*>(ensure(ctx, ctx->chainmap, nbytes, "chain map"));
    check(ctx, cudaMemsetAsync(chain, 0, nbytes, s), "memset");
    timed(ctx, KF_FILL_SITES, s, "chain z pass",
          [&] { return launch_chain_z(g, m, ridgebits, chain, dm, halo, s, &ctx->launches); });
    if (F == g) F = m;  // the z pass output has been read; g must outlive the fill
  } else {
    ensure_surf(ctx, rmax);
  }
  uint32_t* order = static_cast<uint32_t*>(ensure(ctx, ctx->tileorder, tile_order_words(dm, ty) * 4, "tile order"));
  timed(ctx, KF_FILL, s, "tile fill kernel", [&] {
    return launch_tile_fill(entries, offsets, rvals, rgeo, info, selbits, dm, ty, order, F, s, &ctx->launches);
  });
  if (chains) {
    timed(ctx, KF_FILL_SITES, s, "chain y pass",
          [&] { return launch_chain_y(f, g, chain, selbits, F, dm, halo, s, &ctx->launches); });
  } else {
    // 8 lanes per ridge when the spheres average at most 2.5 half-warp steps
    // (about 40 lattice points): half-warps would idle on their last step
    const bool small_spheres = 2 * hi.site_steps <= 5 * hi.ridges;
    timed(ctx, KF_FILL_SITES, s, "site kernel", [&] {
      return launch_sites(ridges, ctr, max_ridges, selbits, static_cast<const uint32_t*>(ctx->surf_off.ptr),
                          static_cast<const uint32_t*>(ctx->surf_pts.ptr), small_spheres, dm, F, s,
                          &ctx->launches);
    });
  }
  return F;
}

// Lattice points of every sphere |d|^2 = r2 for r2 <= rmax, cached per context.
void ensure_surf(bm_ctx* ctx, uint32_t rmax) {
  if (ctx->surf_off.ptr && ctx->surf_max >= rmax) return;
  uint32_t target = rmax < 1024 ? 1024 : rmax;
  if (target > kSurfMaxR2) target = kSurfMaxR2 > rmax ? kSurfMaxR2 : rmax;
  cudaStream_t s = ctx->stream;
  const long long n = (long long)target + 2;
  Buffer cnt;
  uint32_t* c = static_cast<uint32_t*>(ensure(ctx, cnt, (size_t)n * 4, "sphere table"));
  try {
    release(ctx->surf_off);
    release(ctx->surf_pts);
    ctx->surf_max = 0;
    uint32_t* off = static_cast<uint32_t*>(ensure(ctx, ctx->surf_off, (size_t)n * 4, "sphere table"));
    uint32_t* scratch = static_cast<uint32_t*>(ensure(ctx, ctx->scanscratch, scan_scratch_words(n) * 4, "scan"));
    check(ctx, cudaMemsetAsync(c, 0, (size_t)n * 4, s), "memset");
    check(ctx, launch_surf(true, 0, target, c, nullptr, nullptr, s, &ctx->launches), "sphere table");
    check(ctx, launch_scan(c, off, n, scratch, s, &ctx->launches), "sphere table");
    uint32_t total = 0;
    check(ctx, cudaMemcpyAsync(&total, off + target + 1, 4, cudaMemcpyDeviceToHost, s), "sphere table");
    check(ctx, cudaStreamSynchronize(s), "sphere table");
    uint32_t* pts = static_cast<uint32_t*>(ensure(ctx, ctx->surf_pts, ((size_t)total + 1) * 4, "sphere table"));
    check(ctx, launch_surf(false, 0, target, nullptr, off, pts, s, &ctx->launches), "sphere table");
    check(ctx, cudaStreamSynchronize(s), "sphere table");
  } catch (...) {
    release(cnt);
    release(ctx->surf_off);
    release(ctx->surf_pts);
    throw;
  }
  release(cnt);
  ctx->surf_max = target;
}

struct PhaseResult {
  unsigned long long sites = 0, selected = 0, ridges = 0;
  uint32_t rmax = 0;
  StatsAccum acc;
  double osum[2] = {0.0, 0.0};  // the reference's sequential sum and sum of squares
};

// The reference's sequential f64 sums of the calibrated map values
// (metrics.rs:215-224), on stream s, after the statistics accumulator acc has
// its maximum; results land in ctx->ordout.
void ordered_sums(bm_ctx* ctx, const float* d_map, long long n, float scale, const StatsAccum* acc, cudaStream_t s) {
  void* scratch = ensure(ctx, ctx->ordscratch, ordered_sum_scratch_bytes(n), "ordered-sum scratch");
  double* out = static_cast<double*>(ensure(ctx, ctx->ordout, 2 * sizeof(double), "ordered sums"));
  timed(ctx, KF_STATS_ORDER, s, "ordered sums", [&] {
    return launch_ordered_sums(d_map, n, scale, &acc->max_bits, scratch, out, s, &ctx->launches);
  });
}

// The buffers of one phase's distance transform.
struct EdtBufs {
  uint32_t* A;        // x pass output (kept for the chain passes), y pass input
  uint32_t* B;        // y pass output
  void* scratch;      // envelope scratch of the flagged lines
  uint32_t* selbits;  // selection bits
  Counters* ctr;
  uint8_t* redo;      // per-line flags of the windowed passes
};

EdtBufs edt_buffers(bm_ctx* ctx, Dims dm) {
  const size_t N = (size_t)dm.n();
  const size_t bits_bytes = (size_t)dm.nw() * dm.h * dm.d * sizeof(uint32_t);
  EdtBufs b;
  b.A = static_cast<uint32_t*>(ensure(ctx, ctx->dist, N * 4, "distance map"));
  b.B = static_cast<uint32_t*>(ensure(ctx, ctx->dist2, N * 4, "distance map"));
  b.scratch = ensure(ctx, ctx->stack, edt_scratch_bytes(dm), "envelope scratch");
  b.selbits = static_cast<uint32_t*>(ensure(ctx, ctx->selbits, bits_bytes, "selection bits"));
  b.ctr = static_cast<Counters*>(ensure(ctx, ctx->counters, sizeof(Counters), "counters"));
  const size_t redo_bytes = (size_t)dm.w * (dm.h > dm.d ? dm.h : dm.d);
  b.redo = static_cast<uint8_t*>(ensure(ctx, ctx->redo, redo_bytes, "line flags"));
  return b;
}

// The x and y passes of planes z0 .. z1-1: both work within a plane, so a slab
// of planes is a volume of its own (every offset is a whole number of planes,
// which keeps the 16-byte alignment of rows whose width is a multiple of 4).
// The counters accumulate over slabs.
void edt_xy(bm_ctx* ctx, Dims dm, const uint8_t* d_a, const uint8_t* d_b, int mode, const EdtBufs& b, int z0, int z1,
            cudaStream_t s) {
  const Dims sd{dm.w, dm.h, z1 - z0};
  const long long off = (long long)z0 * dm.w * dm.h;
  const uint8_t* a = d_a + off;
  const uint8_t* bb = d_b ? d_b + off : nullptr;
  uint32_t* A = b.A + off;
  uint32_t* B = b.B + off;
  uint32_t* sel = b.selbits + (long long)z0 * dm.h * dm.nw();
  timed(ctx, KF_EDT_X, s, "edt x pass",
        [&] { return launch_edt_x(a, bb, mode, sd, A, sel, b.ctr, s, &ctx->launches); });
  timed(ctx, KF_EDT_Y, s, "edt y pass", [&] {
    return launch_edt_window(1, A, B, sd, b.scratch, b.redo, b.ctr, ctx->wait_cycles, s, &ctx->launches);
  });
}

// One phase: EDT (+ local thickness unless edt_only, + the reference-order
// statistics sums when stats).  d_a / d_b are the device inputs for `mode`;
// results optionally go to d_edt (u32 EDT), d_map (f32 masked diameters) and
// d_sq (u32 propagated r^2).  xy_done: the x and y passes have already run on
// this context's buffers (slab by slab, as the inputs arrived), with its
// counters cleared before them.
void run_phase(bm_ctx* ctx, Dims dm, const uint8_t* d_a, const uint8_t* d_b, int mode, bool edt_only,
               uint32_t* d_edt, float* d_map, uint32_t* d_sq, float scale, bool stats, cudaStream_t s,
               PhaseResult& res, bool xy_done = false) {
  const size_t N = (size_t)dm.n();
  const size_t bits_bytes = (size_t)dm.nw() * dm.h * dm.d * sizeof(uint32_t);
  const EdtBufs eb = edt_buffers(ctx, dm);
  uint32_t* A = eb.A;
  uint32_t* B = eb.B;
  void* scratch = eb.scratch;
  uint32_t* selbits = eb.selbits;
  Counters* ctr = eb.ctr;
  uint8_t* redo = eb.redo;
  if (!xy_done) {
    check(ctx, cudaMemsetAsync(ctr, 0, sizeof(Counters), s), "memset");
    edt_xy(ctx, dm, d_a, d_b, mode, eb, 0, dm.d, s);
  }
  // local thickness keeps the x pass output (the chain passes read it): the z
  // pass then writes its own map
  uint32_t* E = d_edt ? d_edt
                      : (edt_only ? A : static_cast<uint32_t*>(ensure(ctx, ctx->edtmap, N * 4, "distance map")));
  timed(ctx, KF_EDT_Z, s, "edt z pass",
        [&] { return launch_edt_window(2, B, E, dm, scratch, redo, ctr, ctx->wait_cycles, s, &ctx->launches); });

  Counters hc;
  check(ctx, cudaMemcpyAsync(&hc, ctr, sizeof hc, cudaMemcpyDeviceToHost, s), "counter readback");
  check(ctx, cudaStreamSynchronize(s), "edt");
  if (hc.status) fail(ctx, BM_ERR_TIMEOUT, "a bounded device-side wait of the distance transform ran out");
  res.sites = hc.sites;
  res.selected = N - hc.sites;
  res.rmax = hc.rmax;
  if (hc.sites == 0) {
    const int phase = (mode == SEL_BACKGROUND) ? BM_PHASE_BACKGROUND : BM_PHASE_FOREGROUND;
    fail(ctx, BM_ERR_ALL_SELECTED,
         "distance transform is undefined for an all-%s volume unless an exterior convention is specified",
         phase_name(phase));
  }
  if (edt_only) return;

  ensure_lut(ctx, hc.rmax);
  const uint4* lut = static_cast<const uint4*>(ctx->lut.ptr);
  uint2* ridges = static_cast<uint2*>(ensure(ctx, ctx->ridges, (res.selected + 1) * sizeof(uint2), "ridge list"));
  const size_t rwords = (size_t)hc.rmax + 2;
  uint32_t* occ = static_cast<uint32_t*>(ensure(ctx, ctx->occ, rwords * 4, "r2 flags"));
  check(ctx, cudaMemsetAsync(occ, 0, rwords * 4, s), "memset");
  uint32_t* rbits = static_cast<uint32_t*>(ensure(ctx, ctx->ridgebits, bits_bytes, "ridge bits"));
  check(ctx, cudaMemsetAsync(rbits, 0, bits_bytes, s), "memset");
  timed(ctx, KF_RIDGE, s, "ridge kernel",
        [&] { return launch_ridges(E, selbits, dm, lut, ridges, ctr, occ, rbits, s, &ctx->launches); });
  const bool own_e = E != A && E != d_edt;  // E is the context's map: the chain passes may reuse it
  uint32_t* F = fill_phase(ctx, dm, ridges, ctr, res.selected, hc.rmax, occ, selbits, A, B, own_e ? E : nullptr,
                           rbits, d_sq ? d_sq : B, s);
  StatsAccum* acc = static_cast<StatsAccum*>(ensure(ctx, ctx->accum, sizeof(StatsAccum), "stats"));
  check(ctx, cudaMemsetAsync(acc, 0, sizeof(StatsAccum), s), "memset");
  FixedPartial* part = static_cast<FixedPartial*>(
      ensure(ctx, ctx->cpart, kCleanupMaxGrid * sizeof(FixedPartial), "stats partials"));
  // every value of the map is at least 2 * scale (diameters are >= 2), so its
  // f32 exponent is at least that of 2 * scale: the fixed-point base
  const float two_s = 2.0f * scale;
  uint32_t tb;
  std::memcpy(&tb, &two_s, 4);
  const int e2s = (int)(tb >> 23);
  const int e_lo = (e2s >= 1 && e2s + kFixedSpan <= 254) ? e2s : 4096;  // 4096: no fixed-point path
  unsigned cgrid = 0;
  // the statistics' ordered sums read the f32 map: keep one when the caller wants none
  float* cmap = (stats && !d_map) ? static_cast<float*>(ensure(ctx, ctx->ordmap, N * 4, "thickness map")) : d_map;
  timed(ctx, KF_CLEAN_FINAL, s, "cleanup",
        [&] {
          return launch_cleanup(F, selbits, dm, static_cast<const float*>(ctx->lutf.ptr), scale, cmap, acc, part,
                                e_lo, &ctr->tile_next[1], &cgrid, s, &ctx->launches);
        });
  if (stats) ordered_sums(ctx, cmap, (long long)N, scale, acc, s);
  std::vector<FixedPartial> hpart(cgrid);
  check(ctx, cudaMemcpyAsync(&res.acc, acc, sizeof(StatsAccum), cudaMemcpyDeviceToHost, s), "stats readback");
  if (stats)
    check(ctx, cudaMemcpyAsync(res.osum, ctx->ordout.ptr, 2 * sizeof(double), cudaMemcpyDeviceToHost, s),
          "stats readback");
  if (cgrid)
    check(ctx, cudaMemcpyAsync(hpart.data(), part, cgrid * sizeof(FixedPartial), cudaMemcpyDeviceToHost, s),
          "stats readback");
  check(ctx, cudaMemcpyAsync(&hc, ctr, sizeof hc, cudaMemcpyDeviceToHost, s), "counter readback");
  check(ctx, cudaStreamSynchronize(s), "local thickness");
  if (e_lo != 4096) fold_fixed_partials(res.acc, hpart.data(), cgrid, e_lo);
  res.ridges = hc.ridges;
}

// nonzero_stats (metrics.rs:228-241; quantile fields NaN) from the reference's
// own sequential sums osum = {sum, sum of squares}; the exact sums are
// reported beside them.
int finish_stats(bm_ctx* ctx, const StatsAccum& a, const double* osum, bm_stats* out) {
  if (a.count == 0) {
    set_err(ctx, "cannot compute statistics because the selected phase is empty");
    return BM_ERR_EMPTY;
  }
  double xsum, xss;
  exact_sums_to_double(a, &xsum, &xss);
  const double sum = osum[0], ss = osum[1];
  const double c = (double)a.count;
  const double mean = sum / c;
  const double centered = (c * ss - sum * sum) / c;
  const double sd = (a.count > 1 && centered > 0.0) ? std::sqrt(centered / (c - 1.0)) : 0.0;
  float mxf;
  std::memcpy(&mxf, &a.max_bits, 4);
  if (out) {
    out->count = a.count;
    out->mean = mean;
    out->standard_deviation = sd;
    out->maximum = (double)mxf;
    out->median = out->percentile_10 = out->percentile_25 = out->percentile_75 = out->percentile_90 = NAN;
    out->interquartile_range = NAN;
    out->coefficient_of_variation = sd / mean;
    out->sum = sum;
    out->sum_of_squares = ss;
    out->exact_sum = xsum;
    out->exact_sum_of_squares = xss;
  }
  return BM_OK;
}

// Quantiles of the finite positive values of d_map (metrics.rs:242-298):
// median, P10, P25, P75, P90 by numpy-linear interpolation of exact order
// statistics, then (q as f32 * scale_f32) as f64; IQR = P75 - P25.
void quantiles(bm_ctx* ctx, const float* d_map, long long n, unsigned long long count, double scale,
               bm_stats* out, cudaStream_t s) {
  static const double kQ[5] = {0.5, 0.1, 0.25, 0.75, 0.9};  // metrics.rs:247-251
  unsigned long long ranks[10];
  double frac[5];
  for (int i = 0; i < 5; ++i) {
    const double position = kQ[i] * (double)(count - 1);
    const double lo = std::floor(position), hi = std::ceil(position);
    ranks[2 * i] = (unsigned long long)lo;
    ranks[2 * i + 1] = (unsigned long long)hi;
    frac[i] = position - lo;
  }
  uint32_t* hist = static_cast<uint32_t*>(ensure(ctx, ctx->qhist, (size_t)17 * 65536 * 4, "quantile histograms"));
  uint32_t* dtargets = static_cast<uint32_t*>(ensure(ctx, ctx->qtargets, 16 * 4, "quantile targets"));
  check(ctx, cudaMemsetAsync(hist, 0, (size_t)65536 * 4, s), "memset");
  timed(ctx, KF_QUANTILE, s, "quantile histogram", [&] { return launch_hist_hi(d_map, n, hist, s, &ctx->launches); });
  std::vector<uint32_t> hh(65536);
  check(ctx, cudaMemcpyAsync(hh.data(), hist, 65536 * 4, cudaMemcpyDeviceToHost, s), "histogram readback");
  check(ctx, cudaStreamSynchronize(s), "quantile histogram");
  // locate every rank's high-16 bin and its rank inside that bin
  uint32_t tgt[10];
  unsigned long long resid[10];
  for (int r = 0; r < 10; ++r) {
    unsigned long long cum = 0;
    uint32_t b = 0;
    for (; b < 65536; ++b) {
      if (cum + hh[b] > ranks[r]) break;
      cum += hh[b];
    }
    if (b == 65536) fail(ctx, BM_ERR_CUDA, "quantile rank %llu beyond %llu values", ranks[r], cum);
    tgt[r] = b;
    resid[r] = ranks[r] - cum;
  }
  uint32_t uniq[10];
  int nu = 0;
  int slot_of[10];
  for (int r = 0; r < 10; ++r) {
    int j = 0;
    while (j < nu && uniq[j] != tgt[r]) ++j;
    if (j == nu) uniq[nu++] = tgt[r];
    slot_of[r] = j;
  }
  uint32_t* lo = hist + 65536;
  check(ctx, cudaMemcpyAsync(dtargets, uniq, (size_t)nu * 4, cudaMemcpyHostToDevice, s), "targets upload");
  check(ctx, cudaMemsetAsync(lo, 0, (size_t)nu * 65536 * 4, s), "memset");
  timed(ctx, KF_QUANTILE, s, "quantile histogram",
        [&] { return launch_hist_lo(d_map, n, dtargets, nu, lo, s, &ctx->launches); });
  std::vector<uint32_t> hl((size_t)nu * 65536);
  check(ctx, cudaMemcpyAsync(hl.data(), lo, hl.size() * 4, cudaMemcpyDeviceToHost, s), "histogram readback");
  check(ctx, cudaStreamSynchronize(s), "quantile histogram");
  double v[10];
  for (int r = 0; r < 10; ++r) {
    const uint32_t* h = hl.data() + (size_t)slot_of[r] * 65536;
    unsigned long long cum = 0;
    uint32_t b = 0;
    for (; b < 65536; ++b) {
      if (cum + h[b] > resid[r]) break;
      cum += h[b];
    }
    const uint32_t bits = (tgt[r] << 16) | b;
    float f;
    std::memcpy(&f, &bits, 4);
    v[r] = (double)f;
  }
  const float sf = (float)scale;
  double q[5];
  for (int i = 0; i < 5; ++i) {
    const double lv = v[2 * i], uv = v[2 * i + 1];
    const double qv = lv + frac[i] * (uv - lv);  // metrics.rs:289
    q[i] = (double)((float)qv * sf);             // metrics.rs:290
  }
  out->median = q[0];
  out->percentile_10 = q[1];
  out->percentile_25 = q[2];
  out->percentile_75 = q[3];
  out->percentile_90 = q[4];
  out->interquartile_range = q[3] - q[2];
}

template <class F>
int guarded(bm_ctx* ctx, F&& f) {
  if (!ctx) return BM_ERR_INVALID;
  std::lock_guard<std::mutex> lock(ctx->mu);
  ctx->last_error.clear();
  try {
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) {
      cudaGetLastError();
      fail(ctx, BM_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
    }
    return f();
  } catch (const CallError& ce) {
    return ce.status;
  } catch (const std::bad_alloc&) {
    ctx->last_error = "host allocation failed";
    return BM_ERR_OOM;
  }
}

cudaStream_t pick_stream(bm_ctx* ctx, void* stream) {
  return stream ? static_cast<cudaStream_t>(stream) : ctx->stream;
}

int edt_device_impl(bm_ctx* ctx, const uint8_t* d_vol, Dims dm, int phase, uint32_t* d_out, cudaStream_t s) {
  PhaseResult r;
  run_phase(ctx, dm, d_vol, nullptr, phase == BM_PHASE_BACKGROUND ? SEL_BACKGROUND : SEL_FOREGROUND, true, d_out,
            nullptr, nullptr, 1.0f, false, s, r);
  return BM_OK;
}

int lt_device_impl(bm_ctx* ctx, const uint8_t* d_vol, Dims dm, int phase, float* d_out, uint32_t* d_sq,
                   cudaStream_t s) {
  PhaseResult r;
  run_phase(ctx, dm, d_vol, nullptr, phase == BM_PHASE_BACKGROUND ? SEL_BACKGROUND : SEL_FOREGROUND, false,
            nullptr, d_out, d_sq, 1.0f, false, s, r);
  return BM_OK;
}

void check_phase(bm_ctx* ctx, int phase) {
  if (phase != BM_PHASE_FOREGROUND && phase != BM_PHASE_BACKGROUND)
    fail(ctx, BM_ERR_INVALID, "phase must be 0 (foreground) or 1 (background); got %d", phase);
}

// Nonzero bytes of a word, as a multiple of 8 (0xff per nonzero byte, then
// one population count).
__device__ __forceinline__ unsigned nz8(uint32_t v) { return (unsigned)__popc(__vcmpne4(v, 0u)); }
__device__ __forceinline__ unsigned both8(uint32_t r, uint32_t b) {
  return (unsigned)__popc(__vcmpne4(r, 0u) & __vcmpne4(b, 0u));
}

// ROI voxels and ROI-clipped bone voxels (the bails of metrics.rs:70-99).
// With both volumes 16-byte aligned, every thread reads two 16-byte words of
// each per step (bytes in flight for the HBM rate); the last n % 32 bytes and
// unaligned inputs take the byte loop.
__global__ void count_roi_kernel(const uint8_t* __restrict__ bone, const uint8_t* __restrict__ roi, long long n,
                                 unsigned long long* __restrict__ out) {
  unsigned long long in_roi = 0, bone_in = 0;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nth = (long long)gridDim.x * blockDim.x;
  long long head = 0;
  if (((reinterpret_cast<uintptr_t>(bone) | reinterpret_cast<uintptr_t>(roi)) & 15u) == 0) {
    const uint4* R = reinterpret_cast<const uint4*>(roi);
    const uint4* B = reinterpret_cast<const uint4*>(bone);
    const long long pairs = n / 32;
    unsigned long long r8 = 0, b8 = 0;
    for (long long i = tid; i < pairs; i += nth) {
      const uint4 r0 = __ldcs(R + 2 * i), r1 = __ldcs(R + 2 * i + 1);
      const uint4 b0 = __ldcs(B + 2 * i), b1 = __ldcs(B + 2 * i + 1);
      r8 += nz8(r0.x) + nz8(r0.y) + nz8(r0.z) + nz8(r0.w) + nz8(r1.x) + nz8(r1.y) + nz8(r1.z) + nz8(r1.w);
      b8 += both8(r0.x, b0.x) + both8(r0.y, b0.y) + both8(r0.z, b0.z) + both8(r0.w, b0.w) + both8(r1.x, b1.x) +
            both8(r1.y, b1.y) + both8(r1.z, b1.z) + both8(r1.w, b1.w);
    }
    in_roi = r8 >> 3;
    bone_in = b8 >> 3;
    head = pairs * 32;
  }
  for (long long i = head + tid; i < n; i += nth) {
    const bool r = roi[i] != 0;
    in_roi += r;
    bone_in += (r && bone[i] != 0);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    in_roi += __shfl_xor_sync(0xffffffffu, in_roi, o);
    bone_in += __shfl_xor_sync(0xffffffffu, bone_in, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (in_roi) atomicAdd(&out[0], in_roi);
    if (bone_in) atomicAdd(&out[1], bone_in);
  }
}

// ROI voxels, ROI-clipped bone voxels, and those of them with a 6-neighbour
// outside the volume or outside the ROI (metrics.rs:166-202).
__global__ void volume_counts_kernel(const uint8_t* __restrict__ bone, const uint8_t* __restrict__ roi, Dims dm,
                                     unsigned long long* __restrict__ out) {
  unsigned long long c_roi = 0, c_bone = 0, c_edge = 0;
  const long long n = dm.n();
  const long long sl = (long long)dm.w * dm.h;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const bool r = roi[i] != 0;
    c_roi += r;
    if (r && bone[i] != 0) {
      ++c_bone;
      const int z = (int)(i / sl);
      const long long rem = i - (long long)z * sl;
      const int y = (int)(rem / dm.w), x = (int)(rem - (long long)y * dm.w);
      const bool edge = x == 0 || y == 0 || z == 0 || x == dm.w - 1 || y == dm.h - 1 || z == dm.d - 1 ||
                        roi[i - 1] == 0 || roi[i + 1] == 0 || roi[i - dm.w] == 0 || roi[i + dm.w] == 0 ||
                        roi[i - sl] == 0 || roi[i + sl] == 0;
      c_edge += edge;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    c_roi += __shfl_xor_sync(0xffffffffu, c_roi, o);
    c_bone += __shfl_xor_sync(0xffffffffu, c_bone, o);
    c_edge += __shfl_xor_sync(0xffffffffu, c_edge, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (c_roi) atomicAdd(&out[0], c_roi);
    if (c_bone) atomicAdd(&out[1], c_bone);
    if (c_edge) atomicAdd(&out[2], c_edge);
  }
}

int volume_metrics_impl(bm_ctx* ctx, const uint8_t* d_bone, const uint8_t* d_roi, Dims dm, const double* sp,
                        bm_volume_metrics* out, cudaStream_t s) {
  for (int i = 0; i < 3; ++i)
    if (!std::isfinite(sp[i]) || sp[i] <= 0.0)
      fail(ctx, BM_ERR_SPACING, "voxel spacings must be finite and positive; got [%g, %g, %g]", sp[0], sp[1], sp[2]);
  unsigned long long* dc = static_cast<unsigned long long*>(ensure(ctx, ctx->counters, sizeof(Counters), "counters"));
  check(ctx, cudaMemsetAsync(dc, 0, 24, s), "memset");
  timed(ctx, KF_COUNT_ROI, s, "volume counts", [&] {
    volume_counts_kernel<<<152 * 8, 256, 0, s>>>(d_bone, d_roi, dm, dc);
    ++ctx->launches;
    return cudaGetLastError();
  });
  unsigned long long hc[3];
  check(ctx, cudaMemcpyAsync(hc, dc, 24, cudaMemcpyDeviceToHost, s), "count readback");
  check(ctx, cudaStreamSynchronize(s), "volume counts");
  const double voxel_volume = ((1.0 * sp[0]) * sp[1]) * sp[2];  // metrics.rs:123 (product)
  out->roi_voxels = hc[0];
  out->bone_voxels = hc[1];
  out->boundary_bone_voxels = hc[2];
  out->bone_volume = (double)hc[1] * voxel_volume;
  out->total_volume = (double)hc[0] * voxel_volume;
  out->bone_volume_fraction = out->bone_volume / out->total_volume;
  out->roi_boundary_bone_fraction = (double)hc[2] / (double)hc[1];
  return BM_OK;
}

// The context's twin (created on first use, with the parent's profiling state).
bm_ctx* twin_of(bm_ctx* ctx) {
  if (!ctx->inputs_ready) check(ctx, cudaEventCreateWithFlags(&ctx->inputs_ready, cudaEventDisableTiming), "event");
  if (ctx->twin) return ctx->twin;
  bm_ctx* t = nullptr;
  const int st = bm_ctx_create(ctx->device, &t);
  if (st != BM_OK) fail(ctx, st, "second stream context creation failed");
  t->profiling = ctx->profiling;
  t->site_method = ctx->site_method;
  t->fill_rows = ctx->fill_rows;
  t->wait_cycles = ctx->wait_cycles;
  ctx->twin = t;
  return t;
}

// metrics.rs:70-78, and the library's flags
void check_call(bm_ctx* ctx, double spacing, unsigned flags) {
  if (!std::isfinite(spacing) || spacing <= 0.0)
    fail(ctx, BM_ERR_SPACING, "voxel spacings must be finite and positive; got [%g, %g, %g]", spacing, spacing,
         spacing);
  if (flags & ~(unsigned)(BM_FLAG_QUANTILES | BM_FLAG_BONEJ_ROI))
    fail(ctx, BM_ERR_INVALID, "unknown flags 0x%x", flags);
}

// Work already done by the upload pipeline of bm_tbth_tbsp: the ROI counts, and
// the x and y passes of either phase.
struct Prestaged {
  unsigned long long roi = 0, bone_in_roi = 0;
  bool bone_xy = false, marrow_xy = false;
};

bool phases_side_by_side(const bm_ctx* ctx, Dims dm) { return ctx->split_phases && dm.n() <= kSplitMaxVoxels; }

int tbth_device_impl(bm_ctx* ctx, const uint8_t* d_bone, const uint8_t* d_roi, Dims dm, double spacing,
                     unsigned flags, bm_stats* th, bm_stats* sp, float* d_thmap, float* d_spmap, cudaStream_t s,
                     const Prestaged* pre = nullptr) {
  check_call(ctx, spacing, flags);
  const long long N = dm.n();
  unsigned long long hc[2];
  if (pre) {
    hc[0] = pre->roi;
    hc[1] = pre->bone_in_roi;
  } else {
    unsigned long long* dcnt =
        static_cast<unsigned long long*>(ensure(ctx, ctx->roicount, 2 * sizeof(unsigned long long), "counts"));
    check(ctx, cudaMemsetAsync(dcnt, 0, 16, s), "memset");
    timed(ctx, KF_COUNT_ROI, s, "count kernel", [&] {
      count_roi_kernel<<<152 * 8, 256, 0, s>>>(d_bone, d_roi, N, dcnt);
      ++ctx->launches;
      return cudaGetLastError();
    });
    check(ctx, cudaMemcpyAsync(hc, dcnt, 16, cudaMemcpyDeviceToHost, s), "count readback");
    check(ctx, cudaStreamSynchronize(s), "count kernel");
  }
  if (hc[0] == 0) fail(ctx, BM_ERR_ROI_EMPTY, "ROI mask contains no included voxels");
  if ((flags & BM_FLAG_BONEJ_ROI) && hc[0] == (unsigned long long)N)
    fail(ctx, BM_ERR_ROI_FULL, "BoneJ compatibility mode requires an ROI mask with both inside and outside voxels");
  if (hc[1] == 0) fail(ctx, BM_ERR_NO_BONE, "ROI contains no bone voxels");
  if (hc[1] == hc[0]) fail(ctx, BM_ERR_NO_MARROW, "ROI contains no marrow voxels");

  const float scale = (float)spacing;  // metrics.rs:213
  const bool want_q = (flags & BM_FLAG_QUANTILES) != 0;
  float* qm = nullptr;
  if (want_q && (!d_thmap || !d_spmap))
    qm = static_cast<float*>(ensure(ctx, ctx->qmap, (size_t)N * 4, "quantile map"));
  // The two phases are independent: the marrow phase runs on the twin context
  // (its own stream and buffers, on a second host thread) while this thread
  // runs the bone phase, so their kernels overlap on the GPU.  Results and
  // errors are reported in the reference's order (bone first).
  PhaseResult rb, rm;
  // Side by side only while one phase cannot fill the GPU: on 1024^3 the two
  // phases' kernels compete (174 ms against 159 ms one after the other), on
  // 512^3 and below they fill each other's gaps.
  const bool bone_xy = pre && pre->bone_xy, marrow_xy = pre && pre->marrow_xy;
  if (!phases_side_by_side(ctx, dm)) {
    float* mb = d_thmap ? d_thmap : qm;
    run_phase(ctx, dm, d_bone, d_roi, SEL_BONE_IN_ROI, false, nullptr, mb, nullptr, scale, true, s, rb, bone_xy);
    int st = finish_stats(ctx, rb.acc, rb.osum, th);
    if (st) return st;
    if (want_q && th) quantiles(ctx, mb, N, rb.acc.count, spacing, th, s);
    float* mm = d_spmap ? d_spmap : qm;
    run_phase(ctx, dm, d_bone, d_roi, SEL_MARROW_IN_ROI, false, nullptr, mm, nullptr, scale, true, s, rm, marrow_xy);
    st = finish_stats(ctx, rm.acc, rm.osum, sp);
    if (st) return st;
    if (want_q && sp) quantiles(ctx, mm, N, rm.acc.count, spacing, sp, s);
    return BM_OK;
  }
  bm_ctx* tw = twin_of(ctx);
  float* mb = d_thmap ? d_thmap : qm;
  float* mm = d_spmap ? d_spmap
                      : (want_q ? static_cast<float*>(ensure(tw, tw->qmap, (size_t)N * 4, "quantile map")) : nullptr);
  check(ctx, cudaEventRecord(ctx->inputs_ready, s), "event record");
  int twin_status = BM_OK;
  std::thread marrow([&] {
    try {
      cudaSetDevice(tw->device);
      check(tw, cudaStreamWaitEvent(tw->stream, ctx->inputs_ready, 0), "stream wait");
      run_phase(tw, dm, d_bone, d_roi, SEL_MARROW_IN_ROI, false, nullptr, mm, nullptr, scale, true, tw->stream, rm,
                marrow_xy);
    } catch (const CallError& e) {
      twin_status = e.status;
    } catch (const std::bad_alloc&) {
      tw->last_error = "host allocation failed";
      twin_status = BM_ERR_OOM;
    }
  });
  int bone_status = BM_OK;
  try {
    run_phase(ctx, dm, d_bone, d_roi, SEL_BONE_IN_ROI, false, nullptr, mb, nullptr, scale, true, s, rb, bone_xy);
  } catch (const CallError& e) {
    bone_status = e.status;
  }
  marrow.join();
  ctx->launches += tw->launches;
  tw->launches = 0;
  if (bone_status != BM_OK) throw CallError{bone_status};
  int st = finish_stats(ctx, rb.acc, rb.osum, th);
  if (st) return st;
  if (want_q && th) quantiles(ctx, mb, N, rb.acc.count, spacing, th, s);
  if (twin_status != BM_OK) {
    ctx->last_error = tw->last_error;
    throw CallError{twin_status};
  }
  st = finish_stats(ctx, rm.acc, rm.osum, sp);
  if (st) return st;
  if (want_q && sp) quantiles(ctx, mm, N, rm.acc.count, spacing, sp, s);
  return BM_OK;
}

uint8_t* stage_input(bm_ctx* ctx, Buffer& b, const uint8_t* host, size_t n, cudaStream_t s) {
  uint8_t* d = static_cast<uint8_t*>(ensure(ctx, b, n, "input volume"));
  check(ctx, cudaMemcpyAsync(d, host, n, cudaMemcpyHostToDevice, s), "input upload");
  return d;
}

// bm_tbth_tbsp from host inputs of at least kPipeMinVoxels: bone and ROI go up
// on a copy stream in kPipeSlabs slabs of planes, and each slab's ROI counts
// and x and y passes (of both phases when they run side by side, else of the
// bone phase) start as soon as the slab has landed, so that the transfer hides
// most of those passes.  The bails are checked once every slab is counted; the
// passes that ran before them only wrote the phases' own buffers.
constexpr long long kPipeMinVoxels = 1ll << 22;
constexpr int kPipeSlabs = 8;

// On every exit: no copy from the caller's buffers, and no pass reading the
// uploaded inputs, is left in flight.
struct UploadFence {
  bm_ctx* ctx;
  bm_ctx* twin;
  ~UploadFence() {
    if (ctx->upload_stream) cudaStreamSynchronize(ctx->upload_stream);
    if (twin) cudaStreamSynchronize(twin->stream);
  }
};

int tbth_host_pipelined(bm_ctx* ctx, const uint8_t* bone, const uint8_t* roi, Dims dm, double spacing, unsigned flags,
                        bm_stats* th, bm_stats* sp, float* d_th, float* d_sp, cudaStream_t s) {
  check_call(ctx, spacing, flags);
  const size_t N = (size_t)dm.n();
  uint8_t* d_bone = static_cast<uint8_t*>(ensure(ctx, ctx->in_a, N, "input volume"));
  uint8_t* d_roi = static_cast<uint8_t*>(ensure(ctx, ctx->in_b, N, "input volume"));
  if (!ctx->upload_stream)
    check(ctx, cudaStreamCreateWithFlags(&ctx->upload_stream, cudaStreamNonBlocking), "stream create");
  while ((int)ctx->slab_ready.size() < kPipeSlabs) {
    cudaEvent_t e = nullptr;
    check(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event create");
    ctx->slab_ready.push_back(e);
  }
  bm_ctx* tw = phases_side_by_side(ctx, dm) ? twin_of(ctx) : nullptr;
  UploadFence fence{ctx, tw};
  const EdtBufs eb = edt_buffers(ctx, dm);
  check(ctx, cudaMemsetAsync(eb.ctr, 0, sizeof(Counters), s), "memset");
  unsigned long long* dcnt =
      static_cast<unsigned long long*>(ensure(ctx, ctx->roicount, 2 * sizeof(unsigned long long), "counts"));
  check(ctx, cudaMemsetAsync(dcnt, 0, 16, s), "memset");
  // the twin's calls report their errors on this context
  auto on_twin = [&](auto&& f) {
    try {
      f();
    } catch (const CallError&) {
      ctx->last_error = tw->last_error;
      throw;
    }
  };
  EdtBufs et{};
  if (tw) on_twin([&] {
    et = edt_buffers(tw, dm);
    check(tw, cudaMemsetAsync(et.ctr, 0, sizeof(Counters), tw->stream), "memset");
  });
  const int K = dm.d < kPipeSlabs ? dm.d : kPipeSlabs;
  const size_t plane = (size_t)dm.w * dm.h;
  for (int k = 0; k < K; ++k) {
    const int z0 = (int)((long long)dm.d * k / K), z1 = (int)((long long)dm.d * (k + 1) / K);
    const size_t off = (size_t)z0 * plane, len = (size_t)(z1 - z0) * plane;
    check(ctx, cudaMemcpyAsync(d_bone + off, bone + off, len, cudaMemcpyHostToDevice, ctx->upload_stream),
          "input upload");
    check(ctx, cudaMemcpyAsync(d_roi + off, roi + off, len, cudaMemcpyHostToDevice, ctx->upload_stream),
          "input upload");
    check(ctx, cudaEventRecord(ctx->slab_ready[k], ctx->upload_stream), "event record");
    check(ctx, cudaStreamWaitEvent(s, ctx->slab_ready[k], 0), "stream wait");
    timed(ctx, KF_COUNT_ROI, s, "count kernel", [&] {
      count_roi_kernel<<<152 * 8, 256, 0, s>>>(d_bone + off, d_roi + off, (long long)len, dcnt);
      ++ctx->launches;
      return cudaGetLastError();
    });
    edt_xy(ctx, dm, d_bone, d_roi, SEL_BONE_IN_ROI, eb, z0, z1, s);
    if (tw) on_twin([&] {
      check(tw, cudaStreamWaitEvent(tw->stream, ctx->slab_ready[k], 0), "stream wait");
      edt_xy(tw, dm, d_bone, d_roi, SEL_MARROW_IN_ROI, et, z0, z1, tw->stream);
    });
  }
  unsigned long long hc[2];
  check(ctx, cudaMemcpyAsync(hc, dcnt, 16, cudaMemcpyDeviceToHost, s), "count readback");
  check(ctx, cudaStreamSynchronize(s), "count kernel");
  Prestaged pre;
  pre.roi = hc[0];
  pre.bone_in_roi = hc[1];
  pre.bone_xy = true;
  pre.marrow_xy = tw != nullptr;
  return tbth_device_impl(ctx, d_bone, d_roi, dm, spacing, flags, th, sp, d_th, d_sp, s, &pre);
}

}  // namespace

namespace bm {
// Message returned by bm_last_error(NULL, ...) on this thread (used by the
// entry points that take no context).
void set_thread_error(const char* msg) { g_create_error = msg; }

// The per-call working buffers of a context (released by bm_ctx_trim; the
// cached tables stay).
std::vector<Buffer*> work_buffers(bm_ctx* ctx) {
  return {&ctx->in_a,      &ctx->in_b,       &ctx->dist,        &ctx->dist2,   &ctx->stack,  &ctx->edtmap,
          &ctx->chainmap,  &ctx->fillmap,    &ctx->selbits,     &ctx->ridgebits, &ctx->ridges, &ctx->accum,
          &ctx->cpart,     &ctx->outmap,     &ctx->outmap2,     &ctx->occ,     &ctx->rank,   &ctx->rvals,
          &ctx->bincounts, &ctx->binoffsets, &ctx->binentries,  &ctx->scanscratch, &ctx->redo, &ctx->qhist,
          &ctx->qtargets,  &ctx->qmap,       &ctx->rgeo,        &ctx->ordmap,  &ctx->ordscratch, &ctx->ordout,
          &ctx->tileorder};
}

size_t cached_bytes(const bm_ctx* ctx) {
  size_t t = 0;
  for (const Buffer* b : work_buffers(const_cast<bm_ctx*>(ctx))) t += b->bytes;
  if (ctx->twin) t += cached_bytes(ctx->twin);
  return t;
}
}  // namespace bm

extern "C" {

int bm_ctx_create(int device, bm_ctx** out) {
  if (!out) return BM_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_err(nullptr, "no CUDA device available: %s", e == cudaSuccess ? "device count is 0" : cudaGetErrorString(e));
    return BM_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= ndev) {
    set_err(nullptr, "device %d out of range (0..%d)", device, ndev - 1);
    return BM_ERR_INVALID;
  }
  bm_ctx* ctx = new (std::nothrow) bm_ctx();
  if (!ctx) return BM_ERR_OOM;
  ctx->device = device;
  e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_err(nullptr, "context creation failed: %s", cudaGetErrorString(e));
    delete ctx;
    return BM_ERR_CUDA;
  }
  *out = ctx;
  return BM_OK;
}

int bm_ctx_trim(bm_ctx* ctx) {
  return guarded(ctx, [&]() -> int {
    cudaStreamSynchronize(ctx->stream);
    if (ctx->twin) bm_ctx_trim(ctx->twin);
    for (Buffer* b : work_buffers(ctx)) release(*b);
    return BM_OK;
  });
}

void bm_ctx_destroy(bm_ctx* ctx) {
  if (!ctx) return;
  {
    std::lock_guard<std::mutex> plock(ctx->pool_mu);
    if (ctx->pool) pool_destroy(ctx->pool);
    ctx->pool = nullptr;
  }
  {
    std::lock_guard<std::mutex> lock(ctx->mu);
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->twin) bm_ctx_destroy(ctx->twin);
    ctx->twin = nullptr;
    if (ctx->inputs_ready) cudaEventDestroy(ctx->inputs_ready);
    if (ctx->upload_stream) {
      cudaStreamSynchronize(ctx->upload_stream);
      cudaStreamDestroy(ctx->upload_stream);
    }
    for (cudaEvent_t e : ctx->slab_ready) cudaEventDestroy(e);
    for (Buffer* b : work_buffers(ctx)) release(*b);
    for (Buffer* b : {&ctx->lut, &ctx->counters, &ctx->roicount, &ctx->host_pinned, &ctx->fillinfo}) release(*b);
    for (const ProfRec& r : ctx->prof) {
      cudaEventDestroy(r.start);
      cudaEventDestroy(r.stop);
    }
    for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
    release(ctx->surf_off);
    release(ctx->surf_pts);
    release(ctx->lutf);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
  }
  delete ctx;
}

const char* bm_status_string(int status) {
  switch (status) {
    case BM_OK: return "ok";
    case BM_ERR_ALL_SELECTED: return "all voxels selected";
    case BM_ERR_DIMS: return "invalid dimensions";
    case BM_ERR_OOM: return "out of device memory";
    case BM_ERR_CUDA: return "CUDA error";
    case BM_ERR_TIMEOUT: return "device wait timed out";
    case BM_ERR_INVALID: return "invalid argument";
    case BM_ERR_EMPTY: return "empty phase";
    case BM_ERR_ROI_EMPTY: return "empty ROI";
    case BM_ERR_NO_BONE: return "no bone in ROI";
    case BM_ERR_NO_MARROW: return "no marrow in ROI";
    case BM_ERR_NO_DEVICE: return "no CUDA device";
    case BM_ERR_SPACING: return "invalid spacing";
    case BM_ERR_ROI_FULL: return "ROI has no outside voxels";
    case BM_ERR_BUSY: return "busy";
    default: return "unknown status";
  }
}

size_t bm_last_error(const bm_ctx* ctx, char* buf, size_t len) {
  const std::string& s = ctx ? ctx->last_error : g_create_error;
  if (buf && len) {
    const size_t n = s.size() < len - 1 ? s.size() : len - 1;
    std::memcpy(buf, s.data(), n);
    buf[n] = 0;
  }
  return s.size();
}

uint64_t bm_ctx_launch_count(const bm_ctx* ctx) { return ctx ? ctx->launches : 0; }

int bm_ctx_set_concurrent_phases(bm_ctx* ctx, int on) {
  return guarded(ctx, [&]() -> int {
    ctx->split_phases = on != 0;
    return BM_OK;
  });
}

int bm_ctx_set_site_method(bm_ctx* ctx, int method) {
  return guarded(ctx, [&]() -> int {
    if (method != BM_SITES_AUTO && method != BM_SITES_SPHERES && method != BM_SITES_CHAINS)
      fail(ctx, BM_ERR_INVALID, "site method must be 0 (auto), 1 (spheres) or 2 (chains); got %d", method);
    ctx->site_method = method;
    if (ctx->twin) ctx->twin->site_method = method;
    return BM_OK;
  });
}

int bm_ctx_set_fill_tile_rows(bm_ctx* ctx, int rows) {
  return guarded(ctx, [&]() -> int {
    if (rows != 0 && rows != 16 && rows != 32 && rows != 64)
      fail(ctx, BM_ERR_INVALID, "fill tile rows must be 0 (by volume size), 16, 32 or 64; got %d", rows);
    ctx->fill_rows = rows;
    if (ctx->twin) ctx->twin->fill_rows = rows;
    return BM_OK;
  });
}

int bm_ctx_set_wait_cycles(bm_ctx* ctx, long long cycles) {
  return guarded(ctx, [&]() -> int {
    ctx->wait_cycles = cycles < 0 ? -1 : cycles;
    if (ctx->twin) ctx->twin->wait_cycles = ctx->wait_cycles;
    return BM_OK;
  });
}

int bm_profile_enable(bm_ctx* ctx, int on) {
  return guarded(ctx, [&]() -> int {
    fold_profile(ctx);
    if (on) {
      for (int i = 0; i < KF_COUNT; ++i) {
        ctx->prof_ms[i] = 0.0;
        ctx->prof_n[i] = 0;
      }
    }
    ctx->profiling = on != 0;
    if (ctx->twin) bm_profile_enable(ctx->twin, on);
    return BM_OK;
  });
}

int bm_profile_read(bm_ctx* ctx, bm_kernel_time* out, size_t cap, size_t* count) {
  return guarded(ctx, [&]() -> int {
    fold_profile(ctx);
    if (ctx->twin) {  // the twin's kernels count as this context's
      bm_ctx* t = ctx->twin;
      std::lock_guard<std::mutex> tl(t->mu);
      fold_profile(t);
      for (int i = 0; i < KF_COUNT; ++i) {
        ctx->prof_ms[i] += t->prof_ms[i];
        ctx->prof_n[i] += t->prof_n[i];
        t->prof_ms[i] = 0.0;
        t->prof_n[i] = 0;
      }
    }
    size_t n = 0;
    for (int i = 0; i < KF_COUNT; ++i) {
      if (out && n < cap) {
        std::memset(out[n].name, 0, sizeof out[n].name);
        std::strncpy(out[n].name, kFamilyName[i], sizeof out[n].name - 1);
        out[n].launches = ctx->prof_n[i];
        out[n].total_ms = ctx->prof_ms[i];
      }
      ++n;
    }
    if (count) *count = n;
    return BM_OK;
  });
}

int bm_edt_sq_device(bm_ctx* ctx, const uint8_t* d_volume, size_t width, size_t height, size_t depth, int phase,
                     uint32_t* d_out, void* stream) {
  return guarded(ctx, [&]() -> int {
    if (!d_volume || !d_out) fail(ctx, BM_ERR_INVALID, "null pointer");
    check_phase(ctx, phase);
    const Dims dm = check_dims(ctx, width, height, depth);
    return edt_device_impl(ctx, d_volume, dm, phase, d_out, pick_stream(ctx, stream));
  });
}

int bm_edt_sq(bm_ctx* ctx, const uint8_t* volume, size_t width, size_t height, size_t depth, int phase,
              uint32_t* out) {
  return guarded(ctx, [&]() -> int {
    if (!volume || !out) fail(ctx, BM_ERR_INVALID, "null pointer");
    check_phase(ctx, phase);
    const Dims dm = check_dims(ctx, width, height, depth);
    const size_t N = (size_t)dm.n();
    cudaStream_t s = ctx->stream;
    uint8_t* d_in = stage_input(ctx, ctx->in_a, volume, N, s);
    uint32_t* d_out = static_cast<uint32_t*>(ensure(ctx, ctx->fillmap, N * 4, "output"));
    edt_device_impl(ctx, d_in, dm, phase, d_out, s);
    check(ctx, cudaMemcpyAsync(out, d_out, N * 4, cudaMemcpyDeviceToHost, s), "result download");
    check(ctx, cudaStreamSynchronize(s), "result download");
    return BM_OK;
  });
}

int bm_local_thickness_device(bm_ctx* ctx, const uint8_t* d_volume, size_t width, size_t height, size_t depth,
                              int phase, float* d_out, uint32_t* d_squared_thickness, void* stream) {
  return guarded(ctx, [&]() -> int {
    if (!d_volume || !d_out) fail(ctx, BM_ERR_INVALID, "null pointer");
    check_phase(ctx, phase);
    const Dims dm = check_dims(ctx, width, height, depth);
    return lt_device_impl(ctx, d_volume, dm, phase, d_out, d_squared_thickness, pick_stream(ctx, stream));
  });
}

int bm_local_thickness(bm_ctx* ctx, const uint8_t* volume, size_t width, size_t height, size_t depth, int phase,
                       float* out, uint32_t* squared_thickness) {
  return guarded(ctx, [&]() -> int {
    if (!volume || !out) fail(ctx, BM_ERR_INVALID, "null pointer");
    check_phase(ctx, phase);
    const Dims dm = check_dims(ctx, width, height, depth);
    const size_t N = (size_t)dm.n();
    cudaStream_t s = ctx->stream;
    uint8_t* d_in = stage_input(ctx, ctx->in_a, volume, N, s);
    float* d_out = static_cast<float*>(ensure(ctx, ctx->outmap, N * 4, "output"));
    uint32_t* d_sq = squared_thickness ? static_cast<uint32_t*>(ensure(ctx, ctx->fillmap, N * 4, "output")) : nullptr;
    lt_device_impl(ctx, d_in, dm, phase, d_out, d_sq, s);
    check(ctx, cudaMemcpyAsync(out, d_out, N * 4, cudaMemcpyDeviceToHost, s), "result download");
    if (squared_thickness)
      check(ctx, cudaMemcpyAsync(squared_thickness, d_sq, N * 4, cudaMemcpyDeviceToHost, s), "result download");
    check(ctx, cudaStreamSynchronize(s), "result download");
    return BM_OK;
  });
}

int bm_nonzero_stats_device(bm_ctx* ctx, const float* d_values, size_t n, double scale, unsigned flags,
                            bm_stats* out, void* stream) {
  return guarded(ctx, [&]() -> int {
    if (!d_values || !out) fail(ctx, BM_ERR_INVALID, "null pointer");
    if (flags & ~(unsigned)BM_FLAG_QUANTILES) fail(ctx, BM_ERR_INVALID, "unknown flags 0x%x", flags);
    cudaStream_t s = pick_stream(ctx, stream);
    StatsAccum* acc = static_cast<StatsAccum*>(ensure(ctx, ctx->accum, sizeof(StatsAccum), "stats"));
    check(ctx, cudaMemsetAsync(acc, 0, sizeof(StatsAccum), s), "memset");
    timed(ctx, KF_QUANTILE, s, "moments kernel",
          [&] { return launch_moments(d_values, (long long)n, (float)scale, acc, s, &ctx->launches); });
    ordered_sums(ctx, d_values, (long long)n, (float)scale, acc, s);
    StatsAccum ha;
    double osum[2];
    check(ctx, cudaMemcpyAsync(&ha, acc, sizeof ha, cudaMemcpyDeviceToHost, s), "stats readback");
    check(ctx, cudaMemcpyAsync(osum, ctx->ordout.ptr, sizeof osum, cudaMemcpyDeviceToHost, s), "stats readback");
    check(ctx, cudaStreamSynchronize(s), "moments kernel");
    int st = finish_stats(ctx, ha, osum, out);
    if (st) return st;
    if (flags & BM_FLAG_QUANTILES) quantiles(ctx, d_values, (long long)n, ha.count, scale, out, s);
    return BM_OK;
  });
}

int bm_nonzero_stats(bm_ctx* ctx, const float* values, size_t n, double scale, unsigned flags, bm_stats* out) {
  return guarded(ctx, [&]() -> int {
    if (!values || !out) fail(ctx, BM_ERR_INVALID, "null pointer");
    if (flags & ~(unsigned)BM_FLAG_QUANTILES) fail(ctx, BM_ERR_INVALID, "unknown flags 0x%x", flags);
    cudaStream_t s = ctx->stream;
    float* d = static_cast<float*>(ensure(ctx, ctx->qmap, (n ? n : 1) * 4, "values"));
    if (n) check(ctx, cudaMemcpyAsync(d, values, n * 4, cudaMemcpyHostToDevice, s), "values upload");
    StatsAccum* acc = static_cast<StatsAccum*>(ensure(ctx, ctx->accum, sizeof(StatsAccum), "stats"));
    check(ctx, cudaMemsetAsync(acc, 0, sizeof(StatsAccum), s), "memset");
    timed(ctx, KF_QUANTILE, s, "moments kernel",
          [&] { return launch_moments(d, (long long)n, (float)scale, acc, s, &ctx->launches); });
    ordered_sums(ctx, d, (long long)n, (float)scale, acc, s);
    StatsAccum ha;
    double osum[2];
    check(ctx, cudaMemcpyAsync(&ha, acc, sizeof ha, cudaMemcpyDeviceToHost, s), "stats readback");
    check(ctx, cudaMemcpyAsync(osum, ctx->ordout.ptr, sizeof osum, cudaMemcpyDeviceToHost, s), "stats readback");
    check(ctx, cudaStreamSynchronize(s), "moments kernel");
    int st = finish_stats(ctx, ha, osum, out);
    if (st) return st;
    if (flags & BM_FLAG_QUANTILES) quantiles(ctx, d, (long long)n, ha.count, scale, out, s);
    return BM_OK;
  });
}

int bm_volume_metrics_device(bm_ctx* ctx, const uint8_t* d_bone, const uint8_t* d_roi, size_t width, size_t height,
                             size_t depth, const double spacing_um[3], bm_volume_metrics* out, void* stream) {
  return guarded(ctx, [&]() -> int {
    if (!d_bone || !d_roi || !spacing_um || !out) fail(ctx, BM_ERR_INVALID, "null pointer");
    const Dims dm = check_dims(ctx, width, height, depth);
    return volume_metrics_impl(ctx, d_bone, d_roi, dm, spacing_um, out, pick_stream(ctx, stream));
  });
}

int bm_volume_metrics_compute(bm_ctx* ctx, const uint8_t* bone, const uint8_t* roi, size_t width, size_t height,
                              size_t depth, const double spacing_um[3], bm_volume_metrics* out) {
  return guarded(ctx, [&]() -> int {
    if (!bone || !roi || !spacing_um || !out) fail(ctx, BM_ERR_INVALID, "null pointer");
    const Dims dm = check_dims(ctx, width, height, depth);
    const size_t N = (size_t)dm.n();
    cudaStream_t s = ctx->stream;
    const uint8_t* d_bone = stage_input(ctx, ctx->in_a, bone, N, s);
    const uint8_t* d_roi = stage_input(ctx, ctx->in_b, roi, N, s);
    return volume_metrics_impl(ctx, d_bone, d_roi, dm, spacing_um, out, s);
  });
}

int bm_tbth_tbsp_device(bm_ctx* ctx, const uint8_t* d_bone, const uint8_t* d_roi, size_t width, size_t height,
                        size_t depth, double spacing_um, unsigned flags, bm_stats* thickness, bm_stats* spacing,
                        float* d_thickness_map, float* d_spacing_map, void* stream) {
  return guarded(ctx, [&]() -> int {
    if (!d_bone || !d_roi) fail(ctx, BM_ERR_INVALID, "null pointer");
    const Dims dm = check_dims(ctx, width, height, depth);
    return tbth_device_impl(ctx, d_bone, d_roi, dm, spacing_um, flags, thickness, spacing, d_thickness_map,
                            d_spacing_map, pick_stream(ctx, stream));
  });
}

int bm_tbth_tbsp(bm_ctx* ctx, const uint8_t* bone, const uint8_t* roi, size_t width, size_t height, size_t depth,
                 double spacing_um, unsigned flags, bm_stats* thickness, bm_stats* spacing, float* thickness_map,
                 float* spacing_map) {
  return guarded(ctx, [&]() -> int {
    if (!bone || !roi) fail(ctx, BM_ERR_INVALID, "null pointer");
    const Dims dm = check_dims(ctx, width, height, depth);
    const size_t N = (size_t)dm.n();
    cudaStream_t s = ctx->stream;
    float* d_th = thickness_map ? static_cast<float*>(ensure(ctx, ctx->outmap, N * 4, "output")) : nullptr;
    float* d_sp = spacing_map ? static_cast<float*>(ensure(ctx, ctx->outmap2, N * 4, "output")) : nullptr;
    int st;
    if ((long long)N >= kPipeMinVoxels) {
      st = tbth_host_pipelined(ctx, bone, roi, dm, spacing_um, flags, thickness, spacing, d_th, d_sp, s);
    } else {
      const uint8_t* d_bone = stage_input(ctx, ctx->in_a, bone, N, s);
      const uint8_t* d_roi = stage_input(ctx, ctx->in_b, roi, N, s);
      st = tbth_device_impl(ctx, d_bone, d_roi, dm, spacing_um, flags, thickness, spacing, d_th, d_sp, s);
    }
    if (st) return st;
    if (thickness_map)
      check(ctx, cudaMemcpyAsync(thickness_map, d_th, N * 4, cudaMemcpyDeviceToHost, s), "result download");
    if (spacing_map)
      check(ctx, cudaMemcpyAsync(spacing_map, d_sp, N * 4, cudaMemcpyDeviceToHost, s), "result download");
    check(ctx, cudaStreamSynchronize(s), "result download");
    return BM_OK;
  });
}

}  // extern "C"
