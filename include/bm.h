/*
 * bm.h -- C ABI of the GB300 (sm_103a) Tb.Th / Tb.Sp library.
 *
 * This is the drop-in boundary for the trabecular thickness / separation
 * path of bone-morphometry v0.7.0-rc.3 (Rust).  Every entry point is plain C:
 * pointers, sizes and status codes, no CUDA or C++ types.  A Rust caller
 * binds it with an extern "C" block and re-implements the two module
 * functions (edt.rs:57-60, local_thickness.rs:16) on top of it.
 *
 * Volumes use the reference layout (volume.rs:44-46): index = (z*height + y)*width + x,
 * x fastest, one byte per voxel.  Host-pointer entry points copy inputs to the
 * device and results back; *_device entry points take device pointers and a
 * cudaStream_t passed as void* (NULL = the context's own stream) and return
 * once the results are complete (stream synchronised).
 *
 * Errors follow the reference's bails (anyhow::bail!); bm_last_error() returns
 * the reference's message text for the last failing call on the context.
 *
 * Thread safety: a context serialises its calls with an internal mutex; use
 * one context per host thread for concurrency.  There is no CPU fallback: with
 * no usable GPU, bm_ctx_create fails with BM_ERR_NO_DEVICE.
 */
#ifndef BM_H
#define BM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BM_ABI_VERSION 2

typedef enum bm_status {
  BM_OK = 0,
  BM_ERR_ALL_SELECTED = 1, /* edt.rs:61-66: EDT of an all-selected volume              */
  BM_ERR_DIMS = 2,         /* volume.rs:12-34: a dimension < 2, or size overflow        */
  BM_ERR_OOM = 3,          /* device allocation failed                                   */
  BM_ERR_CUDA = 4,         /* any other CUDA runtime error                                */
  BM_ERR_TIMEOUT = 5,      /* a bounded device-side wait ran out                         */
  BM_ERR_INVALID = 6,      /* null pointer, bad phase / flag, shape mismatch (metrics.rs:79-89) */
  BM_ERR_EMPTY = 7,        /* metrics.rs:228-230: no finite positive map value           */
  BM_ERR_ROI_EMPTY = 8,    /* metrics.rs:90-92: ROI has no included voxel                */
  BM_ERR_NO_BONE = 9,      /* metrics.rs:99-101                                           */
  BM_ERR_NO_MARROW = 10,   /* metrics.rs:102-104                                          */
  BM_ERR_NO_DEVICE = 11,   /* no CUDA device / driver                                    */
  BM_ERR_SPACING = 12,     /* metrics.rs:70-78: spacing not finite and positive          */
  BM_ERR_ROI_FULL = 13,    /* metrics.rs:93-95: BoneJ mode needs inside and outside voxels */
  BM_ERR_BUSY = 14         /* server queue full / over budget (serving only)             */
} bm_status;

/* edt.rs:8-24 -- Foreground selects value != 0, Background selects value == 0. */
typedef enum bm_phase { BM_PHASE_FOREGROUND = 0, BM_PHASE_BACKGROUND = 1 } bm_phase;

/* metrics.rs:27-38 (DistributionStats), in micrometres.  Quantile fields are
 * NaN unless BM_FLAG_QUANTILES was given (metrics.rs:242-255); then
 * interquartile_range = p75 - p25 and coefficient_of_variation = sd / mean.
 * sum and sum_of_squares are the reference's own f64 accumulators
 * (metrics.rs:215-224: the scaled f32 values added one after the other in
 * index order, one rounding per value), reproduced bit for bit; mean and
 * standard_deviation follow from them with the reference's formulas
 * (metrics.rs:232-241).  exact_sum and exact_sum_of_squares are the same sums
 * computed exactly and rounded once to f64 (no counterpart in the reference). */
typedef struct bm_stats {
  uint64_t count;
  double mean;
  double standard_deviation;
  double maximum;
  double median;
  double percentile_10;
  double percentile_25;
  double percentile_75;
  double percentile_90;
  double interquartile_range;
  double coefficient_of_variation;
  double sum;
  double sum_of_squares;
  double exact_sum;
  double exact_sum_of_squares;
} bm_stats;

/* Flags for bm_tbth_tbsp*. */
#define BM_FLAG_QUANTILES 1u  /* also compute median / P10 / P25 / P75 / P90 (Standard, Experimental modes) */
#define BM_FLAG_BONEJ_ROI 2u  /* metrics.rs:93-95: reject an ROI without outside voxels      */

typedef struct bm_ctx bm_ctx;

/* Create a context on CUDA device `device` (its own stream, cached device
 * buffers, the cached search-template table). */
int bm_ctx_create(int device, bm_ctx** out);
void bm_ctx_destroy(bm_ctx* ctx);

/* Human-readable name of a status code (static string). */
const char* bm_status_string(int status);

/* Copy the last error message of `ctx` into buf (NUL-terminated, truncated to
 * len); returns the full message length.  ctx may be NULL for errors raised
 * by bm_ctx_create and bm_edt_sq_device_noalloc (per host thread). */
size_t bm_last_error(const bm_ctx* ctx, char* buf, size_t len);

/* Release every cached device buffer of the context (kept otherwise, grown on
 * demand, so repeated calls of one shape allocate nothing). */
int bm_ctx_trim(bm_ctx* ctx);

/* Exact squared Euclidean distance transform of the selected phase.
 * Replaces edt.rs:57-60 `euclidean_distance_transform_squared(&BinaryVolume,
 * Phase) -> Result<Vec<u32>>`: out[i] = squared distance (voxel units) from a
 * selected voxel's centre to the nearest non-selected voxel centre, 0 for
 * non-selected voxels; no exterior halo.  BM_ERR_ALL_SELECTED when every voxel
 * is selected; BM_ERR_DIMS when a dimension is < 2 (volume.rs:27-34). */
int bm_edt_sq(bm_ctx* ctx, const uint8_t* volume, size_t width, size_t height, size_t depth,
              int phase, uint32_t* out);

/* Local thickness map in voxel units (diameters).
 * Replaces local_thickness.rs:16 `local_thickness(&BinaryVolume, Phase) ->
 * Result<Vec<f32>>`.  out[i] is 0 for non-selected voxels.  When
 * squared_thickness is not NULL it receives the propagated squared-thickness
 * map (u32 r^2 before the square root, unmasked; local_thickness.rs:169-202). */
int bm_local_thickness(bm_ctx* ctx, const uint8_t* volume, size_t width, size_t height,
                       size_t depth, int phase, float* out, uint32_t* squared_thickness);

/* Tb.Th and Tb.Sp of one specimen.  Replaces the hot block of
 * metrics.rs:64-121 (`analyze`): validity bails, phase_inside for bone and
 * marrow (volume.rs:84-105), local_thickness of each (metrics.rs:111,119) and
 * nonzero_stats scaled by spacing (metrics.rs:112-116,120).  bone and roi are
 * binary (any non-zero value counts).  thickness_map / spacing_map may be NULL;
 * otherwise they receive the masked f32 diameter maps in voxel units. */
int bm_tbth_tbsp(bm_ctx* ctx, const uint8_t* bone, const uint8_t* roi, size_t width, size_t height,
                 size_t depth, double spacing_um, unsigned flags, bm_stats* thickness,
                 bm_stats* spacing, float* thickness_map, float* spacing_map);

/* nonzero_stats of a map of n f32 values (metrics.rs:204-269): over the finite
 * positive values, v = (raw * (float)scale) as f64; mean / SD / max from exact
 * sums; with BM_FLAG_QUANTILES also median, P10, P25, P75, P90 (numpy-linear
 * interpolation of exact order statistics) and IQR.  BM_ERR_EMPTY when no
 * value is finite and positive (metrics.rs:228-230). */
int bm_nonzero_stats(bm_ctx* ctx, const float* values, size_t n, double scale, unsigned flags,
                     bm_stats* out);
int bm_nonzero_stats_device(bm_ctx* ctx, const float* d_values, size_t n, double scale, unsigned flags,
                            bm_stats* out, void* stream);

/* Bone volume block of `analyze` (metrics.rs:123-132, 166-202): with the
 * ROI-clipped bone (bone != 0 && roi != 0) and voxel volume s0*s1*s2,
 * bone_volume = bone voxels * voxel volume, total_volume = ROI voxels * voxel
 * volume, bone_volume_fraction = their ratio, and roi_boundary_bone_fraction =
 * share of ROI-clipped bone voxels with a 6-neighbour outside the volume or
 * outside the ROI (NaN without bone). */
typedef struct bm_volume_metrics {
  uint64_t bone_voxels;
  uint64_t roi_voxels;
  uint64_t boundary_bone_voxels;
  double bone_volume;
  double total_volume;
  double bone_volume_fraction;
  double roi_boundary_bone_fraction;
} bm_volume_metrics;

int bm_volume_metrics_compute(bm_ctx* ctx, const uint8_t* bone, const uint8_t* roi, size_t width, size_t height,
                              size_t depth, const double spacing_um[3], bm_volume_metrics* out);
int bm_volume_metrics_device(bm_ctx* ctx, const uint8_t* d_bone, const uint8_t* d_roi, size_t width,
                             size_t height, size_t depth, const double spacing_um[3], bm_volume_metrics* out,
                             void* stream);

/* Device-pointer variants (inputs and outputs in device memory). */
int bm_edt_sq_device(bm_ctx* ctx, const uint8_t* d_volume, size_t width, size_t height,
                     size_t depth, int phase, uint32_t* d_out, void* stream);
int bm_local_thickness_device(bm_ctx* ctx, const uint8_t* d_volume, size_t width, size_t height,
                              size_t depth, int phase, float* d_out, uint32_t* d_squared_thickness,
                              void* stream);
int bm_tbth_tbsp_device(bm_ctx* ctx, const uint8_t* d_bone, const uint8_t* d_roi, size_t width,
                        size_t height, size_t depth, double spacing_um, unsigned flags,
                        bm_stats* thickness, bm_stats* spacing, float* d_thickness_map,
                        float* d_spacing_map, void* stream);

/* The exact squared EDT of bm_edt_sq_device without any device allocation.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc (a fixed device-memory budget owned by their own allocator, a
 * footprint that must not grow after start-up, an embedding whose allocator
 * they do not control).  Takes no context; all scratch lives in one static
 * device array of 32 MiB held by every GPU that loads the library until the
 * process exits, so volumes of up to about 2.7 million voxels (128^3 fits)
 * are accepted and larger ones rejected with BM_ERR_DIMS.  Every call looks
 * up the array's device address on the current device (cudaGetSymbolAddress,
 * which allocates nothing), so the address stays right after a
 * cudaDeviceReset; the first call on a device also loads the library's device
 * code there (lazy module loading): make it before any stream capture.  All
 * calls share the array and
 * leave their data in it (the counters that must start at zero are cleared on
 * each call); calls that overlap on the GPU race and must be serialised by the
 * caller.  stream NULL = the legacy default stream; the call returns after
 * synchronising it.  Errors: bm_last_error(NULL, ...). */
int bm_edt_sq_device_noalloc(const uint8_t* d_volume, size_t width, size_t height, size_t depth,
                             int phase, uint32_t* d_out, void* stream);

/* ---- batched and served forms --------------------------------------------
 * A specimen for the batch and the server: bone and roi are host or device
 * pointers (see the call), spacing in micrometres.  The buffers must stay
 * valid until the call (batch) or the ticket (server) completes. */
typedef struct bm_specimen {
  const uint8_t* bone;
  const uint8_t* roi;
  size_t width, height, depth;
  double spacing_um;
} bm_specimen;

/* Tb.Th / Tb.Sp of n specimens of uneven sizes.  The context's worker pool
 * (bm_ctx_set_workers; by default 4 workers, each with its own stream and
 * buffers) takes specimens as workers free up, so their kernels overlap on the
 * GPU.  The workers take the context's site method, fill tile rows and phase
 * scheduling (bm_ctx_set_site_method, bm_ctx_set_fill_tile_rows,
 * bm_ctx_set_concurrent_phases; the pool is recreated when they change).  Per-specimen results and statuses go to thickness[i],
 * spacing[i], status[i]; the call returns BM_OK when every specimen succeeded,
 * else the first non-zero status (the others still complete).
 * device_pointers != 0: bone/roi are device pointers on the context's device. */
int bm_batch_tbth_tbsp(bm_ctx* ctx, const bm_specimen* items, size_t n, int device_pointers, unsigned flags,
                       bm_stats* thickness, bm_stats* spacing, int* status);
/* Set the number of workers of the context's pool (1..64; recreates the pool
 * when the count changes). */
int bm_ctx_set_workers(bm_ctx* ctx, int workers);

/* Request server: submitted specimens (host pointers) are admitted in arrival
 * order while the estimated device footprint of the requests in flight stays
 * within hbm_budget_bytes and a worker is free; admitted requests run
 * concurrently on the workers' streams (continuous batching: a request that
 * arrives while others run starts as soon as a worker and budget free up).
 * Results carry per-request timestamps for latency percentiles. */
typedef struct bm_server bm_server;
typedef struct bm_result {
  int status;
  bm_stats thickness;
  bm_stats spacing;
  double submit_s, start_s, end_s; /* seconds on a steady clock */
  uint64_t footprint_bytes;
  char message[256];               /* error text when status != BM_OK */
} bm_result;
int bm_server_create(int device, int workers, double hbm_budget_bytes, bm_server** out);
/* BM_ERR_BUSY if the request alone exceeds the budget. */
int bm_server_submit(bm_server* srv, const bm_specimen* item, unsigned flags, uint64_t* ticket);
/* A request read from TIFF stacks on the worker (bm_tiff_read semantics): the
 * bone stack (threshold, strict 0/255 check when strict_binary != 0) and the
 * ROI stack (0/1/255; roi_path NULL = every voxel in the ROI, as the reference
 * does without an ROI directory) are decoded straight into the worker's
 * page-locked buffers and copied to the GPU from there.  The stacks' headers
 * are read at submission to size the request; decoding errors come back in
 * the result (status and message). */
int bm_server_submit_tiff(bm_server* srv, const char* bone_path, const char* roi_path, unsigned threshold,
                          int strict_binary, double spacing_um, unsigned flags, uint64_t* ticket);
/* wait != 0: block until the ticket completes; else BM_ERR_BUSY while pending.
 * A completed ticket's result is returned once and then forgotten. */
int bm_server_poll(bm_server* srv, uint64_t ticket, int wait, bm_result* out);
/* Requests waiting for admission, requests running, bytes in flight. */
int bm_server_stats(bm_server* srv, uint64_t* queued, uint64_t* running, double* bytes_in_flight);
void bm_server_destroy(bm_server* srv);
/* Estimated device bytes one specimen of n voxels occupies while it runs. */
uint64_t bm_footprint_bytes(size_t width, size_t height, size_t depth);

/* ---- TIFF stacks ----------------------------------------------------------
 * Reads a multi-page 8-bit grayscale TIFF as the reference's
 * read_binary_tiff / read_roi_tiff do (tiff_io.rs:19-149): every page Gray(8)
 * with the first page's dimensions; samples validated per `accepted`
 * (BM_TIFF_ANY, BM_TIFF_ZERO_OR_255 = the strict-binary check,
 * BM_TIFF_ROI_MASK = 0/1/255) and stored as (sample > threshold) ? 1 : 0,
 * page after page (z), row after row (y), x fastest.  Uncompressed, PackBits,
 * LZW and Deflate data, with or without horizontal differencing, strips or
 * tiles, classic TIFF or BigTIFF, either byte order.  Pages are decoded in
 * parallel straight into `out` (pass pinned host memory to copy it to the GPU
 * without staging).  out == NULL: only the dimensions, of the pages before the
 * first page that fails a structure check (page type, size); the decoding
 * call reports that failure after validating the earlier pages' samples, in
 * the reference's order.  Errors carry the reference's messages; read them with
 * bm_last_error(NULL, ...).  BM_ERR_DIMS when a dimension is < 2
 * (volume.rs:27-34). */
enum { BM_TIFF_ANY = 0, BM_TIFF_ZERO_OR_255 = 1, BM_TIFF_ROI_MASK = 2 };
int bm_tiff_read(const char* path, unsigned threshold, int accepted, uint8_t* out, size_t capacity,
                 size_t* width, size_t* height, size_t* depth);

/* Tb.Th and Tb.Sp of bm_tbth_tbsp run side by side by default for volumes of
 * up to 2^28 voxels: the marrow phase on a second internal context (its own
 * stream and buffers, about doubling the per-phase device memory) while the
 * bone phase runs; larger volumes fill the GPU with one phase and run them one
 * after the other.  on == 0 always runs them one after the other on this
 * context (each kernel then has the GPU to itself, e.g. to time kernels
 * alone).  Results are identical either way. */
int bm_ctx_set_concurrent_phases(bm_ctx* ctx, int on);

/* How the sphere fill finds the non-selected voxels a ridge ball reaches
 * (local_thickness.rs:169-202 paints them too): BM_SITES_SPHERES tests every
 * lattice point of every ridge sphere; BM_SITES_CHAINS pushes the ridge r^2
 * backwards along the distance transform's tied argmins (two window passes
 * over the volume, two more u32 maps of device memory); BM_SITES_AUTO (the
 * default) picks chains when the spheres' lattice points would take the site
 * test more than 0.2 half-warp steps per voxel of the volume.  Results are
 * identical either way. */
enum { BM_SITES_AUTO = 0, BM_SITES_SPHERES = 1, BM_SITES_CHAINS = 2 };
int bm_ctx_set_site_method(bm_ctx* ctx, int method);

/* Rows of y in the sphere fill's tiles (32 x rows x 16 voxels): 0 (the
 * default) picks 64 for volumes of at least 3 * 2^24 voxels (fewer ball
 * entries and plane tests per voxel), 32 from 2^24 voxels and 16 below (more
 * tiles, shorter serial chains); 16, 32 or 64 forces it.  Results are
 * identical either way. */
int bm_ctx_set_fill_tile_rows(bm_ctx* ctx, int rows);

/* Cycle limit of the device-side bounded waits of this context's kernels (the
 * TMA-staged y pass waits on its copy's mbarrier): cycles < 0 restores the
 * default (4e9 cycles, about 2 s); 0 makes every first wait give up at once,
 * which exercises the timeout path without a fault: the block records the
 * timeout, waits (with the default bound) for its copy in flight, and the
 * call returns BM_ERR_TIMEOUT with the context still usable.  For tests. */
int bm_ctx_set_wait_cycles(bm_ctx* ctx, long long cycles);

/* Kernel launches issued by this context since creation (library kernels only). */
uint64_t bm_ctx_launch_count(const bm_ctx* ctx);

/* Per-kernel-family device time, measured with CUDA events recorded on the
 * launching stream around every library kernel while profiling is enabled. */
typedef struct bm_kernel_time {
  char name[32];
  uint64_t launches;
  double total_ms;
} bm_kernel_time;

/* Enable (on != 0, clearing previous totals) or disable event timing. */
int bm_profile_enable(bm_ctx* ctx, int on);
/* Synchronise the context's pending work, fold recorded events into totals and
 * copy up to cap families into out; *count receives the number of families. */
int bm_profile_read(bm_ctx* ctx, bm_kernel_time* out, size_t cap, size_t* count);

#ifdef __cplusplus
}
#endif

#endif /* BM_H */
