// Batched and served forms of the Tb.Th / Tb.Sp path (include/bm.h).
//
// A worker pool: each worker is a host thread that owns a bm_ctx (its own CUDA
// stream and buffer cache) and runs whole specimens through the per-specimen
// pipeline.  Several workers keep several specimens in flight, so the kernels
// of one overlap the host synchronisations and the small kernels of another on
// the same GPU.  Admission is FIFO: the head of the queue starts when a worker
// is free and the estimated device footprint of the running specimens plus its
// own stays within the budget.  The arithmetic is the per-specimen path's, so a
// specimen's results do not depend on what else is in flight.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "bm_internal.h"

namespace bm {

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Job {
  bm_specimen sp{};
  unsigned flags = 0;
  bool device = false;
  // TIFF-path request: stacks decoded on the worker (bone_path not empty)
  std::string bone_path, roi_path;
  unsigned threshold = 0;
  bool strict = false;
  uint64_t id = 0;
  uint64_t bytes = 0;
  bm_result res{};
  bool done = false;
};

// A worker's page-locked staging for TIFF-path requests (grown on demand).
struct PinnedStage {
  uint8_t* p = nullptr;
  size_t n = 0;
  ~PinnedStage() {
    if (p) cudaFreeHost(p);
  }
  uint8_t* get(size_t bytes) {
    if (bytes <= n) return p;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    if (cudaHostAlloc(reinterpret_cast<void**>(&p), bytes, cudaHostAllocDefault) != cudaSuccess) {
      p = nullptr;
      return nullptr;
    }
    n = bytes;
    return p;
  }
};

void copy_message(bm_result& r, const char* msg) {
  std::strncpy(r.message, msg ? msg : "", sizeof r.message - 1);
  r.message[sizeof r.message - 1] = 0;
}

}  // namespace

// Settings every worker context takes from the pool (no effect on results).
struct PoolSettings {
  int site_method = BM_SITES_AUTO;
  int fill_rows = 0;
  bool split_phases = true;
  bool operator==(const PoolSettings& o) const {
    return site_method == o.site_method && fill_rows == o.fill_rows && split_phases == o.split_phases;
  }
};

class Pool {
 public:
  Pool(int device, int workers, double budget, PoolSettings settings)
      : device_(device), budget_(budget), settings_(settings) {
    for (int i = 0; i < workers; ++i) {
      bm_ctx* c = nullptr;
      const int st = bm_ctx_create(device, &c);
      if (st != BM_OK) {
        status_ = st;
        break;
      }
      c->site_method = settings.site_method;
      c->fill_rows = settings.fill_rows;
      c->split_phases = settings.split_phases;
      ctxs_.push_back(c);
    }
    if (status_ == BM_OK)
      for (size_t i = 0; i < ctxs_.size(); ++i) threads_.emplace_back([this, i] { worker_main((int)i); });
  }

  ~Pool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_work_.notify_all();
    for (auto& t : threads_) t.join();
    for (bm_ctx* c : ctxs_) bm_ctx_destroy(c);
  }

  int status() const { return status_; }
  double budget() const { return budget_; }
  const PoolSettings& settings() const { return settings_; }

  void submit(Job* j) {
    {
      std::lock_guard<std::mutex> lk(mu_);
      j->res.submit_s = now_s();
      queue_.push_back(j);
    }
    cv_work_.notify_all();
  }

  void wait(Job* j) {
    std::unique_lock<std::mutex> lk(mu_);
    cv_done_.wait(lk, [&] { return j->done; });
  }

  bool is_done(Job* j) {
    std::lock_guard<std::mutex> lk(mu_);
    return j->done;
  }

  void counters(uint64_t* queued, uint64_t* running, double* bytes) {
    std::lock_guard<std::mutex> lk(mu_);
    if (queued) *queued = queue_.size();
    if (running) *running = running_;
    if (bytes) *bytes = inflight_;
  }

 private:
  void worker_main(int w) {
    bm_ctx* ctx = ctxs_[w];
    PinnedStage bone_stage, roi_stage;
    for (;;) {
      Job* j = nullptr;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_work_.wait(lk, [&] {
          return stop_ || (!queue_.empty() && (running_ == 0 || inflight_ + (double)queue_.front()->bytes <= budget_));
        });
        if (stop_) return;
        j = queue_.front();
        queue_.pop_front();
        inflight_ += (double)j->bytes;
        ++running_;
        j->res.start_s = now_s();
      }
      run(ctx, j, bone_stage, roi_stage);
      const double job_bytes = (double)j->bytes;
      {
        std::lock_guard<std::mutex> lk(mu_);
        j->res.end_s = now_s();
        j->done = true;
      }
      cv_done_.notify_all();
      // keep idle caches within the budget: drop this worker's buffers when
      // they hold well more than the specimen it just ran needed
      const double cached = (double)cached_bytes(ctx);
      if (cached > 2.0 * job_bytes && cached > budget_ / (double)ctxs_.size()) bm_ctx_trim(ctx);
      {
        std::lock_guard<std::mutex> lk(mu_);
        inflight_ -= job_bytes;
        --running_;
      }
      cv_work_.notify_all();
    }
  }

  static void run(bm_ctx* ctx, Job* j, PinnedStage& bone_stage, PinnedStage& roi_stage) {
    j->res.footprint_bytes = j->bytes;
    if (!j->bone_path.empty()) {
      run_tiff(ctx, j, bone_stage, roi_stage);
      return;
    }
    const bm_specimen& s = j->sp;
    if (j->device)
      j->res.status = bm_tbth_tbsp_device(ctx, s.bone, s.roi, s.width, s.height, s.depth, s.spacing_um, j->flags,
                                          &j->res.thickness, &j->res.spacing, nullptr, nullptr, nullptr);
    else
      j->res.status = bm_tbth_tbsp(ctx, s.bone, s.roi, s.width, s.height, s.depth, s.spacing_um, j->flags,
                                   &j->res.thickness, &j->res.spacing, nullptr, nullptr);
    if (j->res.status != BM_OK) {
      char buf[256];
      bm_last_error(ctx, buf, sizeof buf);
      copy_message(j->res, buf);
    }
  }

  // Decode the stacks into this worker's page-locked buffers, then run the
  // specimen from there (tiff_io.rs:19-31 for the stacks, main.rs for the ROI
  // default: every voxel).
  static void run_tiff(bm_ctx* ctx, Job* j, PinnedStage& bone_stage, PinnedStage& roi_stage) {
    char buf[256];
    size_t w = 0, h = 0, d = 0;
    int st = bm_tiff_read(j->bone_path.c_str(), j->threshold, j->strict ? BM_TIFF_ZERO_OR_255 : BM_TIFF_ANY, nullptr,
                          0, &w, &h, &d);
    const size_t n = w * h * d;
    uint8_t* bone = nullptr;
    uint8_t* roi = nullptr;
    if (st == BM_OK) {
      bone = bone_stage.get(n);
      roi = roi_stage.get(n);
      if (!bone || !roi) {
        j->res.status = BM_ERR_OOM;
        copy_message(j->res, "page-locked staging allocation failed");
        return;
      }
      st = bm_tiff_read(j->bone_path.c_str(), j->threshold, j->strict ? BM_TIFF_ZERO_OR_255 : BM_TIFF_ANY, bone, n,
                        &w, &h, &d);
    }
    if (st == BM_OK) {
      if (j->roi_path.empty()) {
        std::memset(roi, 1, n);
      } else {
        size_t rw = 0, rh = 0, rd = 0;
        st = bm_tiff_read(j->roi_path.c_str(), 0, BM_TIFF_ROI_MASK, nullptr, 0, &rw, &rh, &rd);
        if (st == BM_OK && rw == w && rh == h && rd == d)
          st = bm_tiff_read(j->roi_path.c_str(), 0, BM_TIFF_ROI_MASK, roi, n, &rw, &rh, &rd);
        if (st == BM_OK && (rw != w || rh != h || rd != d)) {
          // metrics.rs:79-89
          std::snprintf(buf, sizeof buf, "binary image dimensions %zux%zux%zu do not match ROI dimensions %zux%zux%zu",
                        w, h, d, rw, rh, rd);
          j->res.status = BM_ERR_INVALID;
          copy_message(j->res, buf);
          return;
        }
      }
    }
    if (st != BM_OK) {
      bm_last_error(nullptr, buf, sizeof buf);
      j->res.status = st;
      copy_message(j->res, buf);
      return;
    }
    j->res.status = bm_tbth_tbsp(ctx, bone, roi, w, h, d, j->sp.spacing_um, j->flags, &j->res.thickness,
                                 &j->res.spacing, nullptr, nullptr);
    if (j->res.status != BM_OK) {
      bm_last_error(ctx, buf, sizeof buf);
      copy_message(j->res, buf);
    }
  }

  int device_;
  double budget_;
  PoolSettings settings_;
  int status_ = BM_OK;
  std::vector<bm_ctx*> ctxs_;
  std::vector<std::thread> threads_;
  std::mutex mu_;
  std::condition_variable cv_work_, cv_done_;
  std::deque<Job*> queue_;
  double inflight_ = 0.0;
  uint64_t running_ = 0;
  bool stop_ = false;
};

Pool* pool_create(int device, int workers, double budget, PoolSettings settings, int* status) {
  Pool* p = new Pool(device, workers, budget, settings);
  if (p->status() != BM_OK) {
    *status = p->status();
    delete p;
    return nullptr;
  }
  *status = BM_OK;
  return p;
}

void pool_destroy(Pool* p) { delete p; }

}  // namespace bm

using namespace bm;

struct bm_server {
  std::unique_ptr<Pool> pool;
  std::mutex mu;
  uint64_t next = 1;
  std::unordered_map<uint64_t, std::unique_ptr<Job>> jobs;
};

extern "C" {

uint64_t bm_footprint_bytes(size_t width, size_t height, size_t depth) {
  // per voxel: inputs 2; per phase (the two phases run side by side, each on
  // its own buffers): four u32 maps 16 (x/y pass, z pass, chain map), envelope
  // scratch 8, ridge records <= 8, bin entries ~5, f32 thickness map 4 (read by
  // the statistics' ordered sums, ~0.2 more of their scratch), quantile map 4,
  // bitmasks ~1; tables 2 x 64 MiB
  const uint64_t n = (uint64_t)width * height * depth;
  return n * 95u + (128ull << 20);
}

int bm_ctx_set_workers(bm_ctx* ctx, int workers) {
  if (!ctx || workers < 1 || workers > 64) return BM_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->pool_mu);
  if (workers == ctx->workers) return BM_OK;  // the pool stays (with its grown buffers)
  if (ctx->pool) {
    pool_destroy(ctx->pool);
    ctx->pool = nullptr;
  }
  ctx->workers = workers;
  return BM_OK;
}

int bm_batch_tbth_tbsp(bm_ctx* ctx, const bm_specimen* items, size_t n, int device_pointers, unsigned flags,
                       bm_stats* thickness, bm_stats* spacing, int* status) {
  if (!ctx || (n && !items)) return BM_ERR_INVALID;
  std::lock_guard<std::mutex> lk(ctx->pool_mu);
  // the workers take the context's site method, fill tile rows and phase scheduling
  PoolSettings want;
  want.site_method = ctx->site_method;
  want.fill_rows = ctx->fill_rows;
  want.split_phases = ctx->split_phases;
  if (ctx->pool && !(ctx->pool->settings() == want)) {
    pool_destroy(ctx->pool);
    ctx->pool = nullptr;
  }
  if (!ctx->pool) {
    int st = BM_OK;
    ctx->pool = pool_create(ctx->device, ctx->workers, 1e300, want, &st);
    if (!ctx->pool) return st;
  }
  std::vector<Job> jobs(n);
  for (size_t i = 0; i < n; ++i) {
    jobs[i].sp = items[i];
    jobs[i].flags = flags;
    jobs[i].device = device_pointers != 0;
    jobs[i].id = i;
    jobs[i].bytes = bm_footprint_bytes(items[i].width, items[i].height, items[i].depth);
  }
  // largest specimens first: the pool takes them as workers free up, so the
  // batch ends on short ones instead of waiting for one large straggler
  std::vector<size_t> order(n);
  for (size_t i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
    return items[a].width * items[a].height * items[a].depth > items[b].width * items[b].height * items[b].depth;
  });
  for (size_t i : order) ctx->pool->submit(&jobs[i]);
  int first = BM_OK;
  for (size_t i = 0; i < n; ++i) {
    ctx->pool->wait(&jobs[i]);
    if (thickness) thickness[i] = jobs[i].res.thickness;
    if (spacing) spacing[i] = jobs[i].res.spacing;
    if (status) status[i] = jobs[i].res.status;
    if (first == BM_OK && jobs[i].res.status != BM_OK) first = jobs[i].res.status;
  }
  return first;
}

int bm_server_create(int device, int workers, double hbm_budget_bytes, bm_server** out) {
  if (!out || workers < 1 || workers > 64 || !(hbm_budget_bytes > 0)) return BM_ERR_INVALID;
  *out = nullptr;
  int st = BM_OK;
  Pool* p = pool_create(device, workers, hbm_budget_bytes, PoolSettings{}, &st);
  if (!p) return st;
  bm_server* s = new bm_server();
  s->pool.reset(p);
  *out = s;
  return BM_OK;
}

int bm_server_submit(bm_server* srv, const bm_specimen* item, unsigned flags, uint64_t* ticket) {
  if (!srv || !item || !ticket) return BM_ERR_INVALID;
  auto j = std::make_unique<Job>();
  j->sp = *item;
  j->flags = flags;
  j->device = false;
  j->bytes = bm_footprint_bytes(item->width, item->height, item->depth);
  if ((double)j->bytes > srv->pool->budget()) return BM_ERR_BUSY;
  Job* raw = j.get();
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    j->id = srv->next++;
    *ticket = j->id;
    srv->jobs.emplace(j->id, std::move(j));
  }
  srv->pool->submit(raw);
  return BM_OK;
}

int bm_server_submit_tiff(bm_server* srv, const char* bone_path, const char* roi_path, unsigned threshold,
                          int strict_binary, double spacing_um, unsigned flags, uint64_t* ticket) {
  if (!srv || !bone_path || !ticket || threshold > 255) return BM_ERR_INVALID;
  size_t w = 0, h = 0, d = 0;
  const int st = bm_tiff_read(bone_path, threshold, BM_TIFF_ANY, nullptr, 0, &w, &h, &d);  // headers only
  if (st != BM_OK) return st;
  auto j = std::make_unique<Job>();
  j->bone_path = bone_path;
  if (roi_path) j->roi_path = roi_path;
  j->threshold = threshold;
  j->strict = strict_binary != 0;
  j->sp.width = w;
  j->sp.height = h;
  j->sp.depth = d;
  j->sp.spacing_um = spacing_um;
  j->flags = flags;
  j->bytes = bm_footprint_bytes(w, h, d);
  if ((double)j->bytes > srv->pool->budget()) return BM_ERR_BUSY;
  Job* raw = j.get();
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    j->id = srv->next++;
    *ticket = j->id;
    srv->jobs.emplace(j->id, std::move(j));
  }
  srv->pool->submit(raw);
  return BM_OK;
}

int bm_server_poll(bm_server* srv, uint64_t ticket, int wait, bm_result* out) {
  if (!srv || !out) return BM_ERR_INVALID;
  Job* j = nullptr;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->jobs.find(ticket);
    if (it == srv->jobs.end()) return BM_ERR_INVALID;
    j = it->second.get();
  }
  if (wait) srv->pool->wait(j);
  else if (!srv->pool->is_done(j)) return BM_ERR_BUSY;
  *out = j->res;
  std::lock_guard<std::mutex> lk(srv->mu);
  srv->jobs.erase(ticket);
  return BM_OK;
}

int bm_server_stats(bm_server* srv, uint64_t* queued, uint64_t* running, double* bytes_in_flight) {
  if (!srv) return BM_ERR_INVALID;
  srv->pool->counters(queued, running, bytes_in_flight);
  return BM_OK;
}

void bm_server_destroy(bm_server* srv) { delete srv; }

}  // extern "C"
