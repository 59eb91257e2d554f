// Serving loop (pnm_server_*): a scheduler thread that admits queued extraction requests under a
// device-memory budget, coalesces whatever is queued when a stream slot frees into one batch
// (pnm_batch.cu), runs up to max_inflight batches concurrently on their own streams, and keeps
// each request's results resident until the caller releases it. A batch whose requests are all
// released stays allocated in a small cache keyed by its volume shapes (counted against the
// budget, evicted oldest first): a later group of the same shapes reuses it with new origins and
// spacings instead of allocating again. Served batches enqueue their stages on every run: with
// shapes that repeat only a few times, capturing a graph per shape costs more than it returns.
//
// Locking: `mu` guards the queue, the request table, the group lists and the statistics. The
// scheduler never holds it across a CUDA call that can wait on a stream (batch creation, upload,
// launch, wait, destroy), so user threads that submit, poll or copy out are never held up by a
// running batch. Completion is signalled by a host function enqueued after each batch; it only
// stores a timestamp and a flag (no CUDA calls, no lock) and wakes the scheduler.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "pnm_ctx.h"

namespace {

using Clock = std::chrono::steady_clock;
using pnm::Status;

constexpr int64_t kDefaultBudget = 120ll * 1000 * 1000 * 1000;  // 120 GB
constexpr int kDefaultInflight = 3;
constexpr int kDefaultBatchVolumes = 64;
constexpr int64_t kDefaultBatchVoxels = 1ll << 28;
constexpr int kCacheEntries = 96;   // idle batches kept for reuse
constexpr int kPinBlocks = 512;     // pinned result blocks: running + held + cached batches

struct Group;

struct Request {
  int64_t id = 0;
  const float* sdf = nullptr;
  int32_t dims[3] = {0, 0, 0};  // xyz
  float org[3], spc[3];
  Clock::time_point t_submit, t_done;
  int state = PNM_REQ_QUEUED;
  int status = PNM_OK;
  Group* group = nullptr;
  int index = 0;
  pnm_batch_volume info{};
  long long voxels() const { return (long long)dims[0] * dims[1] * dims[2]; }
};

struct Group {
  pnm_batch* batch = nullptr;
  void* pin = nullptr;              // this batch's pinned block (per-run figures)
  std::vector<int32_t> dims;        // shapes (xyz per volume): the cache key
  std::vector<Request*> reqs;
  int slot = -1;
  int64_t bytes = 0;
  std::atomic<int> gpu_done{0};
  Clock::time_point t_gpu_done;
  Clock::time_point t_launch;
  int live = 0;  // requests not yet released
  bool finished = false;
  bool ok = false;
  struct pnm_server* srv = nullptr;
};

struct Slot {
  cudaStream_t stream = nullptr;
  bool busy = false;
};

struct Cached {
  std::vector<int32_t> dims;
  pnm_batch* batch;
  void* pin;
  int64_t bytes;
};

}  // namespace

struct pnm_server {
  int device = 0;
  int sm_count = 0;
  pnm_server_config cfg{};
  std::vector<Slot> slots;
  cudaStream_t io_stream = nullptr;  // copy-outs of held results
  std::mutex mu;
  std::condition_variable cv_sched, cv_done;
  std::deque<Request*> queue;
  std::unordered_map<int64_t, Request*> reqs;
  std::vector<Group*> running;
  std::list<Cached> cache;          // idle batches, most recently used first
  void* pin_arena = nullptr;        // pinned blocks for the batches' per-run figures
  std::vector<void*> pin_free;
  size_t pin_block = 0;
  int64_t cache_hits = 0;
  int64_t next_id = 1;
  int64_t bytes_in_use = 0, peak_bytes = 0;
  int64_t submitted = 0, completed = 0, failed = 0, cancelled = 0, batches = 0;
  int64_t voxels_done = 0;
  std::vector<double> lat_ms;
  Clock::time_point t_first, t_last;
  bool have_first = false;
  bool stop = false;
  std::thread thr;
  std::string last_error;
};

namespace {

void CUDART_CB on_group_done(void* p) {
  Group* g = static_cast<Group*>(p);
  g->t_gpu_done = Clock::now();
  g->gpu_done.store(1, std::memory_order_release);
  g->srv->cv_sched.notify_all();
}

int64_t plan_bytes(const std::vector<int32_t>& dims) {
  int64_t b = 0;
  if (pnm_batch_plan_bytes((int32_t)(dims.size() / 3), dims.data(), &b) != PNM_OK) return -1;
  return b;
}

// Frees a batch and returns its pinned block (caller holds mu; the CUDA calls do not block).
void drop_batch(pnm_server* s, pnm_batch* b, void* pin) {
  if (b) pnm_batch_destroy(b);
  if (pin) s->pin_free.push_back(pin);
}

// Evicts the least recently used idle batch; false when the cache is empty (caller holds mu).
bool evict_one(pnm_server* s) {
  if (s->cache.empty()) return false;
  Cached& c = s->cache.back();
  s->bytes_in_use -= c.bytes;
  drop_batch(s, c.batch, c.pin);
  s->cache.pop_back();
  return true;
}

// A group whose requests are all released: its batch goes to the cache when it ran cleanly
// (caller holds mu).
void retire_group(pnm_server* s, Group* g, bool ok) {
  if (ok && g->batch) {
    s->cache.push_front(Cached{g->dims, g->batch, g->pin, g->bytes});
    while ((int)s->cache.size() > kCacheEntries) evict_one(s);
  } else {
    s->bytes_in_use -= g->bytes;
    drop_batch(s, g->batch, g->pin);
  }
  delete g;
}

// Completes a finished group: checks the run, records per-request figures and latencies.
void finish_group(pnm_server* s, Group* g, std::unique_lock<std::mutex>& lk) {
  lk.unlock();
  const auto t0 = Clock::now();
  int rc = pnm_batch_wait(g->batch);  // the stream is idle: checks, and re-runs on growth
  const auto t1 = Clock::now();
  std::vector<pnm_batch_volume> infos(g->reqs.size());
  if (rc == PNM_OK)
    for (size_t i = 0; i < g->reqs.size() && rc == PNM_OK; ++i)
      rc = pnm_batch_volume_info(g->batch, (int32_t)i, &infos[i]);
  std::string err = rc == PNM_OK ? "" : pnm_batch_last_error(g->batch);
  lk.lock();
  // a re-run after capacity growth finished later than the first completion signal
  const auto t_done = (t1 - t0) > std::chrono::milliseconds(1) ? t1 : g->t_gpu_done;
  for (size_t i = 0; i < g->reqs.size(); ++i) {
    Request* r = g->reqs[i];
    r->t_done = t_done;
    r->status = rc;
    if (rc == PNM_OK) {
      r->state = PNM_REQ_DONE;
      r->info = infos[i];
      ++s->completed;
      s->voxels_done += r->voxels();
      s->lat_ms.push_back(std::chrono::duration<double, std::milli>(t_done - r->t_submit).count());
    } else {
      r->state = PNM_REQ_FAILED;
      ++s->failed;
    }
  }
  if (rc != PNM_OK) s->last_error = err;
  s->t_last = std::max(s->t_last, t_done);
  g->finished = true;
  g->ok = rc == PNM_OK;
  s->slots[g->slot].busy = false;
  s->running.erase(std::find(s->running.begin(), s->running.end(), g));
  s->cv_done.notify_all();
}

void fail_requests(pnm_server* s, const std::vector<Request*>& rs, int code) {
  for (Request* r : rs) {
    r->state = PNM_REQ_FAILED;
    r->status = code;
    r->group = nullptr;
    ++s->failed;
  }
  s->cv_done.notify_all();
}

// Forms, allocates and launches one batch from the queue head on a free slot. Returns false when
// nothing could be admitted now (budget) so the scheduler waits for completions.
bool admit_one(pnm_server* s, std::unique_lock<std::mutex>& lk) {
  int slot = -1;
  for (size_t i = 0; i < s->slots.size(); ++i)
    if (!s->slots[i].busy) {
      slot = (int)i;
      break;
    }
  if (slot < 0 || s->queue.empty()) return false;
  std::vector<Request*> take;
  std::vector<int32_t> dims;
  int64_t voxels = 0, bytes = 0;
  while (!s->queue.empty() && (int)take.size() < s->cfg.max_batch_volumes) {
    Request* r = s->queue.front();
    if (!take.empty() && voxels + r->voxels() > s->cfg.max_batch_voxels) break;
    dims.insert(dims.end(), r->dims, r->dims + 3);
    const int64_t b = plan_bytes(dims);
    // idle cached batches give their memory back before anything waits for it
    while (b >= 0 && s->bytes_in_use + b > s->cfg.budget_bytes && evict_one(s)) {
    }
    if (b < 0 || s->bytes_in_use + b > s->cfg.budget_bytes) {
      dims.resize(dims.size() - 3);
      if (take.empty()) {
        if (s->bytes_in_use == 0 || b < 0 || b > s->cfg.budget_bytes) {
          // can never fit: refuse it and keep serving the rest
          s->queue.pop_front();
          fail_requests(s, {r}, b < 0 ? PNM_ERR_SHAPE : PNM_ERR_CAPACITY);
          s->last_error = "request exceeds the server's device-memory budget";
          return true;
        }
        return false;  // wait until running batches or held results free memory
      }
      break;
    }
    bytes = b;
    voxels += r->voxels();
    take.push_back(r);
    s->queue.pop_front();
  }
  if (s->pin_free.empty()) {  // every pinned block is held: free idle batches first
    while (s->pin_free.empty() && evict_one(s)) {
    }
    if (s->pin_free.empty()) {  // all held by results not yet released: retry later
      for (auto it = take.rbegin(); it != take.rend(); ++it) s->queue.push_front(*it);
      return false;
    }
  }
  auto* g = new Group();
  g->srv = s;
  g->slot = slot;
  g->dims = dims;
  g->reqs = take;
  // an idle batch of exactly these shapes is reused (its memory is already counted)
  pnm_batch* reuse = nullptr;
  for (auto it = s->cache.begin(); it != s->cache.end(); ++it) {
    if (it->dims == dims) {
      reuse = it->batch;
      g->pin = it->pin;
      g->bytes = it->bytes;
      s->cache.erase(it);
      ++s->cache_hits;
      break;
    }
  }
  if (!reuse) {
    g->pin = s->pin_free.back();
    s->pin_free.pop_back();
    g->bytes = bytes;
    s->bytes_in_use += bytes;
  }
  g->live = (int)take.size();
  for (size_t i = 0; i < take.size(); ++i) {
    take[i]->state = PNM_REQ_RUNNING;
    take[i]->group = g;
    take[i]->index = (int)i;
  }
  s->slots[slot].busy = true;
  s->peak_bytes = std::max(s->peak_bytes, s->bytes_in_use);
  s->running.push_back(g);
  ++s->batches;
  const Slot sl = s->slots[slot];
  lk.unlock();
  // allocation, upload and launch without the lock
  std::vector<float> org, spc;
  for (Request* r : take) {
    org.insert(org.end(), r->org, r->org + 3);
    spc.insert(spc.end(), r->spc, r->spc + 3);
  }
  Status st = reuse ? pnm::batch_rebind(reuse, sl.stream, org.data(), spc.data(), false)
                    : pnm::batch_new(s->device, s->sm_count, sl.stream, g->pin,
                                     PNM_BATCH_NO_GRAPH, (int)take.size(), dims.data(), org.data(),
                                     spc.data(), &g->batch);
  if (reuse) g->batch = reuse;
  int rc = st.code;
  std::string err = st.msg;
  for (size_t i = 0; rc == PNM_OK && i < take.size(); ++i)
    rc = pnm_batch_set_sdf(g->batch, (int32_t)i, take[i]->sdf);
  if (rc == PNM_OK) rc = pnm_batch_launch(g->batch);
  if (rc == PNM_OK && cudaLaunchHostFunc(sl.stream, on_group_done, g) != cudaSuccess) {
    cudaGetLastError();
    rc = PNM_ERR_CUDA;
  }
  if (rc != PNM_OK && g->batch && err.empty()) err = pnm_batch_last_error(g->batch);
  g->t_launch = Clock::now();
  lk.lock();
  if (rc != PNM_OK) {
    s->running.erase(std::find(s->running.begin(), s->running.end(), g));
    s->slots[slot].busy = false;
    fail_requests(s, take, rc);
    s->last_error = err;
    g->reqs.clear();
    lk.unlock();
    if (g->batch) cudaStreamSynchronize(sl.stream);
    lk.lock();
    retire_group(s, g, false);
  }
  return true;
}

void scheduler(pnm_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (true) {
    auto ready = [&] {
      if (s->stop) return true;
      for (Group* g : s->running)
        if (g->gpu_done.load(std::memory_order_acquire)) return true;
      if (!s->queue.empty())
        for (const Slot& sl : s->slots)
          if (!sl.busy) return true;
      return false;
    };
    // completion signals are lock-free, so a short timeout bounds a missed wake-up
    s->cv_sched.wait_for(lk, std::chrono::microseconds(200), ready);
    for (size_t i = 0; i < s->running.size();) {
      Group* g = s->running[i];
      if (g->gpu_done.load(std::memory_order_acquire)) {
        finish_group(s, g, lk);  // erases g from running
        i = 0;
      } else {
        ++i;
      }
    }
    if (s->stop) {
      if (s->running.empty()) break;
      continue;
    }
    while (admit_one(s, lk)) {
    }
  }
}

Request* find(pnm_server* s, int64_t t) {
  auto it = s->reqs.find(t);
  return it == s->reqs.end() ? nullptr : it->second;
}

}  // namespace

extern "C" {

int pnm_server_create(pnm_ctx* ctx, const pnm_server_config* cfg, pnm_server** out) {
  if (!ctx || !out) return PNM_ERR_ARG;
  *out = nullptr;
  auto* s = new (std::nothrow) pnm_server();
  if (!s) return PNM_ERR_INTERNAL;
  if (cfg) s->cfg = *cfg;
  if (s->cfg.budget_bytes <= 0) s->cfg.budget_bytes = kDefaultBudget;
  if (s->cfg.max_inflight <= 0) s->cfg.max_inflight = kDefaultInflight;
  if (s->cfg.max_batch_volumes <= 0) s->cfg.max_batch_volumes = kDefaultBatchVolumes;
  if (s->cfg.max_batch_voxels <= 0) s->cfg.max_batch_voxels = kDefaultBatchVoxels;
  s->device = ctx->c.device;
  s->sm_count = ctx->c.sm_count;
  bool ok = cudaSetDevice(s->device) == cudaSuccess &&
            cudaStreamCreateWithFlags(&s->io_stream, cudaStreamNonBlocking) == cudaSuccess;
  s->slots.resize(s->cfg.max_inflight);
  for (Slot& sl : s->slots)
    ok = ok && cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) == cudaSuccess;
  s->pin_block = (pnm::batch_pinned_bytes(s->cfg.max_batch_volumes) + 255) & ~(size_t)255;
  ok = ok && cudaMallocHost(&s->pin_arena, s->pin_block * kPinBlocks) == cudaSuccess;
  if (ok)
    for (int i = kPinBlocks - 1; i >= 0; --i)
      s->pin_free.push_back(static_cast<char*>(s->pin_arena) + s->pin_block * i);
  if (!ok) {
    cudaGetLastError();
    ctx->c.last_error = "pnm_server_create: stream / pinned allocation failed";
    pnm_server_destroy(s);
    return PNM_ERR_CUDA;
  }
  s->thr = std::thread(scheduler, s);
  *out = s;
  return PNM_OK;
}

void pnm_server_destroy(pnm_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    for (Request* r : s->queue) {
      r->state = PNM_REQ_CANCELLED;
      ++s->cancelled;
    }
    s->queue.clear();
    s->stop = true;
  }
  s->cv_sched.notify_all();
  if (s->thr.joinable()) s->thr.join();
  cudaSetDevice(s->device);
  std::vector<Group*> groups;
  for (auto& kv : s->reqs) {
    Group* g = kv.second->group;
    if (g && std::find(groups.begin(), groups.end(), g) == groups.end()) groups.push_back(g);
    delete kv.second;
  }
  for (Group* g : groups) {
    if (g->batch) pnm_batch_destroy(g->batch);
    delete g;
  }
  for (Cached& c : s->cache) pnm_batch_destroy(c.batch);
  s->cache.clear();
  for (Slot& sl : s->slots) {
    if (sl.stream) {
      cudaStreamSynchronize(sl.stream);
      cudaStreamDestroy(sl.stream);
    }
  }
  if (s->pin_arena) cudaFreeHost(s->pin_arena);
  if (s->io_stream) cudaStreamDestroy(s->io_stream);
  delete s;
}

const char* pnm_server_last_error(const pnm_server* s) { return s ? s->last_error.c_str() : ""; }

int pnm_server_submit(pnm_server* s, const float* sdf, int32_t nx, int32_t ny, int32_t nz,
                      const float origin_xyz[3], const float spacing_xyz[3], int64_t* ticket) {
  if (!s || !ticket || !origin_xyz || !spacing_xyz) return PNM_ERR_ARG;
  *ticket = 0;
  const pnm::Dims d{nx, ny, nz};
  Status st = pnm::check_dims(d, spacing_xyz, true);
  if (st.good() && d.n() > 0 && !sdf) st = Status{PNM_ERR_ARG, "sdf is null"};
  auto* r = new (std::nothrow) Request();
  if (!r) return PNM_ERR_INTERNAL;
  r->sdf = sdf;
  r->dims[0] = nx;
  r->dims[1] = ny;
  r->dims[2] = nz;
  std::memcpy(r->org, origin_xyz, sizeof(r->org));
  std::memcpy(r->spc, spacing_xyz, sizeof(r->spc));
  r->t_submit = Clock::now();
  std::lock_guard<std::mutex> lk(s->mu);
  if (!st.good()) {
    s->last_error = st.msg;
    delete r;
    return st.code;
  }
  r->id = s->next_id++;
  if (!s->have_first) {
    s->t_first = r->t_submit;
    s->t_last = r->t_submit;
    s->have_first = true;
  }
  s->reqs[r->id] = r;
  ++s->submitted;
  s->queue.push_back(r);
  *ticket = r->id;
  s->cv_sched.notify_all();
  return PNM_OK;
}

int pnm_server_state(pnm_server* s, int64_t ticket, int32_t* state, int32_t* status) {
  if (!s) return PNM_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  Request* r = find(s, ticket);
  if (!r) return PNM_ERR_ARG;
  if (state) *state = r->state;
  if (status) *status = r->status;
  return PNM_OK;
}

int pnm_server_wait(pnm_server* s, int64_t ticket, double timeout_s) {
  if (!s) return PNM_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  Request* r = find(s, ticket);
  if (!r) return PNM_ERR_ARG;
  auto done = [&] { return r->state >= PNM_REQ_DONE; };
  if (timeout_s > 0) {
    if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done))
      return PNM_ERR_NOT_CONVERGED;
  } else {
    s->cv_done.wait(lk, done);
  }
  return r->state == PNM_REQ_CANCELLED ? PNM_ERR_ARG : r->status;
}

int pnm_server_cancel(pnm_server* s, int64_t ticket) {
  if (!s) return PNM_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  Request* r = find(s, ticket);
  if (!r || r->state != PNM_REQ_QUEUED) {
    s->last_error = r ? "request is no longer queued (running or finished)" : "unknown ticket";
    return PNM_ERR_ARG;
  }
  s->queue.erase(std::find(s->queue.begin(), s->queue.end(), r));
  r->state = PNM_REQ_CANCELLED;
  ++s->cancelled;
  s->cv_done.notify_all();
  return PNM_OK;
}

int pnm_server_result(pnm_server* s, int64_t ticket, pnm_batch_volume* info, pnm_pore** d_pores,
                      int32_t** d_seg, int32_t** d_pairs) {
  if (!s) return PNM_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  Request* r = find(s, ticket);
  if (!r || r->state != PNM_REQ_DONE) return PNM_ERR_ARG;
  if (info) *info = r->info;
  pnm_pore* p = nullptr;
  int32_t *sg = nullptr, *pr = nullptr;
  if (r->group && r->group->batch) pnm_batch_results_dev(r->group->batch, &p, &sg, &pr);
  if (d_pores) *d_pores = p ? p + r->info.pore_offset : nullptr;
  if (d_seg) *d_seg = sg ? sg + r->info.voxel_offset : nullptr;
  if (d_pairs) *d_pairs = pr ? pr + 2 * r->info.pair_offset : nullptr;
  return PNM_OK;
}

int pnm_server_copy_out(pnm_server* s, int64_t ticket, pnm_pore* pores, int32_t* seg,
                        int32_t* pairs) {
  if (!s) return PNM_ERR_ARG;
  pnm_batch_volume info;
  pnm_pore* dp = nullptr;
  int32_t *ds = nullptr, *dq = nullptr;
  int rc = pnm_server_result(s, ticket, &info, &dp, &ds, &dq);
  if (rc != PNM_OK) return rc;
  // results stay valid until released; only the caller releases, so no lock is needed here
  const long long n = (long long)info.nx * info.ny * info.nz;
  cudaSetDevice(s->device);
  cudaError_t e = cudaSuccess;
  if (pores && info.n_pores && e == cudaSuccess)
    e = cudaMemcpyAsync(pores, dp, info.n_pores * sizeof(pnm_pore), cudaMemcpyDeviceToHost,
                        s->io_stream);
  if (seg && n && e == cudaSuccess)
    e = cudaMemcpyAsync(seg, ds, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s->io_stream);
  if (pairs && info.n_pairs && e == cudaSuccess)
    e = cudaMemcpyAsync(pairs, dq, 2 * info.n_pairs * sizeof(int32_t), cudaMemcpyDeviceToHost,
                        s->io_stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->io_stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    std::lock_guard<std::mutex> lk(s->mu);
    s->last_error = std::string("copy-out: ") + cudaGetErrorString(e);
    return PNM_ERR_CUDA;
  }
  return PNM_OK;
}

int pnm_server_release(pnm_server* s, int64_t ticket) {
  if (!s) return PNM_ERR_ARG;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    Request* r = find(s, ticket);
    if (!r || (r->state != PNM_REQ_DONE && r->state != PNM_REQ_FAILED &&
               r->state != PNM_REQ_CANCELLED))
      return PNM_ERR_ARG;
    Group* g = r->group;
    s->reqs.erase(ticket);
    delete r;
    if (g && --g->live == 0 && g->finished) retire_group(s, g, g->ok);
    s->cv_sched.notify_all();  // memory may have freed up for queued requests
  }
  return PNM_OK;
}

int pnm_server_get_stats(pnm_server* s, pnm_server_stats* out) {
  if (!s || !out) return PNM_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  std::memset(out, 0, sizeof(*out));
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->failed = s->failed;
  out->cancelled = s->cancelled;
  out->queued = (int64_t)s->queue.size();
  for (Group* g : s->running) out->running += (int64_t)g->reqs.size();
  out->batches = s->batches;
  out->bytes_in_use = s->bytes_in_use;
  out->peak_bytes = s->peak_bytes;
  out->voxels_completed = s->voxels_done;
  if (!s->lat_ms.empty()) {
    std::vector<double> v = s->lat_ms;
    std::sort(v.begin(), v.end());
    auto q = [&](double f) {
      const size_t i = (size_t)std::min<double>((double)v.size() - 1, f * (double)(v.size() - 1) + 0.5);
      return v[i];
    };
    out->p50_ms = q(0.50);
    out->p99_ms = q(0.99);
    double sum = 0;
    for (double x : v) sum += x;
    out->mean_ms = sum / (double)v.size();
    out->max_ms = v.back();
  }
  out->cache_hits = s->cache_hits;
  out->cached = (int64_t)s->cache.size();
  if (s->have_first) {
    out->busy_s = std::chrono::duration<double>(s->t_last - s->t_first).count();
    if (out->busy_s > 0) out->gvoxel_per_s = (double)s->voxels_done / out->busy_s / 1e9;
  }
  return PNM_OK;
}

int pnm_server_reset_stats(pnm_server* s) {
  if (!s) return PNM_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  s->submitted = s->completed = s->failed = s->cancelled = s->batches = s->cache_hits = 0;
  s->voxels_done = 0;
  s->peak_bytes = s->bytes_in_use;
  s->lat_ms.clear();
  s->have_first = false;
  return PNM_OK;
}

}  // extern "C"
