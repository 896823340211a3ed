// Serving loop: continuous admission of independent siting jobs under an HBM
// budget (no counterpart in the reference, which runs one process per DEM).
//
// Jobs queue in arrival order.  One worker thread owns the context and keeps
// up to max_jobs jobs in flight on the GPU at once: the head of the queue is
// admitted as soon as its workspace (plan_batch of the job alone, host
// arithmetic only) fits in the free part of the server's device arena, a
// region of hbm_budget bytes, and its host staging fits the pinned arena.
// An admitted job's stages (upload, VIX, FINDMAX, VIEWSHED) run on one of six
// stage streams: two per size tier (up to 1M cells, up to 4M, larger), the
// smaller tiers at higher stream priority, so that the block scheduler gives
// a small job's CTAs the SMs as soon as a large job's running CTAs end (a
// small job need not wait for a large one's stages; results do not depend on
// the order).  A host callback at their end hands the job back to the
// worker, which then enqueues its greedy selection on the SITE stream
// (highest priority, one cooperative launch a job), so selections run in the
// order their stages finish; a second callback at the end of the selection
// and readback tells the worker the job is done, and the worker copies its
// results out and frees its memory.  So a request that arrives while
// others are on the GPU starts at once if memory and a slot are free, and its
// kernels overlap theirs on the device.  A job whose own workspace exceeds
// the budget is refused when it is submitted, so the queue never blocks on
// it.  Results never depend on what else is in flight: each job has its own
// buffers and the same kernels as siting_run.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "batch.h"
#include "ctx.h"
#include "siting.h"

using namespace siting;

namespace {

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// First-fit allocator over [0, size) with coalescing of freed ranges.
class RangeAlloc {
 public:
  void reset(size_t size) {
    free_.clear();
    if (size) free_[0] = size;
    used_ = 0;
  }
  bool alloc(size_t bytes, size_t *off) {
    bytes = align256(std::max<size_t>(bytes, 1));
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < bytes) continue;
      *off = it->first;
      const size_t rest = it->second - bytes, start = it->first + bytes;
      free_.erase(it);
      if (rest) free_[start] = rest;
      used_ += bytes;
      return true;
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = align256(std::max<size_t>(bytes, 1));
    used_ -= bytes;
    auto next = free_.lower_bound(off);
    size_t start = off, len = bytes;
    if (next != free_.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == off) {
        start = prev->first;
        len += prev->second;
        free_.erase(prev);
      }
    }
    if (next != free_.end() && off + bytes == next->first) {
      len += next->second;
      free_.erase(next);
    }
    free_[start] = len;
  }
  size_t used() const { return used_; }

 private:
  std::map<size_t, size_t> free_;
  size_t used_ = 0;
};

struct Request {
  siting_params p;
  const uint16_t *elevs;
  int pitch;
  int32_t *obs;
  uint8_t *sel;
  siting_job_info info;
  size_t ws = 0;          // device workspace of the job alone
  size_t pin = 0;         // pinned host staging of the job
  bool done = false;
  // while in flight
  BatchPlan plan;
  size_t d_off = 0, h_off = 0;
  cudaEvent_t staged = nullptr;
};

// Pinned host bytes of one job: its DEM (uploaded from here), VIX tables,
// SITE job table, then its outputs (SITE counters, error flag, observers,
// selection) read back into here.
struct PinLayout {
  size_t dem, tabs, wtab, out, obs, sel, total;
};

PinLayout pin_layout(const BatchPlan &bp) {
  const Job &J = bp.jobs[0];
  PinLayout L;
  size_t o = 0;
  L.dem = o;
  o += align256((size_t)J.n * J.n * 2);
  L.tabs = o;
  o += align256(bp.tab_bytes);
  L.wtab = o;
  o += align256(bp.wtab_bytes);
  L.out = o;
  o += 256;
  L.obs = o;
  o += align256((size_t)J.g.nwanted * 4);
  L.sel = o;
  o += align256((size_t)J.g.nwanted);
  L.total = o;
  return L;
}

constexpr int kTiers = 3, kStageStreams = 2 * kTiers;

// SITE CTAs of a served job: at most kServeSiteCtas SMs (or the fewest that
// hold its candidates), so that a selection, whose CTAs fill their SMs'
// register files, leaves most of the GPU to other jobs' stages.
constexpr int kServeSiteCtas = 48;

const siting_plan *serve_plan(int sm_count, const siting_params *p) {
  thread_local siting_plan plan;
  siting_geometry g{};
  geometry_of(p->nrows, p->bw, p->nwanted0, &g);
  const int need = std::max(1, (g.nwanted + 4095) / 4096);
  plan = siting_plan{0, -1, -1,
                     std::min(site_default_ctas(std::max(1, g.nwanted), sm_count),
                              std::max(need, kServeSiteCtas))};
  return &plan;
}

}  // namespace

struct siting_server {
  siting_ctx *ctx = nullptr;
  size_t budget = 0;
  int max_jobs = 64;
  bool reserve = false;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<long long> queue;          // waiting for admission
  std::deque<long long> staged;        // stages done, selection not yet enqueued
  std::deque<long long> finished;      // done on the GPU, results not yet copied out
  std::unordered_map<long long, Request> reqs;
  long long next_id = 1;
  int inflight = 0;
  bool stop = false;
  std::thread worker;
  siting_server_stats st{};
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  double busy_since = 0;
  // device arena (hbm_budget bytes) and pinned host arena
  unsigned char *d_arena = nullptr;
  unsigned char *h_arena = nullptr;
  size_t h_size = 0;
  RangeAlloc d_alloc, h_alloc;
  cudaStream_t stage[kStageStreams] = {};
  cudaStream_t site = nullptr;
  int next_stage[kTiers] = {};
  int admissions = 0;
  std::vector<cudaEvent_t> ev_pool;

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  void run();
  int setup();
  int launch_stages(long long id, Request &r);
  int launch_site(long long id, Request &r);
  void finish(long long id, Request &r);
  // A job whose work could not be enqueued: nothing more is queued for it;
  // wait for what was, then report (called with the lock held).
  void fail_job(long long id, Request &r, int rc, const std::string &msg) {
    cudaStreamSynchronize(site);
    for (auto &s : stage) cudaStreamSynchronize(s);
    r.info.status = rc;
    std::strncpy(r.info.error, msg.c_str(), sizeof(r.info.error) - 1);
    finish(id, r);
    cv_done.notify_all();
  }
};

namespace {

struct DoneMsg {
  siting_server *s;
  long long id;
  bool site_done;  // false: the stages are done
};

// Host callback at the end of a job's stages or of its selection: no CUDA
// calls here, only the hand-over to the worker.
void CUDART_CB job_step_done(void *arg) {
  DoneMsg *m = static_cast<DoneMsg *>(arg);
  {
    // notified under the lock: once it is released the server may be gone
    std::lock_guard<std::mutex> g(m->s->mu);
    (m->site_done ? m->s->finished : m->s->staged).push_back(m->id);
    m->s->cv_work.notify_one();
  }
  delete m;
}

cudaError_t enqueue_callback(cudaStream_t st, siting_server *s, long long id, bool site_done) {
  DoneMsg *m = new DoneMsg{s, id, site_done};
  const cudaError_t e = cudaLaunchHostFunc(st, job_step_done, m);
  if (e != cudaSuccess) delete m;
  return e;
}

}  // namespace

int siting_server::setup() {
  siting_ctx *ctx = this->ctx;
  if (!d_arena) {
    void *p;
    int rc = ws_get(ctx, kBatch, budget, &p);
    if (rc) return rc;
    d_arena = static_cast<unsigned char *>(p);
    d_alloc.reset(budget);
  }
  if (!site) {
    int least = 0, greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    // priorities: numerically lower is served first; SITE first, then the
    // stage tiers from small jobs to large ones
    CK(cudaStreamCreateWithPriority(&site, cudaStreamNonBlocking, greatest));
    for (int t = 0; t < kTiers; t++) {
      const int span = least - greatest;  // >= 0
      const int pr = std::min(least, greatest + 1 + (span > 1 ? t * (span - 1) / (kTiers - 1) : 0));
      for (int i = 0; i < 2; i++)
        CK(cudaStreamCreateWithPriority(&stage[2 * t + i], cudaStreamNonBlocking, pr));
    }
  }
  return SITING_OK;
}

// Enqueues an admitted job's pinned DEM copy and upload and its three stages
// on a stage stream, ending in a host callback.  Called by the worker without
// the lock held.
int siting_server::launch_stages(long long id, Request &r) {
  siting_ctx *ctx = this->ctx;
  const BatchPlan &bp = r.plan;
  const Job &J = bp.jobs[0];
  const PinLayout L = pin_layout(bp);
  unsigned char *base = d_arena + r.d_off;
  unsigned char *pin = h_arena + r.h_off;
  const long long cells = (long long)J.n * J.n;
  const int tier = cells <= (1ll << 20) ? 0 : cells <= (4ll << 20) ? 1 : 2;
  cudaStream_t s1 = stage[2 * tier + next_stage[tier]];
  next_stage[tier] ^= 1;
  // the DEM into pinned memory (a window of a larger raster row by row), so
  // that its upload is asynchronous
  const int sp = r.pitch ? r.pitch : J.n;
  uint16_t *hdem = reinterpret_cast<uint16_t *>(pin + L.dem);
  for (int x = 0; x < J.n; x++)
    std::memcpy(hdem + (size_t)x * J.n, r.elevs + (size_t)x * sp, (size_t)J.n * 2);
  SiteScratch s;
  site_carve_scratch(base + J.o_site, J.n, J.g.nwanted, J.G, J.p.roi, &s);
  const size_t site_zero = (unsigned char *)s.order - (base + J.o_site);
  int *err = reinterpret_cast<int *>(base + J.o_err);
  CK(cudaMemsetAsync(base + J.o_site, 0, site_zero, s1));
  CK(cudaMemsetAsync(err, 0, 256, s1));
  CK(cudaMemcpy2DAsync(base + J.o_dem, (size_t)J.pitch * 2, hdem, (size_t)J.n * 2,
                       (size_t)J.n * 2, J.n, cudaMemcpyHostToDevice, s1));
  vix_fill_tables(pin + L.tabs + J.o_tab, J.p.roi, J.p.ntests);
  CK(cudaMemcpyAsync(base + bp.o_tabs, pin + L.tabs, bp.tab_bytes, cudaMemcpyHostToDevice, s1));
  const DemView dem{reinterpret_cast<const uint16_t *>(base + J.o_dem), J.n, J.pitch, true};
  int32_t *d_obs = reinterpret_cast<int32_t *>(base + J.o_obs);
  uint8_t *d_sel = reinterpret_cast<uint8_t *>(base + J.o_sel);
  uint64_t *d_sheds = reinterpret_cast<uint64_t *>(base + J.o_sheds);
  CK(launch_vix(dem, J.p.roi, J.p.oht, J.p.tht, J.p.ntests, base + J.o_vix,
                base + bp.o_tabs + J.o_tab, J.vp, err, s1));
  CK(launch_findmax(base + J.o_vix, J.n, J.g.blocksize, J.g.nblocks, J.g.nwantedperblock, d_obs,
                    s1));
  CK(launch_sheds(dem, J.p.roi, J.p.oht, J.p.tht, J.g.nwanted, d_obs, d_sheds, J.sp, err, s1));
  CK(cudaEventRecord(r.staged, s1));
  CK(enqueue_callback(s1, this, id, false));
  return SITING_OK;
}

// Enqueues a staged job's selection and readback on the SITE stream, ending
// in a host callback.  Called by the worker without the lock held.
int siting_server::launch_site(long long id, Request &r) {
  siting_ctx *ctx = this->ctx;
  const BatchPlan &bp = r.plan;
  const Job &J = bp.jobs[0];
  const PinLayout L = pin_layout(bp);
  unsigned char *base = d_arena + r.d_off;
  unsigned char *pin = h_arena + r.h_off;
  SiteScratch s;
  site_carve_scratch(base + J.o_site, J.n, J.g.nwanted, J.G, J.p.roi, &s);
  int *err = reinterpret_cast<int *>(base + J.o_err);
  int32_t *d_obs = reinterpret_cast<int32_t *>(base + J.o_obs);
  uint8_t *d_sel = reinterpret_cast<uint8_t *>(base + J.o_sel);
  const uint64_t *d_sheds = reinterpret_cast<const uint64_t *>(base + J.o_sheds);
  CK(cudaStreamWaitEvent(site, r.staged, 0));
  CK(cudaMemsetAsync(d_sel, 0, J.g.nwanted, site));
  SiteJob sj{J.n, J.p.roi, J.p.intervis, J.g.nwanted, d_obs, d_sheds, J.g.blocksize,
             J.g.nblocks, J.g.nwantedperblock, d_sel, s, J.G, err};
  CK(launch_site_jobs(&sj, 1, base + bp.o_wtabs + bp.o_wtab[0], pin + L.wtab, site));
  long long *hout = reinterpret_cast<long long *>(pin + L.out);
  CK(cudaMemcpyAsync(hout, s.out, 3 * sizeof(long long), cudaMemcpyDeviceToHost, site));
  CK(cudaMemcpyAsync(hout + 4, err, sizeof(int), cudaMemcpyDeviceToHost, site));
  CK(cudaMemcpyAsync(pin + L.obs, d_obs, (size_t)J.g.nwanted * 4, cudaMemcpyDeviceToHost, site));
  CK(cudaMemcpyAsync(pin + L.sel, d_sel, J.g.nwanted, cudaMemcpyDeviceToHost, site));
  CK(enqueue_callback(site, this, id, true));
  return SITING_OK;
}

// Results of a job whose work has ended: copied from pinned memory into the
// caller's buffers; its memory is released.  Called with the lock held.
void siting_server::finish(long long id, Request &r) {
  const BatchPlan &bp = r.plan;
  const Job &J = bp.jobs[0];
  const PinLayout L = pin_layout(bp);
  unsigned char *pin = h_arena + r.h_off;
  const long long *hout = reinterpret_cast<const long long *>(pin + L.out);
  int flag = (int)(hout[4] & 0xffffffff);
  if (r.info.status == SITING_OK && flag) {
    r.info.status = check_err_flags(ctx, &flag, 1);
    std::strncpy(r.info.error, ctx->err.c_str(), sizeof(r.info.error) - 1);
  }
  if (r.info.status == SITING_OK) {
    std::memcpy(r.obs, pin + L.obs, (size_t)J.g.nwanted * 4);
    std::memcpy(r.sel, pin + L.sel, J.g.nwanted);
    siting_result &res = r.info.result;
    res = siting_result{};
    res.nusedsheds = (int)hout[0];
    res.cumarea = hout[1];
    res.coverage = 100.0 * res.cumarea / ((double)J.n * J.n);
    res.nwanted = J.g.nwanted;
    res.site_rounds = (int)hout[2];
  }
  (void)id;
  r.info.t_done = now();
  d_alloc.release(r.d_off, r.ws);
  h_alloc.release(r.h_off, r.pin);
  if (r.staged) ev_pool.push_back(r.staged);
  r.staged = nullptr;
  r.plan = BatchPlan{};
  r.done = true;
  st.completed++;
  if (--inflight == 0) st.busy_s += r.info.t_done - busy_since;
}

void siting_server::run() {
  cudaSetDevice(ctx->device);
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    auto admissible = [&] {
      if (queue.empty() || inflight >= max_jobs) return false;
      const Request &r = reqs[queue.front()];
      size_t o;
      if (!d_alloc.alloc(r.ws, &o)) return false;
      d_alloc.release(o, r.ws);
      if (!h_alloc.alloc(r.pin, &o)) return false;
      h_alloc.release(o, r.pin);
      return true;
    };
    cv_work.wait(lk, [&] {
      return !finished.empty() || !staged.empty() || admissible() ||
             (stop && queue.empty() && inflight == 0);
    });
    while (!staged.empty()) {  // selections, in the order the stages finished
      const long long id = staged.front();
      staged.pop_front();
      Request &r = reqs[id];
      lk.unlock();
      const int rc = launch_site(id, r);
      const std::string msg = rc ? ctx->err : std::string();
      lk.lock();
      if (rc) fail_job(id, r, rc, msg);
    }
    while (!finished.empty()) {
      const long long id = finished.front();
      finished.pop_front();
      finish(id, reqs[id]);
      cv_done.notify_all();
    }
    bool admitted = false;
    while (admissible()) {
      const long long id = queue.front();
      queue.pop_front();
      Request &r = reqs[id];
      d_alloc.alloc(r.ws, &r.d_off);
      h_alloc.alloc(r.pin, &r.h_off);
      st.peak_workspace = std::max(st.peak_workspace, d_alloc.used());
      if (inflight++ == 0) busy_since = now();
      r.info.t_start = now();
      r.info.batch_id = admissions + 1;
      r.info.batch_jobs = inflight;
      admitted = true;
      if (ev_pool.empty()) {
        cudaEvent_t e = nullptr;
        cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        ev_pool.push_back(e);
      }
      r.staged = ev_pool.back();
      ev_pool.pop_back();
      lk.unlock();
      const int rc = r.staged ? launch_stages(id, r) : SITING_ECUDA;
      const std::string msg = rc ? ctx->err : std::string();
      lk.lock();
      if (rc) fail_job(id, r, rc, msg);
    }
    if (admitted) {
      admissions++;
      st.batches++;
    }
    if (stop && queue.empty() && inflight == 0 && finished.empty() && staged.empty()) break;
  }
}

extern "C" {

int siting_server_create(int device, size_t hbm_budget, int max_batch_jobs, int reserve,
                         siting_server **out) {
  if (!out || hbm_budget == 0) return SITING_EINVAL;
  *out = nullptr;
  siting_ctx *ctx = nullptr;
  int rc = siting_ctx_create(device, hbm_budget, &ctx);
  if (rc) return rc;
  siting_server *s = new siting_server;
  s->ctx = ctx;
  s->budget = hbm_budget;
  s->max_jobs = max_batch_jobs > 0 ? max_batch_jobs : 64;
  s->reserve = reserve != 0;
  // pinned host arena: DEMs on their way up and results on their way down
  s->h_size = std::max<size_t>(64 << 20, std::min<size_t>(1ull << 30, hbm_budget / 4));
  if (cudaMallocHost(reinterpret_cast<void **>(&s->h_arena), s->h_size) != cudaSuccess) {
    cudaGetLastError();
    siting_ctx_destroy(ctx);
    delete s;
    return SITING_ENOMEM;
  }
  s->h_alloc.reset(s->h_size);
  if ((rc = s->setup())) {
    cudaFreeHost(s->h_arena);
    siting_ctx_destroy(ctx);
    delete s;
    return rc;
  }
  s->worker = std::thread([s] { s->run(); });
  *out = s;
  return SITING_OK;
}

int siting_server_destroy(siting_server *s) {
  if (!s) return SITING_EINVAL;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  s->worker.join();
  cudaSetDevice(s->ctx->device);
  if (s->site) cudaStreamSynchronize(s->site);
  for (auto &st : s->stage)
    if (st) cudaStreamDestroy(st);
  if (s->site) cudaStreamDestroy(s->site);
  for (auto e : s->ev_pool) cudaEventDestroy(e);
  cudaFreeHost(s->h_arena);
  siting_ctx_destroy(s->ctx);
  delete s;
  return SITING_OK;
}

int siting_server_submit(siting_server *s, const siting_params *p, const uint16_t *elevs,
                         int pitch, int32_t *obs, uint8_t *selected, long long *ticket) {
  if (!s || !p || !elevs || !obs || !selected || !ticket) return SITING_EINVAL;
  if (pitch != 0 && pitch < p->nrows) return SITING_EINVAL;
  // admission: the job alone must fit the budget and the pinned arena
  // (planning is host-only)
  BatchPlan plan;
  std::string e;
  const int rc = plan_batch(s->ctx->sm_count, 1, p, serve_plan(s->ctx->sm_count, p), &plan, &e);
  std::lock_guard<std::mutex> g(s->mu);
  const size_t pin = rc ? 0 : pin_layout(plan).total;
  if (rc || plan.ws > s->budget || pin > s->h_size) {
    s->st.refused++;
    return rc ? rc : SITING_ENOMEM;
  }
  const long long id = s->next_id++;
  Request &r = s->reqs[id];
  r.p = *p;
  r.elevs = elevs;
  r.pitch = pitch;
  r.obs = obs;
  r.sel = selected;
  r.ws = plan.ws;
  r.pin = pin;
  r.plan = std::move(plan);
  std::memset(&r.info, 0, sizeof(r.info));
  r.info.t_submit = s->now();
  s->queue.push_back(id);
  s->st.submitted++;
  *ticket = id;
  s->cv_work.notify_one();
  return SITING_OK;
}

int siting_server_wait(siting_server *s, long long ticket, double timeout_s,
                       siting_job_info *info) {
  if (!s) return SITING_EINVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return SITING_EINVAL;
  auto ready = [&] {
    auto f = s->reqs.find(ticket);
    return f == s->reqs.end() || f->second.done;
  };
  if (timeout_s < 0)
    s->cv_done.wait(lk, ready);
  else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready))
    return SITING_ETIMEOUT;
  it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return SITING_EINVAL;  // released by another waiter
  if (info) *info = it->second.info;
  s->reqs.erase(it);
  return SITING_OK;
}

int siting_server_stats_get(siting_server *s, siting_server_stats *st) {
  if (!s || !st) return SITING_EINVAL;
  std::lock_guard<std::mutex> g(s->mu);
  *st = s->st;
  st->pending = (long long)s->queue.size();
  if (s->inflight) st->busy_s += s->now() - s->busy_since;
  return SITING_OK;
}

}  // extern "C"
