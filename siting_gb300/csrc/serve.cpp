// Serving loop: continuous batching of independent siting jobs under an HBM
// budget (no counterpart in the reference, which runs one process per DEM).
//
// Jobs queue in arrival order.  One worker thread owns the context; whenever
// the GPU is free it takes the longest FIFO prefix of the queue whose batch
// workspace (plan_batch, host arithmetic only) fits the budget, at most
// max_batch_jobs jobs, and runs it as one batch.  Jobs that arrive meanwhile
// wait for the next batch.  A job whose own workspace exceeds the budget is
// refused when it is submitted, so the queue never blocks on it.  The batch
// workspace stays allocated between batches (optionally reserved at start).
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
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

struct Request {
  siting_params p;
  const uint16_t *elevs;
  int pitch;
  int32_t *obs;
  uint8_t *sel;
  siting_job_info info;
  bool done = false;
};

}  // namespace

struct siting_server {
  siting_ctx *ctx = nullptr;
  size_t budget = 0;
  int max_jobs = 64;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<long long> queue;
  std::unordered_map<long long, Request> reqs;
  long long next_id = 1;
  bool stop = false;
  std::thread worker;
  siting_server_stats st{};
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  void run();
};

void siting_server::run() {
  cudaSetDevice(ctx->device);
  std::unique_lock<std::mutex> lk(mu);
  int batch_id = 0;
  for (;;) {
    cv_work.wait(lk, [&] { return stop || !queue.empty(); });
    if (queue.empty()) break;  // stop requested and drained
    // the longest FIFO prefix that fits the budget
    std::vector<long long> ids;
    std::vector<siting_params> ps;
    size_t ws = 0;
    for (long long id : queue) {
      if ((int)ids.size() == max_jobs) break;
      ps.push_back(reqs[id].p);
      BatchPlan plan;
      std::string e;
      if (plan_batch(ctx->sm_count, (int)ps.size(), ps.data(), nullptr, &plan, &e) ||
          (plan.ws > budget && !ids.empty())) {
        ps.pop_back();
        break;
      }
      ids.push_back(id);
      ws = plan.ws;
    }
    const double t_start = now();
    std::vector<const uint16_t *> el;
    std::vector<int> pitch;
    std::vector<int32_t *> ob;
    std::vector<uint8_t *> se;
    for (long long id : ids) {
      queue.pop_front();
      Request &r = reqs[id];
      r.info.t_start = t_start;
      el.push_back(r.elevs);
      pitch.push_back(r.pitch);
      ob.push_back(r.obs);
      se.push_back(r.sel);
    }
    const int nb = (int)ids.size();
    lk.unlock();
    std::vector<siting_result> res(nb);
    const int rc = run_batch(ctx, nb, ps.data(), el.data(), pitch.data(), true, ob.data(),
                             se.data(), res.data(), nullptr);
    const std::string msg = rc ? ctx->err : std::string();
    lk.lock();
    const double t_done = now();
    batch_id++;
    for (int j = 0; j < nb; j++) {
      Request &r = reqs[ids[j]];
      r.info.status = rc;
      r.info.result = res[j];
      r.info.t_done = t_done;
      r.info.batch_id = batch_id;
      r.info.batch_jobs = nb;
      std::strncpy(r.info.error, msg.c_str(), sizeof(r.info.error) - 1);
      r.done = true;
    }
    st.completed += nb;
    st.batches++;
    st.busy_s += t_done - t_start;
    if (!rc && ws > st.peak_workspace) st.peak_workspace = ws;
    cv_done.notify_all();
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
  if (reserve) {
    void *p;
    if ((rc = ws_get(ctx, kBatch, hbm_budget, &p))) {
      siting_ctx_destroy(ctx);
      return rc;
    }
  }
  siting_server *s = new siting_server;
  s->ctx = ctx;
  s->budget = hbm_budget;
  s->max_jobs = max_batch_jobs > 0 ? max_batch_jobs : 64;
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
  siting_ctx_destroy(s->ctx);
  delete s;
  return SITING_OK;
}

int siting_server_submit(siting_server *s, const siting_params *p, const uint16_t *elevs,
                         int pitch, int32_t *obs, uint8_t *selected, long long *ticket) {
  if (!s || !p || !elevs || !obs || !selected || !ticket) return SITING_EINVAL;
  if (pitch != 0 && pitch < p->nrows) return SITING_EINVAL;
  // admission: the job alone must fit the budget (planning is host-only)
  BatchPlan plan;
  std::string e;
  const int rc = plan_batch(s->ctx->sm_count, 1, p, nullptr, &plan, &e);
  std::lock_guard<std::mutex> g(s->mu);
  if (rc || plan.ws > s->budget) {
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
  return SITING_OK;
}

}  // extern "C"
