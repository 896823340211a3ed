// Batched form: many independent jobs (DEMs of any size and parameters) per
// call.  The greedy SITE selections, whose dependent rounds leave most SMs
// idle when run one job at a time, run many jobs at once: the jobs' CTA
// groups are packed into as few cooperative launches ("waves") as the SM
// count allows, largest groups first, each group with its own barrier and
// scratch.  The stages of each wave's jobs are enqueued on the context's
// stream in wave order: VIX and FINDMAX as grids over all the wave's jobs'
// items (small jobs) or one launch per job, then one VIEWSHED launch per job;
// each SITE launch runs on a second stream as soon as its jobs' viewsheds
// exist, so the selections overlap the later waves' stages.  One workspace
// holds every job's buffers; results are collected after a single
// synchronisation.  A device-resident batch of small jobs is captured as a
// CUDA graph and replayed when the same batch comes again.
#include <algorithm>
#include <numeric>
#include <vector>

#include "batch.h"
#include "ctx.h"
#include "kernels.h"
#include "siting.h"

using namespace siting;

namespace {

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// CTAs of a job's SITE group in a batch: the fewest that keep each CTA's
// candidates within the kernel's per-CTA capacity, so many jobs share the SMs.
int batch_site_ctas(int nsheds, int sm_count) {
  const int g = std::max(1, (nsheds + 4095) / 4096);
  return std::min(std::min(g, std::max(1, nsheds)), sm_count);
}

constexpr int kBatchWaveCtas = 96;

bool site_fits(const Job &J, int G) {
  return site_smem_bytes(J.p.roi, J.g.nwanted, G, J.g.nblocks, J.g.nwantedperblock,
                         J.g.blocksize) <= 220 * 1024;
}

}  // namespace

namespace siting {

// Launch plan and workspace layout of a batch: pure host arithmetic (no
// device work), so that admission control can size a batch before running it.
int plan_batch(int sm_count, int njobs, const siting_params *params, const siting_plan *plans,
               BatchPlan *bp, std::string *err) {
  auto bad = [&](int j, const std::string &m) {
    *err = "job " + std::to_string(j) + ": " + m;
    return SITING_EINVAL;
  };
  std::vector<Job> &jobs = bp->jobs;
  jobs.assign(njobs, Job{});
  size_t ws = 0, tab_bytes = 0;
  for (int j = 0; j < njobs; j++) {
    Job &J = jobs[j];
    J.p = params[j];
    std::string m;
    if (validate(&J.p, 1, &m)) return bad(j, m);
    geometry_of(J.p.nrows, J.p.bw, J.p.nwanted0, &J.g);
    J.n = J.p.nrows;
    J.pitch = (J.n + 7) & ~7;
    J.nr = 2 * J.p.roi + 1;
    J.nwpr = (J.nr + 63) / 64;
    J.per = (size_t)J.nr * J.nwpr;
    const siting_plan *pl = plans ? &plans[j] : nullptr;
    J.vp = vix_plan_for(J.n, J.p.roi, J.p.ntests, pl ? pl->vix_tile : 0, pl ? pl->vix_smem : -1);
    J.sp = shed_plan_for(J.p.roi, pl ? pl->shed_smem : -1);
    J.G = (pl && pl->site_ctas > 0) ? std::min(pl->site_ctas, sm_count)
                                     : batch_site_ctas(J.g.nwanted, sm_count);
    if (!site_supported(J.p.roi, J.g.nwanted, J.G)) return bad(j, "beyond the SITE kernel's limits");
    J.auto_G = !(pl && pl->site_ctas > 0);
    if (!site_fits(J, J.G)) return bad(j, "SITE shared-memory plan too large");
  }
  // SITE launches: pack the groups into waves of <= sm_count CTAs, intervis
  // jobs first (their selections take several times more rounds), largest
  // groups first within each kind.  Waves run in order, each as soon as its
  // jobs' viewsheds exist, so the long selections overlap later jobs' stages
  // and the last wave, which nothing overlaps, holds the short ones.
  std::vector<int> order(njobs);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    if (jobs[a].p.intervis != jobs[b].p.intervis) return jobs[a].p.intervis > jobs[b].p.intervis;
    return jobs[a].G > jobs[b].G;
  });
  // A SITE CTA fills its SM's register file, so a launch holds its SMs
  // alone: waves take at most kBatchWaveCtas SMs, leaving the rest to the
  // later jobs' stages that the waves overlap (the last wave, which runs after
  // every stage, may take them all below).
  const int wave_cap = std::min(sm_count, kBatchWaveCtas);
  std::vector<std::vector<int>> &waves = bp->waves;
  std::vector<int> &wave_ctas = bp->wave_ctas;
  waves.clear();
  wave_ctas.clear();
  for (int j : order) {
    size_t w = 0;
    while (w < waves.size() && wave_ctas[w] + jobs[j].G > std::max(wave_cap, jobs[j].G)) w++;
    if (w == waves.size()) {
      waves.emplace_back();
      wave_ctas.push_back(0);
    }
    waves[w].push_back(j);
    wave_ctas[w] += jobs[j].G;
  }
  // a wave lasts as long as its slowest group: SMs a wave leaves free go to
  // its automatically planned groups in proportion to their candidates (a
  // group's rounds shorten with more CTAs), up to the single-job default.
  // The last wave runs after every job's stages, with nothing to share the
  // GPU with: it may grow to every SM (64 jobs of 256^2-512^2: 39.9 ->
  // 26.3 ms; the 64-DEM mix of 512^2-2048^2 with waves of 96: 231 ms).
  for (size_t w = 0; w < waves.size(); w++) {
    const int spare = (w + 1 == waves.size() ? sm_count : wave_cap) - wave_ctas[w];
    double total = 0;
    for (int j : waves[w])
      if (jobs[j].auto_G) total += jobs[j].g.nwanted;
    if (spare <= 0 || total <= 0) continue;
    for (int j : waves[w]) {
      Job &J = jobs[j];
      if (!J.auto_G) continue;
      const int cap = site_default_ctas(J.g.nwanted, sm_count);
      const int want = std::min(cap, J.G + (int)(spare * (J.g.nwanted / total)));
      if (want > J.G && site_supported(J.p.roi, J.g.nwanted, want) && site_fits(J, want)) {
        wave_ctas[w] += want - J.G;
        J.G = want;
      }
    }
  }
  for (int j = 0; j < njobs; j++) {
    Job &J = jobs[j];
    J.o_dem = ws;
    ws += align256((size_t)J.pitch * J.n * 2);
    J.o_vix = ws;
    ws += align256((size_t)J.n * J.n);
    J.o_obs = ws;
    ws += align256((size_t)J.g.nwanted * 4);
    J.o_sel = ws;
    ws += align256((size_t)J.g.nwanted);
    J.o_sheds = ws;
    ws += align256((size_t)J.g.nwanted * J.per * 8);
    J.o_tab = tab_bytes;
    tab_bytes += align256(vix_table_bytes(J.p.roi, J.p.ntests));
    J.o_site = ws;
    ws += align256(site_scratch_bytes(J.n, J.g.nwanted, J.G, J.p.roi));
    J.o_err = ws;
    ws += 256;
  }
  std::vector<size_t> &o_wtab = bp->o_wtab;
  o_wtab.assign(waves.size(), 0);
  size_t wtab_bytes = 0;
  for (size_t w = 0; w < waves.size(); w++) {
    o_wtab[w] = wtab_bytes;
    wtab_bytes += align256(site_job_table_bytes((int)waves[w].size(), wave_ctas[w]));
  }
  bp->o_tabs = ws;
  ws += align256(tab_bytes);
  bp->o_wtabs = ws;
  ws += align256(wtab_bytes);
  bp->ws = ws;
  bp->tab_bytes = tab_bytes;
  bp->wtab_bytes = wtab_bytes;
  return SITING_OK;
}

void batch_graph_reset(siting_ctx *ctx) {
  if (ctx->bg_exec) cudaGraphExecDestroy(ctx->bg_exec);
  ctx->bg_exec = nullptr;
  ctx->bg_key.clear();
}

int run_batch(siting_ctx *ctx, int njobs, const siting_params *params,
              const uint16_t *const *elevs, const int *src_pitch, bool host_io,
              int32_t *const *obs_out, uint8_t *const *sel_out, siting_result *results,
              const siting_plan *plans) {
  if (!ctx || njobs < 0 || (njobs && (!params || !elevs || !obs_out || !sel_out)))
    return fail(ctx, SITING_EINVAL, "run_batch: null argument");
  if (njobs == 0) return SITING_OK;
  for (int j = 0; j < njobs; j++)
    if (!elevs[j] || !obs_out[j] || !sel_out[j])
      return fail(ctx, SITING_EINVAL, "job " + std::to_string(j) + ": null buffer");
  cudaSetDevice(ctx->device);
  std::vector<siting_plan> tuned;  // autotuned plans where the caller gave none
  if (!plans && !ctx->tuned.empty()) {
    tuned.resize(njobs);
    for (int j = 0; j < njobs; j++) {
      const siting_plan *tp = tuned_plan(ctx, params[j].roi, params[j].ntests);
      tuned[j] = tp ? *tp : siting_plan{0, -1, -1, 0};
      tuned[j].site_ctas = 0;  // SITE groups are sized by the batch's packing
    }
    plans = tuned.data();
  }
  BatchPlan plan;
  std::string perr;
  if (int prc = plan_batch(ctx->sm_count, njobs, params, plans, &plan, &perr))
    return fail(ctx, prc, perr);
  std::vector<Job> &jobs = plan.jobs;
  const auto &waves = plan.waves;
  const auto &wave_ctas = plan.wave_ctas;
  const auto &o_wtab = plan.o_wtab;
  const size_t ws = plan.ws, tab_bytes = plan.tab_bytes, wtab_bytes = plan.wtab_bytes;
  const size_t o_tabs = plan.o_tabs, o_wtabs = plan.o_wtabs;
  (void)wave_ctas;

  void *base_v;
  int rc = ws_get(ctx, kBatch, ws, &base_v);
  if (rc) return rc;
  unsigned char *base = static_cast<unsigned char *>(base_v);
  // pinned staging: VIX tables, wave job tables, then per-job readback
  const size_t s_tabs = 0, s_wtabs = align256(tab_bytes);
  const size_t s_out = s_wtabs + align256(wtab_bytes);
  const size_t s_bytes = s_out + (size_t)njobs * 16 * sizeof(long long);
  cudaStream_t st = ctx->stream;
  // the SITE stream has the highest priority: a cooperative SITE launch needs
  // all its SMs at once, and the block scheduler then gives it SMs as stage
  // CTAs end instead of refilling them from the stage grids
  if (!ctx->stream2) {
    int least = 0, greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CK(cudaStreamCreateWithPriority(&ctx->stream2, cudaStreamNonBlocking, greatest));
  }
  while (ctx->wave_ev.size() < waves.size()) {
    cudaEvent_t e;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    ctx->wave_ev.push_back(e);
  }
  cudaStream_t st2 = ctx->stream2;

  // VIX and FINDMAX launch form of each wave.  Automatic: grids over many
  // jobs' items where the wave's jobs average at most 2^18 cells (many grids
  // of a few waves of CTAs each, whose tails the merged grid removes: 64 jobs
  // of 256^2-512^2, 29.9 -> 26.3 ms), one launch per job for larger jobs,
  // whose grids already fill the GPU (256^2-1024^2: 69.1 vs 66.5 ms merged
  // and per job; 512^2-2048^2: 231.3 vs 230.4 ms).
  std::vector<char> merged(waves.size());
  for (size_t w = 0; w < waves.size(); w++) {
    double cells = 0;
    for (int j : waves[w]) cells += (double)jobs[j].n * jobs[j].n;
    merged[w] = ctx->batch_mode == kBatchMerged ||
                (ctx->batch_mode == kBatchAuto && cells <= waves[w].size() * 262144.0);
  }
  // The device-resident form runs as a CUDA graph when every wave's VIX and
  // FINDMAX are merged grids (batches of small jobs, whose launches a replay
  // saves): the first call of a batch
  // captures its copies and launches, and a later call with the same jobs,
  // buffers and workspace replays the graph.  (Batches with larger jobs run
  // their launches directly: as a graph the 64-DEM mix took 240 ms against
  // 234 ms, not explained.)  The graph's host staging is its own pinned
  // buffer, so nothing else overwrites what a replay copies.
  bool all_merged = true;
  for (char mw : merged) all_merged = all_merged && mw;
  const bool graph = !host_io && ctx->batch_graphs && all_merged;
  std::vector<unsigned char> key;
  if (graph) {
    auto put = [&](const void *p, size_t n) {
      const unsigned char *c = static_cast<const unsigned char *>(p);
      key.insert(key.end(), c, c + n);
    };
    put(&njobs, sizeof(njobs));
    put(params, sizeof(siting_params) * njobs);
    put(elevs, sizeof(void *) * njobs);
    put(obs_out, sizeof(void *) * njobs);
    put(sel_out, sizeof(void *) * njobs);
    for (int j = 0; j < njobs; j++) {
      const int sp = src_pitch ? src_pitch[j] : 0;
      put(&sp, sizeof(sp));
      const siting_plan pl = plans ? plans[j] : siting_plan{0, -1, -1, 0};
      put(&pl, sizeof(pl));
    }
    put(&base, sizeof(base));
    put(&ctx->batch_mode, sizeof(ctx->batch_mode));
  }
  unsigned char *stage;
  if (graph) {
    if (ctx->bg_stage_cap < s_bytes) {
      batch_graph_reset(ctx);
      if (ctx->bg_stage) cudaFreeHost(ctx->bg_stage);
      ctx->bg_stage = nullptr;
      ctx->bg_stage_cap = 0;
      CK(cudaMallocHost(&ctx->bg_stage, s_bytes));
      ctx->bg_stage_cap = s_bytes;
    }
    stage = ctx->bg_stage;
  } else if ((rc = stage_get(ctx, s_bytes, &stage))) {
    return rc;
  }

  // Inside a capture, timing events are recorded as external events, so that
  // the graph records them when it runs (a plain record inside a capture only
  // orders the graph's nodes; outside one the flag is refused); the wave
  // events and the join order work across streams.
  auto enqueue = [&](bool capturing) -> int {
  const unsigned rec_flags = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
  CK(cudaEventRecordWithFlags(ctx->ev[5], st, rec_flags));
  for (int j = 0; j < njobs; j++) {  // inputs, VIX tables, zeroed scratch
    Job &J = jobs[j];
    const size_t sp = (size_t)(src_pitch && src_pitch[j] ? src_pitch[j] : J.n) * 2;
    if (host_io || J.n % 8 || (uintptr_t)elevs[j] % 16 || sp != (size_t)J.n * 2)
      CK(cudaMemcpy2DAsync(base + J.o_dem, (size_t)J.pitch * 2, elevs[j], sp, (size_t)J.n * 2, J.n,
                           host_io ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st));
    vix_fill_tables(stage + s_tabs + J.o_tab, J.p.roi, J.p.ntests);
    SiteScratch s;
    site_carve_scratch(base + J.o_site, J.n, J.g.nwanted, J.G, J.p.roi, &s);
    J.site_zero = (unsigned char *)s.order - (base + J.o_site);
    CK(cudaMemsetAsync(base + J.o_site, 0, J.site_zero, st));
    CK(cudaMemsetAsync(base + J.o_err, 0, 256, st));
  }

  CK(cudaMemcpyAsync(base + o_tabs, stage + s_tabs, tab_bytes, cudaMemcpyHostToDevice, st));
  CK(cudaEventRecordWithFlags(ctx->ev[0], st, rec_flags));
  auto dem_of = [&](int j) {
    const Job &J = jobs[j];
    const bool own = host_io || J.n % 8 || (uintptr_t)elevs[j] % 16 ||
                     (src_pitch && src_pitch[j] && src_pitch[j] != J.n);
    return own ? DemView{reinterpret_cast<const uint16_t *>(base + J.o_dem), J.n, J.pitch, true}
               : DemView{elevs[j], J.n, J.n, true};
  };
  auto obs_of = [&](int j) {
    return host_io ? reinterpret_cast<int32_t *>(base + jobs[j].o_obs) : obs_out[j];
  };
  auto sel_of = [&](int j) {
    return host_io ? reinterpret_cast<uint8_t *>(base + jobs[j].o_sel) : sel_out[j];
  };
  // VIX, FINDMAX and VIEWSHED of every job on the context's stream, in the
  // order of the SITE launches; each SITE launch runs on a second stream as
  // soon as its jobs' viewsheds exist, overlapping the later jobs' stages.
  // (SITE launches wait for their peers at group barriers; the kernels they
  // share the SMs with never wait for SITE, so the barriers always complete.)
  std::vector<StageJob> qjobs;
  for (size_t w = 0; w < waves.size(); w++) {
    // VIX and FINDMAX of the wave's jobs: one grid over their (job, tile)
    // items (two when some halos are staged and some not) and one over their
    // (job, block) items, or one launch per stage and job
    qjobs.clear();
    for (int j : waves[w]) {
      const Job &J = jobs[j];
      qjobs.push_back(StageJob{dem_of(j), J.p.roi, J.p.oht, J.p.tht, J.p.ntests, base + J.o_vix,
                               base + o_tabs + J.o_tab, J.vp, J.g.blocksize, J.g.nblocks,
                               J.g.nwantedperblock, obs_of(j),
                               reinterpret_cast<int *>(base + J.o_err)});
    }
    if (merged[w]) {
      CK(launch_vix_queue(qjobs.data(), (int)qjobs.size(), st));
      CK(launch_findmax_queue(qjobs.data(), (int)qjobs.size(), st));
    } else {
      for (int j : waves[w]) {
        const Job &J = jobs[j];
        CK(launch_vix(dem_of(j), J.p.roi, J.p.oht, J.p.tht, J.p.ntests, base + J.o_vix,
                      base + o_tabs + J.o_tab, J.vp, reinterpret_cast<int *>(base + J.o_err), st));
        CK(launch_findmax(base + J.o_vix, J.n, J.g.blocksize, J.g.nblocks, J.g.nwantedperblock,
                          obs_of(j), st));
      }
    }
    // VIEWSHED: one launch per job, its CTA sized to the job's rays (one ray
    // a thread), so CTAs of every job's size pack the SMs
    for (int j : waves[w]) {
      const Job &J = jobs[j];
      CK(launch_sheds(dem_of(j), J.p.roi, J.p.oht, J.p.tht, J.g.nwanted, obs_of(j),
                      reinterpret_cast<uint64_t *>(base + J.o_sheds), J.sp,
                      reinterpret_cast<int *>(base + J.o_err), st));
    }
    CK(cudaEventRecord(ctx->wave_ev[w], st));
  }
  CK(cudaEventRecordWithFlags(ctx->ev[1], st, rec_flags));
  for (size_t w = 0; w < waves.size(); w++) {
    CK(cudaStreamWaitEvent(st2, ctx->wave_ev[w], 0));
    std::vector<SiteJob> sj;
    for (int j : waves[w]) {
      const Job &J = jobs[j];
      SiteScratch s;
      site_carve_scratch(base + J.o_site, J.n, J.g.nwanted, J.G, J.p.roi, &s);
      CK(cudaMemsetAsync(sel_of(j), 0, J.g.nwanted, st2));
      sj.push_back(SiteJob{J.n, J.p.roi, J.p.intervis, J.g.nwanted, obs_of(j),
                           reinterpret_cast<const uint64_t *>(base + J.o_sheds), J.g.blocksize,
                           J.g.nblocks, J.g.nwantedperblock, sel_of(j), s, J.G,
                           reinterpret_cast<int *>(base + J.o_err)});
    }
    CK(launch_site_jobs(sj.data(), (int)sj.size(), base + o_wtabs + o_wtab[w],
                        stage + s_wtabs + o_wtab[w], st2));
  }
  CK(cudaEventRecordWithFlags(ctx->ev[4], st2, rec_flags));
  CK(cudaEventRecord(ctx->ev[2], st2));  // the join of the SITE stream
  CK(cudaStreamWaitEvent(st, ctx->ev[2], 0));
  // outputs and per-job readback (SITE outputs and error flag)
  long long *hout = reinterpret_cast<long long *>(stage + s_out);
  for (int j = 0; j < njobs; j++) {
    const Job &J = jobs[j];
    SiteScratch s;
    site_carve_scratch(base + J.o_site, J.n, J.g.nwanted, J.G, J.p.roi, &s);
    CK(cudaMemcpyAsync(hout + 16 * j, s.out, 3 * sizeof(long long), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hout + 16 * j + 8, base + J.o_err, sizeof(int), cudaMemcpyDeviceToHost,
                       st));
  }
  CK(cudaEventRecordWithFlags(ctx->ev[6], st, rec_flags));
  if (host_io)
    for (int j = 0; j < njobs; j++) {
      const Job &J = jobs[j];
      CK(cudaMemcpyAsync(obs_out[j], base + J.o_obs, (size_t)J.g.nwanted * 4,
                         cudaMemcpyDeviceToHost, st));
      CK(cudaMemcpyAsync(sel_out[j], base + J.o_sel, J.g.nwanted, cudaMemcpyDeviceToHost, st));
    }
  CK(cudaEventRecordWithFlags(ctx->ev[7], st, rec_flags));
  return SITING_OK;
  };

  if (graph && ctx->bg_exec && key == ctx->bg_key) {
    CK(cudaGraphLaunch(ctx->bg_exec, st));  // the same batch again: replay
    ctx->bg_replays++;
  } else if (graph) {
    batch_graph_reset(ctx);
    // capture mode ThreadLocal: other threads' CUDA calls are not affected
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const int erc = enqueue(true);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(st, &g);
    cudaGraphExec_t exec = nullptr;
    const bool ok = erc == SITING_OK && ce == cudaSuccess && g &&
                    cudaGraphInstantiate(&exec, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    if (ok) {
      ctx->bg_exec = exec;
      ctx->bg_key = key;
      ctx->bg_captures++;
      CK(cudaGraphLaunch(ctx->bg_exec, st));
    } else {  // a capture the runtime refused: run the same work directly
      cudaGetLastError();
      if ((rc = enqueue(false))) return rc;
    }
  } else if ((rc = enqueue(false))) {
    return rc;
  }
  CK(cudaStreamSynchronize(st));
  const long long *rout = reinterpret_cast<const long long *>(stage + s_out);
  std::vector<int> flags(njobs);
  for (int j = 0; j < njobs; j++) flags[j] = (int)(rout[16 * j + 8] & 0xffffffff);
  for (int j = 0; j < njobs; j++)
    if (flags[j]) {
      rc = check_err_flags(ctx, &flags[j], 1);
      ctx->err = "job " + std::to_string(j) + ": " + ctx->err;
      return rc;
    }
  float t[8] = {};
  cudaEventElapsedTime(&t[0], ctx->ev[5], ctx->ev[0]);
  cudaEventElapsedTime(&t[1], ctx->ev[0], ctx->ev[1]);  // VIX, FINDMAX, VIEWSHED of all jobs
  cudaEventElapsedTime(&t[4], ctx->ev[1], ctx->ev[4]);  // SITE after them
  cudaEventElapsedTime(&t[5], ctx->ev[6], ctx->ev[7]);
  cudaGetLastError();  // a phase time that cannot be read stays 0 and leaves no error behind
  if (results)
    for (int j = 0; j < njobs; j++) {
      siting_result &r = results[j];
      r = siting_result{};
      r.nusedsheds = (int)rout[16 * j];
      r.cumarea = rout[16 * j + 1];
      r.coverage = 100.0 * r.cumarea / ((double)jobs[j].n * jobs[j].n);
      r.nwanted = jobs[j].g.nwanted;
      r.site_rounds = (int)rout[16 * j + 2];
      r.ms_h2d = t[0];  // batch-wide phase times
      r.ms_vix = t[1];  // VIX, FINDMAX and VIEWSHED of every job (SITE overlaps them)
      r.ms_findmax = 0.f;
      r.ms_viewshed = 0.f;
      r.ms_site = t[4];  // SITE after the last VIEWSHED
      r.ms_d2h = t[5];
    }
  return SITING_OK;
}

}  // namespace siting

extern "C" {

int siting_run_batch(siting_ctx *ctx, int njobs, const siting_params *params,
                     const uint16_t *const *elevs, int32_t *const *obs, uint8_t *const *selected,
                     siting_result *results, const siting_plan *plans) {
  return run_batch(ctx, njobs, params, elevs, nullptr, true, obs, selected, results, plans);
}

int siting_batch_workspace_bytes(siting_ctx *ctx, int njobs, const siting_params *params,
                                 const siting_plan *plans, size_t *bytes) {
  if (!ctx || njobs < 0 || (njobs && !params) || !bytes)
    return fail(ctx, SITING_EINVAL, "batch_workspace_bytes: null argument");
  BatchPlan plan;
  std::string perr;
  if (int rc = plan_batch(ctx->sm_count, njobs, params, plans, &plan, &perr))
    return fail(ctx, rc, perr);
  *bytes = plan.ws;
  return SITING_OK;
}

int siting_run_batch_dev(siting_ctx *ctx, int njobs, const siting_params *params,
                         const uint16_t *const *d_elevs, int32_t *const *d_obs,
                         uint8_t *const *d_selected, siting_result *results,
                         const siting_plan *plans) {
  return run_batch(ctx, njobs, params, d_elevs, nullptr, false, d_obs, d_selected, results, plans);
}

}  // extern "C"
