// Autotuner: times the launch plans of each stage for one job's parameters on
// (a corner of) its DEM and keeps the fastest per (roi, ntests) in the
// context.  Later siting_run*, siting_run_batch* and stage calls that are
// given no plan use it.  Every plan gives the same results (the kernels'
// arithmetic does not depend on tiling or staging), so tuning changes only
// speed.
#include <algorithm>
#include <cstring>
#include <vector>

#include "ctx.h"
#include "kernels.h"
#include "siting.h"

using namespace siting;

namespace {

// Device time of fn: one warm-up call, then the smaller of two timed calls.
template <class F>
int time_ms(siting_ctx *ctx, F fn, float *ms) {
  cudaStream_t st = ctx->stream;
  CK(fn());
  float best = 1e30f;
  for (int i = 0; i < 2; i++) {
    CK(cudaEventRecord(ctx->ev[0], st));
    CK(fn());
    CK(cudaEventRecord(ctx->ev[1], st));
    CK(cudaEventSynchronize(ctx->ev[1]));
    float t = 0;
    CK(cudaEventElapsedTime(&t, ctx->ev[0], ctx->ev[1]));
    best = std::min(best, t);
  }
  *ms = best;
  return SITING_OK;
}

}  // namespace

extern "C" int siting_autotune(siting_ctx *ctx, const siting_params *p, const uint16_t *elevs,
                               int sample_rows, siting_plan *best) {
  if (!ctx || !p || !elevs) return fail(ctx, SITING_EINVAL, "autotune: null argument");
  std::string m;
  if (validate(p, 1, &m)) return fail(ctx, SITING_EINVAL, m);
  cudaSetDevice(ctx->device);
  const int N = p->nrows;
  const int n = std::min(N, sample_rows > 0 ? sample_rows : 1024);
  // the sample: the DEM's top-left n x n corner with the job's observer density
  const long long nw0 = std::max<long long>(1, (long long)p->nwanted0 * n / N * n / N);
  siting_geometry g;
  if (!geometry_of(n, p->bw, (int)nw0, &g))
    return fail(ctx, SITING_EINVAL, "autotune: sample too small for the block geometry");
  const int pitch = (n + 7) & ~7;
  const int nr = 2 * p->roi + 1, nwpr = (nr + 63) / 64;
  const size_t per = (size_t)nr * nwpr;
  void *d_dem, *d_vix, *d_obs, *d_sheds, *d_sel, *tab, *d_err;
  int rc;
  if ((rc = ws_get(ctx, kDem, (size_t)pitch * n * 2, &d_dem))) return rc;
  if ((rc = ws_get(ctx, kVix, (size_t)n * n, &d_vix))) return rc;
  if ((rc = ws_get(ctx, kObs, (size_t)g.nwanted * 4, &d_obs))) return rc;
  if ((rc = ws_get(ctx, kSheds, (size_t)g.nwanted * per * 8, &d_sheds))) return rc;
  if ((rc = ws_get(ctx, kSel, (size_t)g.nwanted, &d_sel))) return rc;
  if ((rc = ws_get(ctx, kErr, 256, &d_err))) return rc;
  const size_t tb = vix_table_bytes(p->roi, p->ntests);
  if ((rc = ws_get(ctx, kTables, tb, &tab))) return rc;
  ctx->tab_host.assign(tb, 0);
  vix_fill_tables(ctx->tab_host.data(), p->roi, p->ntests);
  cudaStream_t st = ctx->stream;
  CK(cudaMemcpyAsync(tab, ctx->tab_host.data(), tb, cudaMemcpyHostToDevice, st));
  CK(cudaMemcpy2DAsync(d_dem, (size_t)pitch * 2, elevs, (size_t)N * 2, (size_t)n * 2, n,
                       cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(d_err, 0, 256, st));
  CK(cudaStreamSynchronize(st));
  ctx->tab_roi = p->roi;
  ctx->tab_ntests = p->ntests;
  const DemView dem{static_cast<const uint16_t *>(d_dem), n, pitch, true};
  int *err = static_cast<int *>(d_err);

  siting_plan out{0, -1, -1, 0};
  // VIX: tile 16/32/64, halo staged or read through L1 (plans the kernel
  // cannot take are mapped to the nearest one it can, then deduplicated)
  std::vector<VixPlan> seen;
  float bt = 1e30f;
  for (int tile : {16, 32, 64})
    for (int sm : {1, 0}) {
      const VixPlan vp = vix_plan_for(n, p->roi, p->ntests, tile, sm);
      if (std::any_of(seen.begin(), seen.end(), [&](const VixPlan &q) {
            return q.tile == vp.tile && q.use_smem == vp.use_smem;
          }))
        continue;
      seen.push_back(vp);
      float t;
      rc = time_ms(ctx, [&] {
        return launch_vix(dem, p->roi, p->oht, p->tht, p->ntests, static_cast<uint8_t *>(d_vix),
                          tab, vp, err, st);
      }, &t);
      if (rc) return rc;
      if (t < bt) {
        bt = t;
        out.vix_tile = vp.tile;
        out.vix_smem = vp.use_smem ? 1 : 0;
      }
    }
  // observers of the sample for the VIEWSHED trials
  CK(launch_vix(dem, p->roi, p->oht, p->tht, p->ntests, static_cast<uint8_t *>(d_vix), tab,
                vix_plan_for(n, p->roi, p->ntests, out.vix_tile, out.vix_smem), err, st));
  CK(launch_findmax(static_cast<uint8_t *>(d_vix), n, g.blocksize, g.nblocks, g.nwantedperblock,
                    static_cast<int32_t *>(d_obs), st));
  bt = 1e30f;
  std::vector<ShedPlan> tried;
  for (int sm : {1, 2, 0}) {
    const ShedPlan sp = shed_plan_for(p->roi, sm);
    bool seen = false;  // the same plan under another setting
    for (const ShedPlan &q : tried)
      seen |= q.threads == sp.threads && q.use_smem == sp.use_smem && q.half == sp.half;
    if (seen) continue;
    tried.push_back(sp);
    float t;
    rc = time_ms(ctx, [&] {
      return launch_sheds(dem, p->roi, p->oht, p->tht, g.nwanted, static_cast<int32_t *>(d_obs),
                          static_cast<uint64_t *>(d_sheds), sp, err, st);
    }, &t);
    if (rc) return rc;
    if (t < bt) {
      bt = t;
      out.shed_smem = sm;
    }
  }
  // SITE group size, only when the sample is the whole job (its rounds and
  // candidates per CTA depend on the DEM's size)
  if (n == N && g.nwanted > 0) {
    const int gmin = (g.nwanted + 4095) / 4096;
    const int gdef = site_default_ctas(g.nwanted, ctx->sm_count);
    std::vector<int> cands = {gdef, std::max(gmin, gdef / 2), std::max(gmin, gdef / 4)};
    std::sort(cands.begin(), cands.end());
    cands.erase(std::unique(cands.begin(), cands.end()), cands.end());
    bt = 1e30f;
    for (int G : cands) {
      if (!site_supported(p->roi, g.nwanted, G) ||
          site_smem_bytes(p->roi, g.nwanted, G, g.nblocks, g.nwantedperblock, g.blocksize) >
              220 * 1024)
        continue;
      void *sp;
      const size_t sb = site_scratch_bytes(n, g.nwanted, G, p->roi);
      if ((rc = ws_get(ctx, kSite, sb, &sp))) return rc;
      SiteScratch s;
      site_carve_scratch(sp, n, g.nwanted, G, p->roi, &s);
      float t;
      rc = time_ms(ctx, [&] {
        cudaError_t e = cudaMemsetAsync(sp, 0, (unsigned char *)s.order - (unsigned char *)sp, st);
        if (e != cudaSuccess) return e;
        return launch_site(n, p->roi, p->intervis, g.nwanted, static_cast<int32_t *>(d_obs),
                           static_cast<uint64_t *>(d_sheds), g.blocksize, g.nblocks,
                           g.nwantedperblock, static_cast<uint8_t *>(d_sel), s, G, err, st);
      }, &t);
      if (rc) return rc;
      if (t < bt) {
        bt = t;
        out.site_ctas = G;
      }
    }
  }
  int h_err = 0;
  CK(cudaMemcpy(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if ((rc = check_err_flags(ctx, &h_err, 1))) return rc;
  bool found = false;
  for (TunedPlan &t : ctx->tuned)
    if (t.roi == p->roi && t.ntests == p->ntests) {
      t.plan = out;
      found = true;
    }
  if (!found) ctx->tuned.push_back(TunedPlan{p->roi, p->ntests, out});
  if (best) *best = out;
  return SITING_OK;
}

extern "C" int siting_autotune_set(siting_ctx *ctx, int roi, int ntests, const siting_plan *plan) {
  if (!ctx || !plan || roi < 0 || ntests < 0) return SITING_EINVAL;
  const siting_plan &q = *plan;
  if ((q.vix_tile != 0 && q.vix_tile != 16 && q.vix_tile != 32 && q.vix_tile != 64) ||
      q.vix_smem < -1 || q.vix_smem > 1 || q.shed_smem < -1 || q.shed_smem > 2 || q.site_ctas < 0)
    return SITING_EINVAL;
  for (TunedPlan &t : ctx->tuned)
    if (t.roi == roi && t.ntests == ntests) {
      t.plan = q;
      return SITING_OK;
    }
  ctx->tuned.push_back(TunedPlan{roi, ntests, q});
  return SITING_OK;
}

extern "C" int siting_autotune_clear(siting_ctx *ctx) {
  if (!ctx) return SITING_EINVAL;
  ctx->tuned.clear();
  return SITING_OK;
}
