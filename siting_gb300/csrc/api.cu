// C ABI of the siting library: context, workspace, stage entry points and the
// whole pipeline (include/siting.h).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "batch.h"
#include "ctx.h"
#include "kernels.h"
#include "siting.h"

using namespace siting;

namespace siting {

int fail(siting_ctx *ctx, int code, const std::string &msg) {
  if (ctx) ctx->err = msg;
  return code;
}

int cuda_fail(siting_ctx *ctx, cudaError_t e, const char *what) {
  return fail(ctx, SITING_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int stage_get(siting_ctx *ctx, size_t bytes, unsigned char **out) {
  if (ctx->h_stage_cap < bytes) {
    if (ctx->h_stage) {
      cudaStreamSynchronize(ctx->stream);
      cudaFreeHost(ctx->h_stage);
      ctx->h_stage = nullptr;
      ctx->h_stage_cap = 0;
    }
    const size_t want = std::max<size_t>(bytes, 1 << 16);
    if (cudaMallocHost(reinterpret_cast<void **>(&ctx->h_stage), want) != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, SITING_ENOMEM, "pinned staging allocation failed");
    }
    ctx->h_stage_cap = want;
  }
  *out = ctx->h_stage;
  return SITING_OK;
}

int check_err_flags(siting_ctx *ctx, const int *h, int n) {
  int f = 0;
  for (int i = 0; i < n; i++) f |= h[i];
  if (f & kErrTmaTimeout) return fail(ctx, SITING_ETIMEOUT, "TMA tile wait expired");
  if (f & kErrBarrierTimeout) return fail(ctx, SITING_ETIMEOUT, "SITE group barrier wait expired");
  if (f & kErrCapacity) return fail(ctx, SITING_ECUDA, "SITE neighbour list overflow");
  if (f & kErrSiteMismatch) return fail(ctx, SITING_ECUDA, "SITE self-check failed");
  if (f & kErrBadInput) return fail(ctx, SITING_EINVAL, "observer index outside the DEM");
  return SITING_OK;
}

// Grows workspace slot `s` to at least `bytes` (contents not preserved).
int ws_get(siting_ctx *ctx, Slot s, size_t bytes, void **out) {
  DevBuf &b = ctx->buf[s];
  bytes = std::max<size_t>(bytes, 256);
  if (b.cap < bytes) {
    const size_t grow = std::max(bytes, b.cap + b.cap / 4);
    if (ctx->budget && ctx->held - b.cap + grow > ctx->budget) {
      if (ctx->held - b.cap + bytes > ctx->budget)
        return fail(ctx, SITING_ENOMEM,
                    "workspace of " + std::to_string(ctx->held - b.cap + bytes) +
                        " bytes exceeds the HBM budget of " + std::to_string(ctx->budget));
    }
    const size_t want = (ctx->budget && ctx->held - b.cap + grow > ctx->budget) ? bytes : grow;
    if (b.p) {
      cudaStreamSynchronize(ctx->stream);
      cudaFree(b.p);
      ctx->held -= b.cap;
      b.p = nullptr;
      b.cap = 0;
    }
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(ctx, SITING_ENOMEM,
                  "cudaMalloc of " + std::to_string(want) + " bytes failed: " +
                      cudaGetErrorString(e));
    }
    b.cap = want;
    ctx->held += want;
  }
  *out = b.p;
  return SITING_OK;
}

bool geometry_of(int nrows, int bw, int nwanted0, siting_geometry *g) {
  // siting.cpp:689-695
  const float bs = (float)nrows / (int)((float)nrows / bw + 0.5f);
  const int nb = (int)(nrows / bs + 0.5f);
  const int npb = (int)((float)nwanted0 / (nb * nb) + 0.99999f);
  g->blocksize = bs;
  g->nblocks = nb;
  g->nwantedperblock = npb;
  g->nwanted = npb * nb * nb;
  const int last = nrows - (int)(bs * (nb - 1));
  return last * last >= npb;
}

int validate(const siting_params *p, int lib_form, std::string *msg) {
  // siting.cpp:680-686 (messages kept), then siting.cpp:693-695
  if (p->nrows <= 0 || p->nrows > 20000) return *msg = "Unreasonable value for nrows", 1;
  if (p->roi < 1 || p->roi > 10000) return *msg = "Unreasonable value for roi.", 1;
  if (p->tht < 0 || p->tht > 1000000) return *msg = "Unreasonable value for tht.", 1;
  if (p->oht < 0 || p->oht > 1000000) return *msg = "Unreasonable value for oht.", 1;
  if (p->ntests < 1 || p->ntests > 1000) return *msg = "Unreasonable value for ntests.", 1;
  if (p->bw < (lib_form ? 1 : 10) || p->bw > 2000)
    return *msg = "Unreasonable value for blocksize0.", 1;
  if (p->nwanted0 < (lib_form ? 1 : 100) || p->nwanted0 > 2000000)
    return *msg = "Unreasonable value for nwanted0.", 1;
  if (p->intervis != 0 && p->intervis != 1) return *msg = "Unreasonable value for intervis.", 1;
  siting_geometry g;
  if (!geometry_of(p->nrows, p->bw, p->nwanted0, &g))
    return *msg = "The last block is too small for nwantedperblock.", 1;
  return 0;
}

const siting_plan *tuned_plan(const siting_ctx *ctx, int roi, int ntests) {
  for (const TunedPlan &t : ctx->tuned)
    if (t.roi == roi && (ntests < 0 || t.ntests == ntests)) return &t.plan;
  return nullptr;
}

}  // namespace siting

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

int check_device(siting_ctx *ctx) {
  cudaDeviceProp prop;
  CK(cudaGetDeviceProperties(&prop, ctx->device));
  if (prop.major < 10)
    return fail(ctx, SITING_EDEVICE,
                std::string("device ") + prop.name + " is not sm_100-class; this build targets sm_103a");
  ctx->sm_count = prop.multiProcessorCount;
  return SITING_OK;
}

// Prepares a DemView for a device DEM with pitch n; if its layout cannot be
// tiled by TMA (row bytes not a multiple of 16, or unaligned base), copies it
// into the context's pitched DEM buffer.
int dem_view(siting_ctx *ctx, const uint16_t *d_elevs, int nrows, DemView *v) {
  const bool aligned = (nrows % 8 == 0) && ((uintptr_t)d_elevs % 16 == 0);
  if (aligned) {
    *v = DemView{d_elevs, nrows, nrows, true};
    return SITING_OK;
  }
  const int pitch = (nrows + 7) & ~7;
  void *p;
  int rc = ws_get(ctx, kDem, (size_t)pitch * nrows * 2, &p);
  if (rc) return rc;
  CK(cudaMemcpy2DAsync(p, (size_t)pitch * 2, d_elevs, (size_t)nrows * 2, (size_t)nrows * 2,
                       nrows, cudaMemcpyDeviceToDevice, ctx->stream));
  *v = DemView{static_cast<const uint16_t *>(p), nrows, pitch, true};
  return SITING_OK;
}

int err_flag(siting_ctx *ctx, int **out) {
  void *p;
  int rc = ws_get(ctx, kErr, 256, &p);
  if (rc) return rc;
  *out = static_cast<int *>(p);
  return SITING_OK;
}

int check_err_flag(siting_ctx *ctx, int *d_err) {
  int h = 0;
  CK(cudaMemcpyAsync(&h, d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return check_err_flags(ctx, &h, 1);
}

int vix_dev(siting_ctx *ctx, const DemView &dem, int roi, int oht, int tht, int ntests,
            uint8_t *d_vix, int *d_err) {
  void *tab;
  const size_t tb = vix_table_bytes(roi, ntests);
  const bool cached = ctx->tab_roi == roi && ctx->tab_ntests == ntests && ctx->buf[kTables].cap >= tb;
  int rc = ws_get(ctx, kTables, tb, &tab);
  if (rc) return rc;
  if (!cached) {
    ctx->tab_host.assign(tb, 0);
    vix_fill_tables(ctx->tab_host.data(), roi, ntests);
    CK(cudaMemcpyAsync(tab, ctx->tab_host.data(), tb, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->tab_roi = roi;
    ctx->tab_ntests = ntests;
  }
  const siting_plan *tp = tuned_plan(ctx, roi, ntests);
  const VixPlan plan = tp ? vix_plan_for(dem.nrows, roi, ntests, tp->vix_tile, tp->vix_smem)
                          : vix_default_plan(dem.nrows, roi, ntests);
  CK(launch_vix(dem, roi, oht, tht, ntests, d_vix, tab, plan, d_err, ctx->stream));
  return SITING_OK;
}

int sheds_dev(siting_ctx *ctx, const DemView &dem, int roi, int oht, int tht, int nsheds,
              const int32_t *d_obs, uint64_t *d_sheds, int *d_err) {
  const siting_plan *tp = tuned_plan(ctx, roi, -1);
  const ShedPlan plan = tp ? shed_plan_for(roi, tp->shed_smem) : shed_default_plan(roi);
  CK(launch_sheds(dem, roi, oht, tht, nsheds, d_obs, d_sheds, plan, d_err, ctx->stream));
  return SITING_OK;
}

int site_ctas_for(siting_ctx *ctx, int roi, int nsheds, int nb, int npb, float bs) {
  const siting_plan *tp = tuned_plan(ctx, roi, -1);
  int G = ctx->site_ctas > 0        ? ctx->site_ctas
          : tp && tp->site_ctas > 0 ? std::max(tp->site_ctas, (nsheds + 4095) / 4096)
                                    : site_spread_ctas(site_default_ctas(nsheds, ctx->sm_count), roi,
                                                       nsheds, nb, npb, bs, ctx->sm_count);
  return std::min(G, ctx->sm_count);
}

// Enqueues SITE on device buffers, then copies its outputs and the error flag
// into the context's pinned readout (collected by site_collect after a sync).
int site_enqueue(siting_ctx *ctx, int nrows, int roi, int intervis, int nsheds,
                 const int32_t *d_obs, const uint64_t *d_sheds, float bs, int nb, int npb,
                 uint8_t *d_selected, int *d_err) {
  if (!ctx->h_out) CK(cudaMallocHost(&ctx->h_out, 16 * sizeof(long long)));
  memset(ctx->h_out, 0, 16 * sizeof(long long));
  if (nsheds <= 0) return SITING_OK;
  const int G = site_ctas_for(ctx, roi, nsheds, nb, npb, bs);
  if (!site_supported(roi, nsheds, G))
    return fail(ctx, SITING_EINVAL, "SITE: roi or nsheds beyond the device kernel's limits");
  if (site_smem_bytes(roi, nsheds, G, nb, npb, bs) > 220 * 1024)
    return fail(ctx, SITING_EINVAL, "SITE: shared-memory plan exceeds 220 KB");
  void *p;
  const size_t sb = site_scratch_bytes(nrows, nsheds, G, roi);
  int rc = ws_get(ctx, kSite, sb, &p);
  if (rc) return rc;
  SiteScratch s;
  site_carve_scratch(p, nrows, nsheds, G, roi, &s);
  // zero coverage, slots, barrier and outputs (order is written before read)
  CK(cudaMemsetAsync(p, 0, (unsigned char *)s.order - (unsigned char *)p, ctx->stream));
  CK(cudaMemsetAsync(d_selected, 0, nsheds, ctx->stream));
  CK(launch_site(nrows, roi, intervis, nsheds, d_obs, d_sheds, bs, nb, npb, d_selected, s, G,
                 d_err, ctx->stream));
  CK(cudaMemcpyAsync(ctx->h_out, s.out, (3 + kSitePhases) * sizeof(long long), cudaMemcpyDeviceToHost,
                     ctx->stream));
  ctx->d_last_order = s.order;
  return SITING_OK;
}

// After a stream sync: SITE outputs into res (nusedsheds, cumarea, coverage).
void site_collect(siting_ctx *ctx, int nrows, siting_result *res) {
  ctx->last_nused = (int)ctx->h_out[0];
  if (!res) return;
  res->nusedsheds = (int)ctx->h_out[0];
  res->cumarea = ctx->h_out[1];
  res->coverage = 100.0 * ctx->h_out[1] / ((double)nrows * nrows);
  res->site_rounds = (int)ctx->h_out[2];
}

bool obs_in_range(const int32_t *obs, int nsheds, int nrows) {
  const long long ncell = (long long)nrows * nrows;
  for (int i = 0; i < nsheds; i++)
    if (obs[i] < 0 || obs[i] >= ncell) return false;
  return true;
}

struct EventTimer {
  siting_ctx *ctx;
  float ms(int a, int b) {
    float v = 0.f;
    cudaEventElapsedTime(&v, ctx->ev[a], ctx->ev[b]);
    return v;
  }
};

}  // namespace

namespace siting {

// The DEM is described to TMA as a 3-D tensor {8, pitch/8, rows}: rows of
// 8-element (16-byte) groups.  A box {8, box_w/8, box_h} then lands in shared
// memory as a dense box_h x box_w row-major window of up to 2048 columns (a
// 2-D box is limited to 256 columns), and the innermost coordinate is always
// 0, so every copy starts on a 16-byte boundary.  box_w must be a multiple of
// 8 and window origins columns multiples of 8.
bool make_dem_tensor_map(CUtensorMap *map, const DemView &dem, int box_w, int box_h) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn || !dem.tma_ok || box_w % 8 || box_w > 2048 || box_h > 256 || dem.pitch % 8) return false;
  cuuint64_t dims[3] = {8, (cuuint64_t)dem.pitch / 8, (cuuint64_t)dem.nrows};
  cuuint64_t strides[2] = {16, (cuuint64_t)dem.pitch * 2};
  cuuint32_t box[3] = {8, (cuuint32_t)box_w / 8, (cuuint32_t)box_h};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, const_cast<uint16_t *>(dem.data), dims,
                  strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace siting

extern "C" {

const char *siting_status_string(int status) {
  switch (status) {
    case SITING_OK: return "ok";
    case SITING_EINVAL: return "invalid argument";
    case SITING_ENOMEM: return "out of device memory or HBM budget";
    case SITING_ECUDA: return "CUDA error";
    case SITING_ETIMEOUT: return "device wait timed out";
    case SITING_EIO: return "file input/output error";
    case SITING_EDEVICE: return "no usable device";
    default: return "unknown status";
  }
}

const char *siting_last_error(const siting_ctx *ctx) {
  return ctx ? ctx->err.c_str() : "no context";
}

int siting_validate(const siting_params *p, int lib_form, char *msg, size_t cap) {
  if (!p) return SITING_EINVAL;
  std::string m;
  if (validate(p, lib_form, &m)) {
    if (msg && cap) snprintf(msg, cap, "%s", m.c_str());
    return SITING_EINVAL;
  }
  if (msg && cap) msg[0] = 0;
  return SITING_OK;
}

int siting_block_geometry(int nrows, int bw, int nwanted0, siting_geometry *out) {
  if (!out || nrows <= 0 || bw <= 0 || nwanted0 <= 0) return SITING_EINVAL;
  return geometry_of(nrows, bw, nwanted0, out) ? SITING_OK : SITING_EINVAL;
}

int siting_ctx_create(int device, size_t hbm_budget, siting_ctx **out) {
  if (!out) return SITING_EINVAL;
  *out = nullptr;
  siting_ctx *ctx = new siting_ctx();
  ctx->device = device;
  ctx->budget = hbm_budget;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) {
    delete ctx;
    return SITING_EDEVICE;
  }
  int rc = check_device(ctx);
  if (rc) {
    delete ctx;
    return rc;
  }
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return SITING_ECUDA;
  }
  for (auto &ev : ctx->ev) cudaEventCreate(&ev);
  *out = ctx;
  return SITING_OK;
}

int siting_ctx_trim(siting_ctx *ctx) {
  if (!ctx) return SITING_EINVAL;
  cudaStreamSynchronize(ctx->stream);
  siting::batch_graph_reset(ctx);  // it refers to the workspace
  for (auto &b : ctx->buf) {
    if (b.p) cudaFree(b.p);
    b = DevBuf{};
  }
  ctx->held = 0;
  ctx->d_last_order = nullptr;
  ctx->last_nused = 0;
  return SITING_OK;
}

int siting_ctx_destroy(siting_ctx *ctx) {
  if (!ctx) return SITING_OK;
  cudaSetDevice(ctx->device);
  siting_ctx_trim(ctx);
  for (auto &ev : ctx->ev)
    if (ev) cudaEventDestroy(ev);
  for (auto &ev : ctx->wave_ev) cudaEventDestroy(ev);
  siting::batch_graph_reset(ctx);
  if (ctx->bg_stage) cudaFreeHost(ctx->bg_stage);
  if (ctx->stream2) cudaStreamDestroy(ctx->stream2);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->h_out) cudaFreeHost(ctx->h_out);
  if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
  delete ctx;
  return SITING_OK;
}

int siting_ctx_sync(siting_ctx *ctx) {
  if (!ctx) return SITING_EINVAL;
  CK(cudaStreamSynchronize(ctx->stream));
  return SITING_OK;
}

void *siting_ctx_stream(siting_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

size_t siting_ctx_workspace_bytes(const siting_ctx *ctx) { return ctx ? ctx->held : 0; }

int siting_ctx_set_site_ctas(siting_ctx *ctx, int nctas) {
  if (!ctx || nctas < 0) return SITING_EINVAL;
  ctx->site_ctas = nctas;
  return SITING_OK;
}

int siting_ctx_set_batch_mode(siting_ctx *ctx, int mode) {
  if (!ctx || mode < siting::kBatchAuto || mode > siting::kBatchPerJob) return SITING_EINVAL;
  ctx->batch_mode = mode;
  return SITING_OK;
}

int siting_ctx_set_batch_graphs(siting_ctx *ctx, int on) {
  if (!ctx || (on != 0 && on != 1)) return SITING_EINVAL;
  ctx->batch_graphs = on != 0;
  if (!on) siting::batch_graph_reset(ctx);
  return SITING_OK;
}

int siting_ctx_batch_graph_stats(const siting_ctx *ctx, long long *captures, long long *replays) {
  if (!ctx) return SITING_EINVAL;
  if (captures) *captures = ctx->bg_captures;
  if (replays) *replays = ctx->bg_replays;
  return SITING_OK;
}

// ---- stage entry points, device buffers ------------------------------------

int siting_calc_vix_dev(siting_ctx *ctx, int nrows, const uint16_t *d_elevs, int roi, int oht,
                        int tht, int ntests, uint8_t *d_vix) {
  if (!ctx) return SITING_EINVAL;
  if (nrows <= 0 || roi < 1 || ntests < 1 || ntests > 1000 || !d_elevs || !d_vix)
    return fail(ctx, SITING_EINVAL, "calc_vix: invalid arguments");
  cudaSetDevice(ctx->device);
  int *d_err;
  int rc = err_flag(ctx, &d_err);
  if (rc) return rc;
  CK(cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
  DemView dem;
  if ((rc = dem_view(ctx, d_elevs, nrows, &dem))) return rc;
  return vix_dev(ctx, dem, roi, oht, tht, ntests, d_vix, d_err);
}

int siting_find_max_dev(siting_ctx *ctx, int nrows, uint8_t *d_vix, float blocksize,
                        int nwanted, int nblocks, int nwantedperblock, int32_t *d_obs) {
  if (!ctx) return SITING_EINVAL;
  if (nrows <= 0 || nblocks <= 0 || nwantedperblock <= 0 || !d_vix || !d_obs ||
      nwanted != nblocks * nblocks * nwantedperblock)
    return fail(ctx, SITING_EINVAL, "find_max: invalid arguments");
  cudaSetDevice(ctx->device);
  CK(launch_findmax(d_vix, nrows, blocksize, nblocks, nwantedperblock, d_obs, ctx->stream));
  return SITING_OK;
}

int siting_calc_sheds_dev(siting_ctx *ctx, int nrows, const uint16_t *d_elevs, int roi, int oht,
                          int tht, int nsheds, const int32_t *d_obs, uint64_t *d_sheds) {
  if (!ctx) return SITING_EINVAL;
  if (nrows <= 0 || roi < 1 || nsheds < 0 || !d_elevs || (nsheds && (!d_obs || !d_sheds)))
    return fail(ctx, SITING_EINVAL, "calc_sheds: invalid arguments");
  cudaSetDevice(ctx->device);
  int *d_err;
  int rc = err_flag(ctx, &d_err);
  if (rc) return rc;
  CK(cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
  DemView dem;
  if ((rc = dem_view(ctx, d_elevs, nrows, &dem))) return rc;
  return sheds_dev(ctx, dem, roi, oht, tht, nsheds, d_obs, d_sheds, d_err);
}

// SITE needs the FINDMAX block geometry only to locate candidates near a
// pick; any geometry whose blocks contain their candidates works, so the
// stage-level entry point builds a one-candidate-per-cell grid when called
// without one.
int siting_site_it_dev(siting_ctx *ctx, int nrows, int roi, int intervis, int nsheds,
                       const int32_t *d_obs, const uint64_t *d_sheds, uint8_t *d_selected,
                       siting_result *res) {
  if (!ctx) return SITING_EINVAL;
  if (nrows <= 0 || roi < 1 || nsheds < 0 || (intervis != 0 && intervis != 1) ||
      (nsheds && (!d_obs || !d_sheds || !d_selected)))
    return fail(ctx, SITING_EINVAL, "site_it: invalid arguments");
  cudaSetDevice(ctx->device);
  int *d_err;
  int rc = err_flag(ctx, &d_err);
  if (rc) return rc;
  CK(cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
  // Without block structure: treat the candidate list as one row of blocks of
  // width nrows (every candidate in "block row 0"), so the neighbour search
  // scans all candidates.  Exact, only slower than the geometry-aware path.
  CK(launch_check_obs(d_obs, nsheds, nrows, d_err, ctx->stream));
  if ((rc = check_err_flag(ctx, d_err))) return rc;
  rc = site_enqueue(ctx, nrows, roi, intervis, nsheds, d_obs, d_sheds, (float)nrows, 1, nsheds,
                    d_selected, d_err);
  if (rc) return rc;
  if ((rc = check_err_flag(ctx, d_err))) return rc;
  site_collect(ctx, nrows, res);
  return SITING_OK;
}

// ---- stage entry points, host buffers (synchronous, like siting.cu) ----------

int siting_calc_vix(siting_ctx *ctx, int nrows, const uint16_t *elevs, int roi, int oht, int tht,
                    int ntests, uint8_t *vix) {
  if (!ctx || !elevs || !vix || nrows <= 0) return fail(ctx, SITING_EINVAL, "calc_vix: invalid arguments");
  cudaSetDevice(ctx->device);
  const int pitch = (nrows + 7) & ~7;
  const size_t ncell = (size_t)nrows * nrows;
  void *d_dem, *d_vix;
  int rc;
  if ((rc = ws_get(ctx, kDem, (size_t)pitch * nrows * 2, &d_dem))) return rc;
  if ((rc = ws_get(ctx, kVix, ncell, &d_vix))) return rc;
  int *d_err;
  if ((rc = err_flag(ctx, &d_err))) return rc;
  CK(cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
  CK(cudaMemcpy2DAsync(d_dem, (size_t)pitch * 2, elevs, (size_t)nrows * 2, (size_t)nrows * 2,
                       nrows, cudaMemcpyHostToDevice, ctx->stream));
  DemView dem{static_cast<const uint16_t *>(d_dem), nrows, pitch, true};
  if ((rc = vix_dev(ctx, dem, roi, oht, tht, ntests, static_cast<uint8_t *>(d_vix), d_err)))
    return rc;
  CK(cudaMemcpyAsync(vix, d_vix, ncell, cudaMemcpyDeviceToHost, ctx->stream));
  return check_err_flag(ctx, d_err);
}

int siting_find_max(siting_ctx *ctx, int nrows, uint8_t *vix, float blocksize, int nwanted,
                    int nblocks, int nwantedperblock, int32_t *obs) {
  if (!ctx || !vix || !obs || nrows <= 0) return fail(ctx, SITING_EINVAL, "find_max: invalid arguments");
  cudaSetDevice(ctx->device);
  const size_t ncell = (size_t)nrows * nrows;
  void *d_vix, *d_obs;
  int rc;
  if ((rc = ws_get(ctx, kVix, ncell, &d_vix))) return rc;
  if ((rc = ws_get(ctx, kObs, (size_t)std::max(nwanted, 1) * 4, &d_obs))) return rc;
  CK(cudaMemcpyAsync(d_vix, vix, ncell, cudaMemcpyHostToDevice, ctx->stream));
  if ((rc = siting_find_max_dev(ctx, nrows, static_cast<uint8_t *>(d_vix), blocksize, nwanted,
                                nblocks, nwantedperblock, static_cast<int32_t *>(d_obs))))
    return rc;
  CK(cudaMemcpyAsync(obs, d_obs, (size_t)nwanted * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaMemcpyAsync(vix, d_vix, ncell, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return SITING_OK;
}

int siting_calc_sheds(siting_ctx *ctx, int nrows, const uint16_t *elevs, int roi, int oht,
                      int tht, int nsheds, const int32_t *obs, uint64_t *sheds) {
  if (!ctx || !elevs || nrows <= 0 || roi < 1 || nsheds < 0 || (nsheds && (!obs || !sheds)))
    return fail(ctx, SITING_EINVAL, "calc_sheds: invalid arguments");
  if (!obs_in_range(obs, nsheds, nrows))
    return fail(ctx, SITING_EINVAL, "calc_sheds: observer index outside the DEM");
  cudaSetDevice(ctx->device);
  const int pitch = (nrows + 7) & ~7;
  const int nr = 2 * roi + 1, nwpr = (nr + 63) / 64;
  const size_t shed_bytes = (size_t)nsheds * nr * nwpr * 8;
  void *d_dem, *d_obs, *d_sheds;
  int rc;
  if ((rc = ws_get(ctx, kDem, (size_t)pitch * nrows * 2, &d_dem))) return rc;
  if ((rc = ws_get(ctx, kObs, (size_t)std::max(nsheds, 1) * 4, &d_obs))) return rc;
  if ((rc = ws_get(ctx, kSheds, shed_bytes, &d_sheds))) return rc;
  int *d_err;
  if ((rc = err_flag(ctx, &d_err))) return rc;
  CK(cudaMemsetAsync(d_err, 0, sizeof(int), ctx->stream));
  CK(cudaMemcpy2DAsync(d_dem, (size_t)pitch * 2, elevs, (size_t)nrows * 2, (size_t)nrows * 2,
                       nrows, cudaMemcpyHostToDevice, ctx->stream));
  if (nsheds) CK(cudaMemcpyAsync(d_obs, obs, (size_t)nsheds * 4, cudaMemcpyHostToDevice, ctx->stream));
  DemView dem{static_cast<const uint16_t *>(d_dem), nrows, pitch, true};
  if ((rc = sheds_dev(ctx, dem, roi, oht, tht, nsheds, static_cast<const int32_t *>(d_obs),
                      static_cast<uint64_t *>(d_sheds), d_err)))
    return rc;
  if (nsheds) CK(cudaMemcpyAsync(sheds, d_sheds, shed_bytes, cudaMemcpyDeviceToHost, ctx->stream));
  return check_err_flag(ctx, d_err);
}

int siting_site_it(siting_ctx *ctx, int nrows, int roi, int intervis, int nsheds,
                   const int32_t *obs, const uint64_t *sheds, uint8_t *selected,
                   siting_result *res) {
  if (!ctx || nrows <= 0 || roi < 1 || nsheds < 0 || (nsheds && (!obs || !sheds || !selected)))
    return fail(ctx, SITING_EINVAL, "site_it: invalid arguments");
  if (!obs_in_range(obs, nsheds, nrows))
    return fail(ctx, SITING_EINVAL, "site_it: observer index outside the DEM");
  cudaSetDevice(ctx->device);
  const int nr = 2 * roi + 1, nwpr = (nr + 63) / 64;
  const size_t shed_bytes = (size_t)nsheds * nr * nwpr * 8;
  void *d_obs, *d_sheds, *d_sel;
  int rc;
  if ((rc = ws_get(ctx, kObs, (size_t)std::max(nsheds, 1) * 4, &d_obs))) return rc;
  if ((rc = ws_get(ctx, kSheds, shed_bytes, &d_sheds))) return rc;
  if ((rc = ws_get(ctx, kSel, (size_t)std::max(nsheds, 1), &d_sel))) return rc;
  if (nsheds) {
    CK(cudaMemcpyAsync(d_obs, obs, (size_t)nsheds * 4, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(d_sheds, sheds, shed_bytes, cudaMemcpyHostToDevice, ctx->stream));
  }
  if ((rc = siting_site_it_dev(ctx, nrows, roi, intervis, nsheds,
                               static_cast<const int32_t *>(d_obs),
                               static_cast<const uint64_t *>(d_sheds),
                               static_cast<uint8_t *>(d_sel), res)))
    return rc;
  if (nsheds) CK(cudaMemcpyAsync(selected, d_sel, nsheds, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return SITING_OK;
}

int siting_last_pick_order(siting_ctx *ctx, int32_t *order, int cap, int *count) {
  if (!ctx || !count || cap < 0 || (cap && !order)) return SITING_EINVAL;
  const int n = std::min(cap, ctx->last_nused);
  *count = ctx->d_last_order ? n : 0;
  if (ctx->d_last_order && n > 0) {
    CK(cudaMemcpyAsync(order, ctx->d_last_order, (size_t)n * 4, cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
  }
  return SITING_OK;
}

int siting_last_site_phase_cycles(siting_ctx *ctx, long long *cycles, int n) {
  if (!ctx || !cycles || n < 0) return SITING_EINVAL;
  for (int i = 0; i < n && i < kSitePhases; i++) cycles[i] = ctx->h_out ? ctx->h_out[3 + i] : 0;
  return SITING_OK;
}

// ---- whole pipeline ---------------------------------------------------------

static int run_pipeline(siting_ctx *ctx, const siting_params *p, const DemView &dem,
                        int32_t *d_obs, uint8_t *d_selected, siting_result *res) {
  siting_geometry g;
  geometry_of(p->nrows, p->bw, p->nwanted0, &g);
  const int n = p->nrows;
  const int nr = 2 * p->roi + 1, nwpr = (nr + 63) / 64;
  void *d_vix, *d_sheds;
  int rc;
  if ((rc = ws_get(ctx, kVix, (size_t)n * n, &d_vix))) return rc;
  if ((rc = ws_get(ctx, kSheds, (size_t)g.nwanted * nr * nwpr * 8, &d_sheds))) return rc;
  int *d_err;
  if ((rc = err_flag(ctx, &d_err))) return rc;
  cudaStream_t st = ctx->stream;
  CK(cudaMemsetAsync(d_err, 0, sizeof(int), st));
  CK(cudaEventRecord(ctx->ev[0], st));
  if ((rc = vix_dev(ctx, dem, p->roi, p->oht, p->tht, p->ntests, static_cast<uint8_t *>(d_vix),
                    d_err)))
    return rc;
  CK(cudaEventRecord(ctx->ev[1], st));
  CK(launch_findmax(static_cast<uint8_t *>(d_vix), n, g.blocksize, g.nblocks, g.nwantedperblock,
                    d_obs, st));
  CK(cudaEventRecord(ctx->ev[2], st));
  if ((rc = sheds_dev(ctx, dem, p->roi, p->oht, p->tht, g.nwanted, d_obs,
                      static_cast<uint64_t *>(d_sheds), d_err)))
    return rc;
  CK(cudaEventRecord(ctx->ev[3], st));
  if ((rc = site_enqueue(ctx, n, p->roi, p->intervis, g.nwanted, d_obs,
                        static_cast<const uint64_t *>(d_sheds), g.blocksize, g.nblocks,
                        g.nwantedperblock, d_selected, d_err)))
    return rc;
  CK(cudaEventRecord(ctx->ev[4], st));
  if ((rc = check_err_flag(ctx, d_err))) return rc;  // synchronizes the stream
  if (res) {
    EventTimer et{ctx};
    site_collect(ctx, n, res);
    res->nwanted = g.nwanted;
    res->ms_vix = et.ms(0, 1);
    res->ms_findmax = et.ms(1, 2);
    res->ms_viewshed = et.ms(2, 3);
    res->ms_site = et.ms(3, 4);
  }
  return SITING_OK;
}

int siting_run_dev(siting_ctx *ctx, const siting_params *p, const uint16_t *d_elevs,
                   int32_t *d_obs, uint8_t *d_selected, siting_result *res) {
  if (!ctx || !p || !d_elevs || !d_obs || !d_selected) return fail(ctx, SITING_EINVAL, "run_dev: null argument");
  std::string m;
  if (validate(p, 1, &m)) return fail(ctx, SITING_EINVAL, m);
  cudaSetDevice(ctx->device);
  DemView dem;
  int rc = dem_view(ctx, d_elevs, p->nrows, &dem);
  if (rc) return rc;
  return run_pipeline(ctx, p, dem, d_obs, d_selected, res);
}

int siting_run(siting_ctx *ctx, const siting_params *p, const uint16_t *elevs, int32_t *obs,
               uint8_t *selected, siting_result *res) {
  if (!ctx || !p || !elevs || !obs || !selected) return fail(ctx, SITING_EINVAL, "run: null argument");
  std::string m;
  if (validate(p, 1, &m)) return fail(ctx, SITING_EINVAL, m);
  cudaSetDevice(ctx->device);
  siting_geometry g;
  geometry_of(p->nrows, p->bw, p->nwanted0, &g);
  const int n = p->nrows, pitch = (n + 7) & ~7;
  void *d_dem, *d_obs, *d_sel;
  int rc;
  if ((rc = ws_get(ctx, kDem, (size_t)pitch * n * 2, &d_dem))) return rc;
  if ((rc = ws_get(ctx, kObs, (size_t)g.nwanted * 4, &d_obs))) return rc;
  if ((rc = ws_get(ctx, kSel, (size_t)g.nwanted, &d_sel))) return rc;
  cudaStream_t st = ctx->stream;
  CK(cudaEventRecord(ctx->ev[5], st));
  CK(cudaMemcpy2DAsync(d_dem, (size_t)pitch * 2, elevs, (size_t)n * 2, (size_t)n * 2, n,
                       cudaMemcpyHostToDevice, st));
  DemView dem{static_cast<const uint16_t *>(d_dem), n, pitch, true};
  rc = run_pipeline(ctx, p, dem, static_cast<int32_t *>(d_obs), static_cast<uint8_t *>(d_sel), res);
  if (rc) return rc;
  CK(cudaEventRecord(ctx->ev[6], st));
  CK(cudaMemcpyAsync(obs, d_obs, (size_t)g.nwanted * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(selected, d_sel, (size_t)g.nwanted, cudaMemcpyDeviceToHost, st));
  CK(cudaEventRecord(ctx->ev[7], st));
  CK(cudaStreamSynchronize(st));
  if (res) {
    EventTimer et{ctx};
    res->ms_h2d = et.ms(5, 0);
    res->ms_d2h = et.ms(6, 7);
  }
  return SITING_OK;
}

// ---- files -------------------------------------------------------------------

int siting_read_dem(const char *path, int nrows, uint16_t *out) {
  if (!path || !out || nrows <= 0) return SITING_EINVAL;
  FILE *f = fopen(path, "rb");
  if (!f) return SITING_EIO;
  const size_t want = (size_t)nrows * nrows;
  const size_t got = fread(out, sizeof(uint16_t), want, f);
  fclose(f);
  return got == want ? SITING_OK : SITING_EIO;
}

int siting_write_observers(const char *path, int nrows, int nsheds, const int32_t *obs,
                           const uint8_t *selected) {
  if (!path || nrows <= 0 || nsheds < 0 || (nsheds && (!obs || !selected))) return SITING_EINVAL;
  FILE *f = fopen(path, "wb");
  if (!f) return SITING_EIO;
  for (int i = 0; i < nsheds; i++)
    if (selected[i]) fprintf(f, "%d,%d\n", obs[i] / nrows, obs[i] % nrows);
  return fclose(f) == 0 ? SITING_OK : SITING_EIO;
}

int siting_pinned_alloc(size_t bytes, void **out) {
  if (!out) return SITING_EINVAL;
  return cudaMallocHost(out, bytes) == cudaSuccess ? SITING_OK : SITING_ENOMEM;
}

int siting_pinned_free(void *p) {
  return cudaFreeHost(p) == cudaSuccess ? SITING_OK : SITING_ECUDA;
}

}  // extern "C"
