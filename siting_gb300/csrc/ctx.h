// Internal: the siting context and helpers shared by the C ABI's files.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "kernels.h"
#include "siting.h"

namespace siting {

struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
};

enum Slot { kDem, kVix, kObs, kSheds, kTables, kSite, kSel, kErr, kBatch, kNumSlots };

// How a batch launches VIX and FINDMAX (siting_ctx_set_batch_mode).
enum BatchMode { kBatchAuto = 0, kBatchMerged = 1, kBatchPerJob = 2 };

// Launch plan measured fastest by siting_autotune for (roi, ntests).
struct TunedPlan {
  int roi, ntests;
  siting_plan plan;
};

}  // namespace siting

struct siting_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  size_t budget = 0;
  size_t held = 0;
  siting::DevBuf buf[siting::kNumSlots];
  cudaEvent_t ev[8] = {};
  std::string err;
  int site_ctas = 0;                  // 0 = automatic
  int batch_mode = 0;                 // siting::BatchMode
  int tab_roi = -1, tab_ntests = -1;  // VIX tables currently on the device
  std::vector<unsigned char> tab_host;
  long long *h_out = nullptr;         // pinned: SITE outputs
  int32_t *d_last_order = nullptr;    // pick order of the last SITE run
  int last_nused = 0;
  unsigned char *h_stage = nullptr;   // pinned staging for batch uploads/readouts
  size_t h_stage_cap = 0;
  std::vector<siting::TunedPlan> tuned;  // autotuned plans, used when no plan is given
  cudaStream_t stream2 = nullptr;         // batches: SITE launches, overlapping `stream`
  std::vector<cudaEvent_t> wave_ev;       // batches: one per SITE launch
  bool batch_graphs = true;               // device-resident batches run as CUDA graphs
  cudaGraphExec_t bg_exec = nullptr;      // the last captured batch
  std::vector<unsigned char> bg_key;      // its jobs, buffers and workspace
  unsigned char *bg_stage = nullptr;      // its pinned host staging
  size_t bg_stage_cap = 0;
  long long bg_captures = 0, bg_replays = 0;
};

namespace siting {

int fail(siting_ctx *ctx, int code, const std::string &msg);
int cuda_fail(siting_ctx *ctx, cudaError_t e, const char *what);
// Grows workspace slot `s` to at least `bytes` (contents not preserved).
int ws_get(siting_ctx *ctx, Slot s, size_t bytes, void **out);
// Pinned host staging of at least `bytes`.
int stage_get(siting_ctx *ctx, size_t bytes, unsigned char **out);
bool geometry_of(int nrows, int bw, int nwanted0, siting_geometry *g);
int validate(const siting_params *p, int lib_form, std::string *msg);
int check_err_flags(siting_ctx *ctx, const int *h_flags, int n);
// The autotuned plan for (roi, ntests), or for roi alone when ntests < 0
// (the VIEWSHED and SITE plans do not depend on ntests); null if none.
const siting_plan *tuned_plan(const siting_ctx *ctx, int roi, int ntests);

}  // namespace siting

#define CK(call)                                                        \
  do {                                                                  \
    cudaError_t e_ = (call);                                            \
    if (e_ != cudaSuccess) return siting::cuda_fail(ctx, e_, #call);    \
  } while (0)
