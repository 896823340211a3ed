// Batched form: launch planning shared by siting_run_batch and the serving
// loop's admission control.
#pragma once

#include <string>
#include <vector>

#include "kernels.h"
#include "siting.h"

struct siting_ctx;

namespace siting {

struct Job {
  siting_params p;
  siting_geometry g;
  int n, pitch, nr, nwpr, G;
  bool auto_G;  // SITE group size chosen here (not by the caller's plan)
  size_t per;
  VixPlan vp;
  ShedPlan sp;
  // workspace offsets
  size_t o_dem, o_vix, o_obs, o_sel, o_sheds, o_tab, o_site, o_err;
  size_t site_zero;  // bytes of the SITE scratch that start at zero
};


struct BatchPlan {
  std::vector<Job> jobs;
  std::vector<std::vector<int>> waves;  // SITE launches: job indices
  std::vector<int> wave_ctas;
  std::vector<size_t> o_wtab;           // per wave: offset of its job table
  size_t ws = 0;                        // device workspace bytes
  size_t tab_bytes = 0, wtab_bytes = 0, o_tabs = 0, o_wtabs = 0;
};

// Plans a batch for a device of sm_count SMs: host arithmetic only, safe to
// call from any thread.  SITING_EINVAL and a message for an invalid job.
int plan_batch(int sm_count, int njobs, const siting_params *params, const siting_plan *plans,
               BatchPlan *bp, std::string *err);

// Drops the context's captured batch graph (its workspace may be gone).
void batch_graph_reset(siting_ctx *ctx);

// Runs a batch.  src_pitch (elements, may be null; 0 = nrows) is the row
// pitch of each job's DEM; host_io selects host or device buffers.
int run_batch(siting_ctx *ctx, int njobs, const siting_params *params,
              const uint16_t *const *elevs, const int *src_pitch, bool host_io,
              int32_t *const *obs_out, uint8_t *const *sel_out, siting_result *results,
              const siting_plan *plans);

}  // namespace siting
