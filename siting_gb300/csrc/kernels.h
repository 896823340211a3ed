// Host-side launch interface of the four stage kernels (internal to the
// library; the public boundary is include/siting.h).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace siting {

// ---- error flags written by kernels (never a trap or a fault) -------------
enum : int {
  kErrTmaTimeout = 1,      // an mbarrier wait for a TMA tile expired
  kErrBarrierTimeout = 2,  // a grid-group barrier wait expired
  kErrSiteMismatch = 4,    // SITE self-check: pick gain != its new coverage
  kErrCapacity = 8,        // a per-CTA work list overflowed its capacity
  kErrBadInput = 16,       // an observer index outside the DEM
};


// A DEM resident on the device: row-major uint16, `pitch` elements per row.
struct DemView {
  const uint16_t *data;
  int nrows;
  int pitch;
  bool tma_ok;  // pitch*2 % 16 == 0 and data 16-byte aligned
};

// Encodes a 2-D TMA descriptor over a DEM with box {box_w, box_h}.
bool make_dem_tensor_map(CUtensorMap *map, const DemView &dem, int box_w, int box_h);

// ---- VIX -------------------------------------------------------------------
struct VixPlan {
  int tile;       // cells per tile side
  int threads;    // threads per CTA
  bool use_smem;  // stage the halo tile in shared memory by TMA
};
// Device tables of the VIX stage (host-computed with the reference's
// expressions): jump[2k], jump[2k+1] = LCG multiplier/increment of k+1 steps
// for k < 2*ntests; rtab[d] = (float)(1.0/d); vtab[v] = VIX byte of v hits.
size_t vix_table_bytes(int roi, int ntests);
void vix_fill_tables(void *host_buf, int roi, int ntests);
VixPlan vix_default_plan(int nrows, int roi, int ntests);
// A caller's plan (tile 16/32/64, smem 1/0/-1), corrected to one that fits.
VixPlan vix_plan_for(int nrows, int roi, int ntests, int tile, int smem);
size_t vix_smem_bytes(const VixPlan &p, int roi, int ntests);
cudaError_t launch_vix(const DemView &dem, int roi, int oht, int tht, int ntests,
                       uint8_t *vix, const void *d_tables, const VixPlan &plan, int *d_err,
                       cudaStream_t st);

// ---- FINDMAX -----------------------------------------------------------------
cudaError_t launch_findmax(uint8_t *vix, int nrows, float blocksize, int nblocks, int npb,
                           int32_t *obs, cudaStream_t st);

// Sets kErrBadInput in *d_err if any obs[i] is outside [0, nrows^2).
cudaError_t launch_check_obs(const int32_t *obs, int nsheds, int nrows, int *d_err,
                             cudaStream_t st);

// ---- VIEWSHED -----------------------------------------------------------------
struct ShedPlan {
  int threads;
  bool use_smem;  // stage the (2roi+1)^2 window by TMA
  bool half;      // two CTAs an observer, each staging the rows on one side of it
};
ShedPlan shed_default_plan(int roi);
ShedPlan shed_plan_for(int roi, int smem);
size_t shed_smem_bytes(const ShedPlan &p, int roi);
cudaError_t launch_sheds(const DemView &dem, int roi, int oht, int tht, int nsheds,
                         const int32_t *obs, uint64_t *sheds, const ShedPlan &plan, int *d_err,
                         cudaStream_t st);

// ---- many jobs per launch (batched form) ---------------------------------------
// One job of a multi-job launch: its DEM, VIX and FINDMAX arguments and buffers.
struct StageJob {
  DemView dem;
  int roi, oht, tht, ntests;
  uint8_t *vix;
  const void *vix_tables;  // vix_fill_tables layout on the device
  VixPlan vplan;
  float bs;                // FINDMAX block geometry
  int nb, npb;
  int32_t *obs;
  int *err;
};
// Jobs per multi-job launch (the job table is the kernel's parameters).
constexpr int kStageQueueMaxJobs = 64;
// VIX of every tile of `jobs`: one grid over the (job, tile) items of the
// jobs whose halo is staged and one over the others (more when a kind has
// over kStageQueueMaxJobs jobs).
cudaError_t launch_vix_queue(const StageJob *jobs, int njobs, cudaStream_t st);
// FINDMAX of every block of `jobs`: one grid over the (job, block) items.
cudaError_t launch_findmax_queue(const StageJob *jobs, int njobs, cudaStream_t st);

// ---- SITE -----------------------------------------------------------------------
// Scratch layout of one SITE job (device, carved from one allocation).
struct SiteScratch {
  uint64_t *cum;             // nrows * ceil(nrows/64) words, zeroed before launch
  uint64_t *nbits;           // the round's new bits of each pick: [64][nr][nwpr+1] words
  unsigned char *nmask;      // [64][nr]: bit j set when word j of that new-bit row is nonzero
  unsigned long long *topk;  // [2][nctas][top-K] x {key, cell}: published top keys
  int *cuts;                 // [2][nctas]: per-CTA prefix cut (intervis)
  int *ncount;               // [2][64]: popcount of each pick's new bits (self-check)
  unsigned *bar;             // group barrier counter, zeroed
  long long *out;            // [0] nused, [1] cumarea, [2] rounds, [3..15] phase cycles
  int32_t *order;            // nsheds: picks in order
  int32_t *gains;            // nsheds: round-1 gains (site_score_kernel)
  void *table;               // job table of a one-job launch (site_job_table_bytes)
};

// Phases of the SITE tracing clocks (siting_last_site_phase_cycles).
constexpr int kSitePhases = 13;

// One SITE job (one DEM) of a launch.
struct SiteJob {
  int nrows, roi, intervis, nsheds;
  const int32_t *obs;
  const uint64_t *sheds;
  float blocksize;
  int nblocks, npb;
  uint8_t *selected;
  SiteScratch scratch;  // zeroed as site_dev does before the launch
  int nctas;
  int *err;
};
// Device bytes of a job table for `njobs` jobs and `total_ctas` CTAs.
size_t site_job_table_bytes(int njobs, int total_ctas);
// Launches the round-1 scoring of every job, then one cooperative launch in
// which each job's CTAs form their own group.  The sum of nctas must not
// exceed the number of co-resident CTAs (one per SM).
// h_stage: page-locked host bytes for the job table (site_job_table_bytes),
// kept unchanged until the copy has run; NULL stages through pageable memory.
cudaError_t launch_site_jobs(const SiteJob *jobs, int njobs, void *d_table, void *h_stage,
                             cudaStream_t st);
size_t site_scratch_bytes(int nrows, int nsheds, int nctas, int roi);
void site_carve_scratch(void *base, int nrows, int nsheds, int nctas, int roi, SiteScratch *s);
int site_default_ctas(int nsheds, int sm_count);
// The CTA count near G0 that spreads a pick's neighbourhood most evenly over
// the CTAs for the job's block geometry (nb blocks a row, npb candidates each).
int site_spread_ctas(int G0, int roi, int nsheds, int nb, int npb, float bs, int sm_count);
// Smallest covered-cell count at which the reference's 95% stop test holds.
long long site_stop_area(int nrows);
size_t site_smem_bytes(int roi, int nsheds, int nctas, int nblocks, int npb, float blocksize);
bool site_supported(int roi, int nsheds, int nctas);
cudaError_t launch_site(int nrows, int roi, int intervis, int nsheds, const int32_t *obs,
                        const uint64_t *sheds, float blocksize, int nblocks, int npb,
                        uint8_t *selected, const SiteScratch &s, int nctas, int *d_err,
                        cudaStream_t st);

}  // namespace siting
