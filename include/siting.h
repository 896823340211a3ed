/*
 * siting.h — C ABI of the GB300 observer-siting library (libsiting_gb300.so).
 *
 * The reference (wenlili/siting) is one program per run: the CLI
 *   cusite nrows roi height targets bw nwanted intervis inputfile outputfile
 * (siting.cu:746-919, siting.cpp:632-780) calling four C-style stage
 * functions on raw buffers.  This header replaces that boundary with plain
 * extern "C" entry points: pointers and sizes only, an int status instead of
 * exit(1), and a context that owns the CUDA stream and the device workspace.
 *
 * Every stage keeps the reference's argument order and meaning.  Two forms
 * exist for each:
 *   siting_<stage>(...)      host buffers; copies in, runs, copies out and
 *                            returns when the results are in host memory
 *                            (the synchronous behaviour of siting.cu).
 *   siting_<stage>_dev(...)  device buffers; stream-ordered on the context's
 *                            stream, returns after enqueueing.
 * Results are bit-identical to the reference's sequential program (seqsite).
 *
 * Status codes: 0 = success; otherwise a SITING_E* value, and
 * siting_last_error(ctx) returns a message.  Argument checks give the same
 * messages as the reference's die() calls (siting.cpp:680-695).
 */
#ifndef SITING_GB300_H
#define SITING_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SITING_OK 0
#define SITING_EINVAL 1   /* argument outside the accepted range */
#define SITING_ENOMEM 2   /* device allocation failed or HBM budget exceeded */
#define SITING_ECUDA 3    /* CUDA runtime error */
#define SITING_ETIMEOUT 4 /* a bounded device wait expired (no fault) */
#define SITING_EIO 5      /* file input/output */
#define SITING_EDEVICE 6  /* no usable device / unsupported architecture */

typedef struct siting_ctx siting_ctx;

/* One siting job: the nine CLI arguments minus the two file names
 * (siting.cpp:668-674; oht = tht = height there). */
typedef struct siting_params {
  int nrows;    /* DEM side, cells */
  int roi;      /* radius of interest, cells */
  int oht;      /* observer height above ground */
  int tht;      /* target height above ground */
  int ntests;   /* random targets per cell ("targets") */
  int bw;       /* requested block width ("bw", blocksize0) */
  int nwanted0; /* requested tentative observers ("nwanted") */
  int intervis; /* 1: new observers must be visible from earlier ones */
} siting_params;

/* Perturbed block geometry of siting.cpp:688-695. */
typedef struct siting_geometry {
  float blocksize;
  int nblocks;
  int nwantedperblock;
  int nwanted;
} siting_geometry;

/* Launch plan of one job (tile shapes and CTA counts); 0 / -1 fields take
 * the library default.  Results never depend on the plan. */
typedef struct siting_plan {
  int vix_tile;     /* VIX cell tile side: 16, 32 or 64 (0 = default) */
  int vix_smem;     /* 1: stage the DEM halo by TMA, 0: read through L1, -1: default */
  int shed_smem;    /* VIEWSHED window: 1 two half windows staged by TMA, one
                       CTA each (up to roi 151, else as 2), 2 the whole window
                       in one CTA, staged up to roi 100, 0 the whole window
                       through L1, -1 default (1 for roi 60..151, else 2) */
  int site_ctas;    /* CTAs of the job's SITE group (0 = default) */
} siting_plan;

/* Outcome and per-stage device times of one job. */
typedef struct siting_result {
  int nusedsheds;    /* observers selected (siting.cpp:617) */
  long long cumarea; /* cells covered by the selected viewsheds */
  double coverage;   /* 100.0 * cumarea / nrows^2, as printed by siting.cpp:617 */
  int nwanted;       /* tentative observers after the geometry perturbation */
  float ms_vix, ms_findmax, ms_viewshed, ms_site; /* CUDA-event stage times */
  float ms_h2d, ms_d2h;                           /* copies (host forms) */
  int site_rounds;   /* greedy rounds run on the device */
} siting_result;

/* ---- errors ----------------------------------------------------------- */
const char *siting_status_string(int status);
/* Message of the last failing call on ctx (never NULL). */
const char *siting_last_error(const siting_ctx *ctx);

/* ---- validation and geometry (no device needed) ------------------------ */
/* Range checks of siting.cpp:680-686 plus the last-block check of
 * siting.cpp:693-695; writes the reference's message to msg on failure.
 * lib_form != 0 accepts the library-only relaxations (bw >= 1, nwanted0 >= 1)
 * used by the batched and serving workloads. */
int siting_validate(const siting_params *p, int lib_form, char *msg,
                    size_t msg_cap);
/* Block geometry of siting.cpp:688-695. */
int siting_block_geometry(int nrows, int bw, int nwanted0,
                          siting_geometry *out);

/* ---- context ------------------------------------------------------------ */
/* Creates a context on `device` with its own non-blocking stream.  hbm_budget
 * caps the workspace bytes the context may hold (0 = no cap). */
int siting_ctx_create(int device, size_t hbm_budget, siting_ctx **out);
int siting_ctx_destroy(siting_ctx *ctx);
/* Waits for all work enqueued on the context's stream. */
int siting_ctx_sync(siting_ctx *ctx);
/* The context's cudaStream_t, as an opaque pointer. */
void *siting_ctx_stream(siting_ctx *ctx);
/* Workspace bytes currently held. */
size_t siting_ctx_workspace_bytes(const siting_ctx *ctx);
/* Releases the workspace (buffers are re-created on demand). */
int siting_ctx_trim(siting_ctx *ctx);
/* Tuning knob: CTAs of the SITE kernel (0 = automatic, capped at the SM
 * count).  Results do not depend on it. */
int siting_ctx_set_site_ctas(siting_ctx *ctx, int nctas);
/* Tuning knob of the batched form (no counterpart in the reference): how a
 * batch launches VIX and FINDMAX.  1 = for the jobs of each SITE launch, one
 * grid over their (job, tile) VIX items (two when some halos are staged and
 * some not) and one over their (job, block) FINDMAX items, 2 = one VIX and
 * one FINDMAX launch per job, 0 = automatic: 1 for the SITE launches whose
 * jobs average at most 2^18 cells, else 2.  Results do not depend on it. */
int siting_ctx_set_batch_mode(siting_ctx *ctx, int mode);
/* Device-resident batches (siting_run_batch_dev) whose VIX and FINDMAX all
 * run as grids over many jobs (see siting_ctx_set_batch_mode) run as CUDA
 * graphs (no counterpart in the reference): the first call of a batch
 * captures its copies and launches, a later call with the same jobs, buffers
 * and workspace replays the graph (on = 1, the default); 0 launches every
 * call directly.  Results do not depend on it. */
int siting_ctx_set_batch_graphs(siting_ctx *ctx, int on);
/* Graphs captured and replayed by the context's batches so far. */
int siting_ctx_batch_graph_stats(const siting_ctx *ctx, long long *captures,
                                 long long *replays);
/* Page-locked host memory for fast copies (cudaMallocHost / cudaFreeHost). */
int siting_pinned_alloc(size_t bytes, void **out);
int siting_pinned_free(void *p);

/* ---- stage 1: VIX (replaces calc_vix, siting.cpp:192 / siting.cu:133) --- */
int siting_calc_vix(siting_ctx *ctx, int nrows, const uint16_t *elevs,
                    int roi, int oht, int tht, int ntests, uint8_t *vix);
int siting_calc_vix_dev(siting_ctx *ctx, int nrows, const uint16_t *d_elevs,
                        int roi, int oht, int tht, int ntests, uint8_t *d_vix);

/* ---- stage 2: FINDMAX (replaces find_max, siting.cpp:235 / siting.cu:226).
 * vix is modified as in siting.cpp: each winner's entry is cleared. -------- */
int siting_find_max(siting_ctx *ctx, int nrows, uint8_t *vix, float blocksize,
                    int nwanted, int nblocks, int nwantedperblock,
                    int32_t *obs);
int siting_find_max_dev(siting_ctx *ctx, int nrows, uint8_t *d_vix,
                        float blocksize, int nwanted, int nblocks,
                        int nwantedperblock, int32_t *d_obs);

/* ---- stage 3: VIEWSHED (replaces calc_sheds, siting.cpp:349 /
 * siting.cu:336).  sheds: nsheds * (2roi+1) * ceil((2roi+1)/64) words,
 * bit (r,c) at word r*nwpr + c/64, bit 63 - c%64 (siting.cpp:247-250). ----- */
int siting_calc_sheds(siting_ctx *ctx, int nrows, const uint16_t *elevs,
                      int roi, int oht, int tht, int nsheds,
                      const int32_t *obs, uint64_t *sheds);
int siting_calc_sheds_dev(siting_ctx *ctx, int nrows, const uint16_t *d_elevs,
                          int roi, int oht, int tht, int nsheds,
                          const int32_t *d_obs, uint64_t *d_sheds);

/* ---- stage 4: SITE (replaces site_it, siting.cpp:501 / siting.cu:596).
 * selected[i] = 1 for chosen observers.  res may be NULL. ---------------- */
int siting_site_it(siting_ctx *ctx, int nrows, int roi, int intervis,
                   int nsheds, const int32_t *obs, const uint64_t *sheds,
                   uint8_t *selected, siting_result *res);
int siting_site_it_dev(siting_ctx *ctx, int nrows, int roi, int intervis,
                       int nsheds, const int32_t *d_obs,
                       const uint64_t *d_sheds, uint8_t *d_selected,
                       siting_result *res);

/* Picks of the context's last SITE run in the order they were made (the
 * sequence the reference's commented-out per-round log prints,
 * siting.cpp:610-615).  Writes min(cap, nusedsheds) entries to order (host)
 * and returns that count in *count. */
int siting_last_pick_order(siting_ctx *ctx, int32_t *order, int cap, int *count);

/* Tracing: device clock cycles CTA 0 spent in each phase of the last SITE
 * run, summed over rounds: 0 set-up, 1 publishing its top keys, 2 round
 * barrier, 9 loading the published lists and keeping the exactly ordered
 * keys, 10 ranking them, 3 choosing the round's picks, 4 finding the
 * candidates near the picks (and, in large rounds, this CTA's rows of the
 * picks' new bits), 11 the barrier after those rows (large rounds), 5
 * compacting the pairs, 6 gain deltas, 12 intervis cut, 7 second barrier and
 * the smallest cut, 8 applying the picks.  Writes min(n, 13) values. */
int siting_last_site_phase_cycles(siting_ctx *ctx, long long *cycles, int n);

/* SITE on device buffers without allocating any memory.  No counterpart in
 * the reference: it is for callers that cannot allocate device memory on
 * their call path (a serving loop that reserves its HBM budget at start-up,
 * or an application whose memory pool already owns the device's memory).
 * Scratch comes from a 16 MiB array in the library's device image, held by
 * every GPU that loads the library until the process exits; a job whose
 * scratch would exceed it returns SITING_ENOMEM, and invalid arguments return
 * SITING_EINVAL (an observer index outside the DEM is found before SITE
 * reads through it).  Runs on `stream` (a cudaStream_t, NULL = default
 * stream) of the current device, synchronises that stream twice and returns
 * when the results are in `selected` and res.  Each call looks up the array's
 * device address on the current device.  All calls share the array: calls
 * that overlap on the GPU race and must be serialised by the caller. */
int siting_site_it_noalloc(int nrows, int roi, int intervis, int nsheds,
                           const int32_t *d_obs, const uint64_t *d_sheds,
                           uint8_t *d_selected, void *stream,
                           siting_result *res);

/* ---- whole pipeline (replaces main's stage sequence, siting.cpp:737-759).
 * obs and selected receive nwanted entries (see siting_block_geometry). --- */
int siting_run(siting_ctx *ctx, const siting_params *p, const uint16_t *elevs,
               int32_t *obs, uint8_t *selected, siting_result *res);
/* Device-resident form: d_elevs is nrows*nrows uint16 on the device; obs and
 * selected (device) receive nwanted entries.  Intermediate VIX and viewshed
 * arrays stay in the context's workspace. */
int siting_run_dev(siting_ctx *ctx, const siting_params *p,
                   const uint16_t *d_elevs, int32_t *d_obs,
                   uint8_t *d_selected, siting_result *res);

/* ---- batched form --------------------------------------------------------
 * Runs `njobs` independent jobs (DEMs of any sizes and parameters) as one
 * batch: the jobs' VIX, FINDMAX and VIEWSHED kernels are enqueued on the
 * context's stream (VIX and FINDMAX of small jobs as grids over many jobs'
 * items, see siting_ctx_set_batch_mode), and the greedy SITE selections of
 * many jobs run concurrently in shared cooperative launches (each job's CTA
 * group with its own barrier and scratch) on a second stream, overlapping the
 * later jobs' stages.  The device-resident form runs as a CUDA graph
 * (siting_ctx_set_batch_graphs).  elevs[j] is job j's row-major uint16 DEM on
 * the host; obs[j] and selected[j] receive nwanted entries.  plans may be
 * NULL.  Each job's results equal siting_run's on the same input.  The
 * phase times in results are the batch's: ms_vix covers VIX, FINDMAX and
 * VIEWSHED of every job, ms_site the SITE work left after them (SITE
 * launches overlap the later jobs' stages). */
int siting_run_batch(siting_ctx *ctx, int njobs, const siting_params *params,
                     const uint16_t *const *elevs, int32_t *const *obs,
                     uint8_t *const *selected, siting_result *results,
                     const siting_plan *plans);
/* Device-resident form: DEMs, observers and selections in device memory. */
int siting_run_batch_dev(siting_ctx *ctx, int njobs, const siting_params *params,
                         const uint16_t *const *d_elevs, int32_t *const *d_obs,
                         uint8_t *const *d_selected, siting_result *results,
                         const siting_plan *plans);

/* Device workspace siting_run_batch would take for these jobs (no device
 * work; plans may be NULL).  No counterpart in the reference. */
int siting_batch_workspace_bytes(siting_ctx *ctx, int njobs,
                                 const siting_params *params,
                                 const siting_plan *plans, size_t *bytes);

/* ---- self-test -----------------------------------------------------------
 * No counterpart in the reference.  Runs one of the device's bounded waits
 * (which 0: the SITE group barrier; 1: the TMA completion mbarrier) against a
 * condition that is never met, giving up after max_cycles clock cycles
 * (1..2^31).  Returns SITING_ETIMEOUT when the wait expired and reported as
 * designed; the context stays usable.  Failure detection is tested this way
 * instead of by faulting the device. */
int siting_selftest_wait(siting_ctx *ctx, int which, long long max_cycles);

/* ---- autotuner -----------------------------------------------------------
 * No counterpart in the reference.  Times the launch plans of each stage
 * (VIX tile 16/32/64 with the halo staged or read through L1; VIEWSHED half
 * windows, the whole window staged, or read through L1; SITE group size when the sample is the whole DEM) on the
 * top-left sample_rows x sample_rows corner of the host DEM elevs (0 = 1024)
 * with p's parameters, and keeps the fastest for (roi, ntests) in the
 * context: later calls given no plan (siting_run*, siting_run_batch* with
 * plans == NULL, the stage functions) use it.  *best (may be NULL) receives
 * it.  Results never depend on the plan. */
int siting_autotune(siting_ctx *ctx, const siting_params *p,
                    const uint16_t *elevs, int sample_rows, siting_plan *best);
/* Keeps *plan for jobs with this (roi, ntests) as if the autotuner had chosen
 * it (a plan tuned in an earlier process, say); the stage functions take the
 * plan of their roi whatever its ntests.  SITING_EINVAL for a field out of
 * range. */
int siting_autotune_set(siting_ctx *ctx, int roi, int ntests, const siting_plan *plan);
/* Forgets every autotuned plan of the context. */
int siting_autotune_clear(siting_ctx *ctx);

/* ---- serving loop --------------------------------------------------------
 * No counterpart in the reference (one process per DEM there).  A server
 * owns a context, a device arena of hbm_budget bytes (allocated at creation)
 * and a worker thread, and keeps up to max_batch_jobs jobs in flight at once:
 * the head of the arrival queue is admitted as soon as its workspace fits in
 * the free part of the arena, while other jobs are on the GPU, and its
 * kernels overlap theirs: its stages run on stage streams whose priority
 * rises as jobs get smaller, its selection on the highest-priority stream as
 * soon as its stages are done, so selections run in the order their stages
 * finish.  A job that alone exceeds the budget is refused at submission
 * (SITING_ENOMEM).  The serving path never allocates device memory.  Each
 * job's results equal siting_run's on the same input. */
typedef struct siting_server siting_server;

typedef struct {
  int status;                 /* SITING_OK or the job's error */
  siting_result result;       /* counts only: no phase times */
  double t_submit, t_start, t_done; /* seconds since the server started;
                                       t_start: admitted to the GPU */
  int batch_id, batch_jobs;   /* the admission that started the job, and the
                                 jobs in flight right after it */
  char error[160];            /* message when status != SITING_OK */
} siting_job_info;

typedef struct {
  long long submitted, completed, refused, batches, pending;
                              /* batches: admissions of one or more jobs */
  size_t peak_workspace;      /* most arena bytes in use at once */
  double busy_s;              /* time with at least one job in flight */
} siting_server_stats;

/* hbm_budget in bytes (required); max_batch_jobs (jobs in flight at once)
 * <= 0 means 64; reserve is accepted for compatibility (the arena is always
 * allocated at creation). */
int siting_server_create(int device, size_t hbm_budget, int max_batch_jobs,
                         int reserve, siting_server **out);
/* Drains the queue, stops the worker and frees the context. */
int siting_server_destroy(siting_server *s);
/* Queues one job.  elevs is the host DEM with a row pitch of pitch elements
 * (0 = nrows), so a window of a larger raster can be submitted without a
 * copy; elevs, obs and selected (nwanted entries each) must stay valid until
 * the job is waited for.  *ticket identifies the job. */
int siting_server_submit(siting_server *s, const siting_params *p,
                         const uint16_t *elevs, int pitch, int32_t *obs,
                         uint8_t *selected, long long *ticket);
/* Waits up to timeout_s seconds (< 0: forever) for a job.  SITING_OK and
 * *info once it is done (the ticket is then released), SITING_ETIMEOUT if it
 * is still queued or running, SITING_EINVAL for an unknown ticket. */
int siting_server_wait(siting_server *s, long long ticket, double timeout_s,
                       siting_job_info *info);
int siting_server_stats_get(siting_server *s, siting_server_stats *st);

/* ---- files (the reference's input and output formats) ------------------ */
/* Reads exactly nrows*nrows uint16 (siting.cpp:726-730). */
int siting_read_dem(const char *path, int nrows, uint16_t *out);
/* Writes "x,y\n" per selected observer in index order (siting.cpp:761-765). */
int siting_write_observers(const char *path, int nrows, int nsheds,
                           const int32_t *obs, const uint8_t *selected);

/* ---- synthetic terrain ------------------------------------------------- */
/* Seeded fBm value noise (optionally blended with ridged noise), min-max
 * scaled to [0, range_max], row-major uint16.  Host only; deterministic
 * across hosts. */
int siting_fbm_dem(uint16_t *out, int nrows, uint64_t seed, int octaves,
                   double persistence, double lacunarity,
                   double base_wavelength, double ridged_weight,
                   int range_max);

#ifdef __cplusplus
}
#endif
#endif /* SITING_GB300_H */
