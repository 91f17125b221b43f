/*
 * mcg_internal.h - context layout shared by the translation units of
 * libmcgb300 (not part of the public ABI).
 */
#ifndef MCG_INTERNAL_H
#define MCG_INTERNAL_H

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "exact_libm.h"
#include "mcg_device.cuh"
#include "mcgb300.h"

/* Per-context state of the batched-slab unit (mcg_batch.cu). */
struct mcg_batch_state {
  int n_slabs = 0, total_cells = 0, max_cells = 0;
  int64_t total_histories = 0;
  std::vector<mcg_slab> slabs;
  std::vector<int32_t> cell_off;
  void *d_slabs = nullptr;  /* mcg_batch_slab_dev[] */
  void *d_items = nullptr;  /* mcg_batch_item[] */
  int n_items = 0, items_cap = 0;
  float4 *d_cells_strict = nullptr, *d_cells_fast = nullptr;
  unsigned long long *d_tally = nullptr;
  unsigned long long *d_item_next = nullptr;
  float min_w = 0.f;
  /* launch shape, chosen by mcg_batch_set_launch or the autotuner */
  int block = 512, tally_mode = 1;
  int defer = 0; /* waiting lanes of the deferred full step, 0: off (mcg_batch_set_deferral) */
  int64_t item_histories = 16384;
  /* history- or event-based; events per pass of the event engine */
  int algorithm = MCG_ALGO_HISTORY, event_steps = 8;
  unsigned long long *d_hist0 = nullptr; /* first history of each slab (event mode) */
  double hist0_fraction = -1.0;          /* fraction of the histories d_hist0 is for */
  /* CUDA graph of one run (memset of the item counter + the kernel) */
  cudaGraphExec_t graph = nullptr;
  bool graph_valid = false;
  int items_built_for = -1; /* item size the list was built for */
};

/* Per-context state of the adjoint unit (mcg_adjoint.cu). */
struct mcg_adj_state {
  float2 *d_aux = nullptr;               /* {w_c, 1/sig_s} per chain cell */
  unsigned long long *d_grad = nullptr;  /* grad_a[n], grad_s[n], loss */
  int n = 0;
  int64_t histories = 0;
  int g_log2 = 36;
};

struct mcg_fit_state; /* mcg_fit.cu */

/* Device buffers of the workers' forms (mcg_worker.cu), kept between calls
 * and grown on demand, so a Worker called repeatedly allocates nothing. */
struct mcg_worker_state {
  void *dev = nullptr;
  size_t bytes = 0;
  cudaStream_t monitor = nullptr; /* progress reads and the abort word */
};

struct mcg_ext {
  mcg_batch_state batch;
  mcg_adj_state adj;
  mcg_fit_state *fit = nullptr;
  mcg_worker_state worker;
};

/* Structure-of-arrays particle buffer of the event-based tracker: per
 * particle the state, the cell index local to its chain or slab, the history
 * (chain) or slab (batched) it belongs to, and its step and scatter counts.
 * In the collision queue the seed is already advanced to the flight
 * sample's state, which determines the sample. */
struct mcg_soa {
  unsigned long long *seed;
  float *x, *mu, *wmc, *res; /* res: the fast weight's rounding residue */
  int32_t *idx, *hid, *nst, *nsc;
};

/* Counters of the event engine, on the device. */
struct mcg_ev_ctl {
  unsigned long long n_in, n_out, n_q;     /* particles in the bank, out, in the queue */
  unsigned long long next, total;          /* histories born so far, of the run */
  unsigned long long birth_base, birth_n;  /* this pass's newborns: slots, count */
  unsigned long long birth_first, passes;
};

/* One slab of the batched form (and of the event engine's slab mode). */
struct mcg_batch_slab_dev {
  int32_t cell_off, m;
  mcg_source src;
};

struct mcg_context {
  int device = 0, mode = MCG_MODE_STRICT;
  int sm_count = 0, smem_optin = 0, cc_major = 0, cc_minor = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.f;
  int last_grid = 0, last_block = 0;
  long long launches = 0;

  /* chain of layers */
  int n_layers = 0, n_cells = 0, cell_lo = 0;
  float min_w = 0.f;
  std::vector<int32_t> layer_start, layer_m;
  std::vector<float> layer_dx, sigs, rates;
  std::vector<float4> cells_strict, cells_fast;
  bool thin = false; /* every cell's sig_a width <= 5e-4 (mcg_step THIN) */
  float4 *d_cells_strict = nullptr, *d_cells_fast = nullptr;
  unsigned long long *d_tally = nullptr;
  int log2_scale = 40;
  unsigned long long *d_counters = nullptr, *d_next = nullptr;

  /* strict libm */
  bool libm_loaded = false;
  mcg_libm_dev libm = {};
  mcg_libm_tab *libm_tab = nullptr;
  uint32_t libm_n_log = 0, libm_n_exp = 0;

  /* particle buffers of the host-pointer entry points */
  mcg_particle *d_part = nullptr;
  int32_t *d_res = nullptr;
  int64_t *d_steps = nullptr, *d_scat = nullptr;
  size_t scratch_cap = 0;

  /* launch shape */
  int block = 0, blocks_per_sm = 0, refill = 8;
  uint32_t max_steps = 1u << 28; /* per-history step limit (MCG_ERR_LIMIT) */
  int tally_mode = 1;            /* MCG_TALLY_SMEM32 */

  /* algorithm: history-based (default) or event-based with K events per pass */
  int algorithm = MCG_ALGO_HISTORY, event_steps = 1, event_passes = 0;
  mcg_soa event_buf[3] = {}; /* bank in, bank out, collision queue */
  size_t event_cap = 0;
  std::vector<void *> event_owned;
  mcg_ev_ctl *event_ctl = nullptr;

  std::vector<void *> owned; /* device allocations freed at destroy */
  mcg_ext *ext = nullptr;
};

int mcg_fail(int code, const char *fmt, ...);
/* cudaMalloc of the geometry set-up (mcg_set_layers, mcg_batch_set); a test
 * can make one of them report cudaErrorMemoryAllocation without attempting
 * it (mcg_testing_fail_allocation). */
cudaError_t mcg_dev_malloc(void **p, size_t bytes);
int mcg_cuda_fail(cudaError_t e, const char *what);
void mcg_cell_params(float sig, float rate, int gi, float dx, float4 &strict, float4 &fast);
int mcg_track_launch(mcg_context *ctx, mcg_particle *d_particles, int64_t n, int32_t *d_results,
                     int64_t *d_steps, int64_t *d_scatters, const mcg_source *src, int64_t first);
int mcg_sync(mcg_context *ctx);
void mcg_ext_destroy(mcg_context *ctx);
int mcg_load_libm(mcg_context *ctx);
extern "C" int mcg_fit_release(mcg_context *ctx);
struct mcg_track_params;
/* Below this many live particles (once the source is exhausted) the event
 * engine finishes the run with one history-based launch. */
inline unsigned long long mcg_event_drain_below(const mcg_context *ctx)
{
  return (unsigned long long)ctx->sm_count * 1024;
}
/* The strict thin-cell step applies: a thin chain, and exception-table
 * thresholds small enough for its test on |yl| (that test implies the
 * midpoint-distance test for thresholds below 0.4; the tables' are about
 * 0.002). */
inline bool mcg_strict_thin(const mcg_context *ctx)
{
  return ctx->thin && ctx->libm.tau_exp_max < 0.25f;
}
int mcg_event_run(mcg_context *ctx, mcg_track_params &P);
int mcg_event_run_slabs(mcg_context *ctx, const float4 *cells, unsigned long long *tally,
                        const void *slabs, const unsigned long long *slab_hist0, int n_slabs,
                        unsigned long long total, float min_w, int steps_per_pass);

#endif
