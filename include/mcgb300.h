/*
 * mcgb300.h - C ABI of the GB300 particle-history tracker (libmcgb300.so).
 *
 * Drop-in for the hot path of lkskstlr/mc-mpi: Layer::simulate with its
 * per-cell weights_absorbed tally (src/layer.cpp:123-361), the GPU seam
 * cusimulate (include/culayer/culayer.hpp:6-13, src/culayer.cu:41-92) and the
 * inter-layer particle hand-over of the sync/async/rma workers
 * (src/worker_sync.cpp:41-120, src/async_comm.cpp, src/rma_comm.cpp).
 *
 * Conventions
 *  - Every function but cusimulate returns an int status (MCG_OK = 0); the
 *    message of the last failure on the calling thread is mcg_last_error().
 *  - Pointers named h_* are host memory, d_* device memory of the context's
 *    GPU; sizes are element counts.
 *  - A context owns its device buffers and one CUDA stream; calls on one
 *    context are stream-ordered and synchronous unless named *_async.  A
 *    context is used by one host thread at a time (like a Layer).
 *  - Cells are indexed globally (Particle::index).  A context holds one chain
 *    of contiguous layers; a history ends when its weight drops below the
 *    minimum (result 0) or it leaves the chain (result -1 left, +1 right).
 *  - Tallies are 64-bit fixed point: each deposit dw adds llrint(dw * 2^S);
 *    the sums are exact, so results do not depend on thread order.
 */
#ifndef MCGB300_H
#define MCGB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Particle, byte-compatible with include/types/particle.hpp:7-17 (24 B). */
typedef struct mcg_particle {
  uint64_t seed;
  float x;
  float mu;
  float wmc;
  int32_t index;
} mcg_particle;

enum mcg_status {
  MCG_OK = 0,
  MCG_ERR_ARG = 1,      /* invalid argument */
  MCG_ERR_CUDA = 2,     /* CUDA runtime error */
  MCG_ERR_OVERFLOW = 3, /* a hand-over queue or fixed-size buffer overflowed */
  MCG_ERR_TIMEOUT = 4,  /* a bounded device-side wait gave up */
  MCG_ERR_STATE = 5,    /* call out of order (no layers set, ...) */
  MCG_ERR_TABLES = 6,   /* strict mode: host-libm exception table missing or stale */
  MCG_ERR_LIMIT = 7     /* a history exceeded the step limit */
};

/* Arithmetic of the step (src/layer.cpp:123-190):
 *  STRICT: the reference's float operations in the reference's order, no
 *          contraction, logf/expf bit-identical to the host C library the
 *          library was built against -> every particle's trajectory, step
 *          count and final state equal the CPU reference's.
 *  FAST:   the same physics with hardware log2/exp2, cached reciprocals and
 *          an accurate 1 - exp; tallies agree statistically. */
enum mcg_mode { MCG_MODE_STRICT = 0, MCG_MODE_FAST = 1 };

typedef struct mcg_context mcg_context;

const char *mcg_last_error(void);
const char *mcg_version(void);

/* Create a context on CUDA device `device`.  Strict mode loads the host-libm
 * exception table built next to the library (or $MCG_LIBM_TABLE). */
int mcg_create(int device, int mode, mcg_context **out);
int mcg_destroy(mcg_context *ctx);
int mcg_set_mode(mcg_context *ctx, int mode);

/* Layers: replaces the Layer constructor / decompose_domain
 * (src/layer.cpp:17-69).  Layer l covers cells [index_start[l],
 * index_start[l] + m[l]) with spacing dx[l]; layers must be contiguous.
 * sigs/rates are per global cell of the chain, first entry = cell
 * index_start[0] (Layer::sigs, Layer::absorption_rates).  Resets the tally. */
int mcg_set_layers(mcg_context *ctx, int n_layers, const int32_t *h_index_start,
                   const int32_t *h_m, const float *h_dx, const float *h_sigs,
                   const float *h_rates, float particle_min_weight);

/* As mcg_set_layers, with the step's two cross sections given per cell:
 * h_sig_a (weight attenuation, sigs*rates in the reference) and h_sig_s
 * (flight sampling, sigs*(1 - rates)); the parameters of the adjoint. */
int mcg_set_layers_xs(mcg_context *ctx, int n_layers, const int32_t *h_index_start,
                      const int32_t *h_m, const float *h_dx, const float *h_sig_a,
                      const float *h_sig_s, float particle_min_weight);

/* decompose_domain(x_min, x_max, ., n_layers, r, nb_cells, ., .) for every r,
 * then mcg_set_layers.  h_sigs/h_rates may be NULL: the constructor's
 * defaults sigs = expf(-x_mid), rates = 0.5 (src/layer.cpp:54-63). */
int mcg_set_slab(mcg_context *ctx, float x_min, float x_max, int32_t nb_cells, int32_t n_layers,
                 const float *h_sigs, const float *h_rates, float particle_min_weight);

/* Fixed-point scale 2^log2_scale of the tally (default 40).  Resets it. */
int mcg_set_tally_scale(mcg_context *ctx, int32_t log2_scale);
int mcg_tally_reset(mcg_context *ctx);
/* Per chain cell: raw fixed-point sums and/or their value as double. */
int mcg_tally_read(mcg_context *ctx, int64_t *h_q, double *h_f64);

/* Run histories of n host particles (Particle array, updated in place with
 * the final state).  h_results (may be NULL): -1/0/+1 per particle.
 * h_steps, h_scatters (may be NULL): particle_step calls and in-cell
 * scatters per particle.  When every given buffer is page-locked (pinned or
 * registered host memory), the GPU reads and writes them in place (each
 * particle crosses the host link once each way during the launch);
 * otherwise they are copied through device memory.  Synchronous. */
int mcg_simulate(mcg_context *ctx, mcg_particle *h_particles, int64_t n, int32_t *h_results,
                 int64_t *h_steps, int64_t *h_scatters);

/* The same on device-resident buffers (no copies); enqueued on the
 * context's stream and waited for.  That stream is non-blocking: buffers
 * written on another stream must be complete before the call (every
 * device-pointer entry point below has the same rule). */
int mcg_simulate_device(mcg_context *ctx, mcg_particle *d_particles, int64_t n,
                        int32_t *d_results, int64_t *d_steps, int64_t *d_scatters);

/* Particles born on the device (no particle upload).  Particle i of the
 * source (i = first .. first+n-1) gets
 *   seed_mode 0: the (i+1)-th value of the rnd_seed chain started at base_seed
 *                (src/random.cpp:24-29, as Layer::create_particles draws them)
 *   seed_mode 1: base_seed + i
 * then x = x0, index = cell0, wmc = w0, and mu = mu0, or (isotropic != 0)
 * mu = 2*rnd_real(seed) - 1 as src/layer.cpp:112 (isotropic == 2: mu in
 * [0,1) via rnd_real).  Only tallies and counters are produced. */
typedef struct mcg_source {
  int32_t seed_mode;
  int32_t isotropic;
  uint64_t base_seed;
  float x0, mu0, w0;
  int32_t cell0;
} mcg_source;
int mcg_simulate_source(mcg_context *ctx, const mcg_source *src, int64_t first, int64_t n);

/* Materialise particles first .. first+n-1 of a source into host memory, as
 * Layer::create_particles does (src/layer.cpp:89-121) for seed_mode 0,
 * isotropic 1. */
int mcg_create_particles(mcg_context *ctx, const mcg_source *src, int64_t first, int64_t n,
                         mcg_particle *h_out);

/* Counters accumulated since the last tally reset. */
typedef struct mcg_counters {
  int64_t histories;     /* finished histories */
  int64_t steps;         /* particle_step calls */
  int64_t scatters;      /* collisions (in-cell direction changes) */
  int64_t leaked_left;   /* histories ending with result -1 */
  int64_t leaked_right;  /* histories ending with result +1 */
  int64_t killed;        /* histories ending below the minimum weight */
  int64_t w_left_q;      /* fixed-point weight carried out to the left */
  int64_t w_right_q;     /* ... to the right */
  int64_t w_killed_q;    /* ... remaining when killed */
  int64_t error_flags;   /* nonzero: a bounded wait or limit tripped */
} mcg_counters;
int mcg_counters_read(mcg_context *ctx, mcg_counters *out);

/* Timing of the last kernel launch of this context (CUDA events around the
 * launch on the context's stream), in milliseconds. */
int mcg_last_kernel_ms(mcg_context *ctx, float *ms);

/* Launch shape (0 = automatic): threads per block, resident blocks per SM,
 * steps between lane refills. */
int mcg_set_launch(mcg_context *ctx, int32_t block, int32_t blocks_per_sm, int32_t refill_steps);

/* Algorithm of the single-chain entry points: MCG_ALGO_HISTORY (default,
 * one lane carries a history to its end) or MCG_ALGO_EVENT (structure-of-
 * arrays particle buffers; each pass advances every live particle by
 * steps_per_pass events, 1 = classic event-based, and compacts the
 * survivors with warp ballots).  Both give identical results. */
enum mcg_algorithm { MCG_ALGO_HISTORY = 0, MCG_ALGO_EVENT = 1 };
int mcg_set_algorithm(mcg_context *ctx, int32_t algorithm, int32_t steps_per_pass);

/* Where the tracker accumulates deposits: 0 shared-memory 64-bit atomics,
 * 1 shared-memory 32-bit halves with carry (default), 2 64-bit atomics on the
 * global tally.  All three give the same exact sums. */
int mcg_set_tally_mode(mcg_context *ctx, int32_t mode);

/* Longest history, in steps, before the tracker stops it with result 2 and
 * the call returns MCG_ERR_LIMIT (default 2^28; the reference has none). */
int mcg_set_step_limit(mcg_context *ctx, int64_t max_steps);

/* Drop-in for the reference GPU seam (include/culayer/culayer.hpp:6-13):
 * runs particles[0..n) until each leaves [min_index, max_index) (no weight
 * cut, as the reference kernel), adds the deposits to weights_absorbed[m]
 * (float, local cell order) and writes every final state back (the reference
 * lost finished particles, src/culayer.cu:31-32,84-86).  Uses a per-thread
 * strict context; on failure prints mcg_last_error() and exits like
 * gpu_errcheck (include/gpu_errcheck/gpu_errcheck.hpp:10-18). */
void cusimulate(int n, mcg_particle *particles, float const *const sigs,
                float const *const absorption_rates, float *const weights_absorbed,
                int min_index, int max_index, float dx);
/* Same, returning a status instead of exiting. */
int mcg_cusimulate(int n, mcg_particle *particles, const float *sigs, const float *absorption_rates,
                   float *weights_absorbed, int min_index, int max_index, float dx);

/* ---- The workers' cycle with on-device hand-over queues ----
 * Drop-in for WorkerSync/WorkerAsync/WorkerRma::spin (src/worker_sync.cpp,
 * src/worker_async.cpp, src/worker_rma.cpp) when every sub-domain (layer of
 * the context's chain) lives on this GPU: each cycle every sub-domain
 * simulates up to per_cycle particles of its queue inside its own cells;
 * leavers are appended to the neighbour's queue (at most queue_capacity
 * waiting particles per sub-domain, else MCG_ERR_OVERFLOW, as the
 * reference's bounded buffers); the n particles of the source are fed to the
 * sub-domain holding src->cell0; the loop ends when all n histories are
 * finished.  Tallies and counters as the other entry points; *h_cycles and
 * *h_handoffs (may be NULL) report the cycles that had particles to simulate
 * and the particles handed over between sub-domains.  Each cycle's particles
 * of all sub-domains are spread over the whole GPU, so a busy sub-domain is
 * not limited to a fixed share of it. */
int mcg_worker_run(mcg_context *ctx, const mcg_source *src, int64_t n, int32_t per_cycle,
                   int64_t queue_capacity, int64_t *h_cycles, int64_t *h_handoffs);

/* ---- The asynchronous workers: hand-over without cycles ----
 * Drop-in for WorkerAsync/WorkerRma::spin (src/worker_async.cpp:19-105,
 * src/worker_rma.cpp) with AsyncComm/RmaComm's send and receive
 * (src/async_comm.cpp:17-168, src/rma_comm.cpp:133-225) replaced by bounded
 * on-device rings, one per sub-domain: one persistent launch in which every
 * warp takes particles from any sub-domain's ring (or newborns from the
 * source for the sub-domain holding src->cell0), simulates each inside its
 * sub-domain and appends leavers to the neighbour's ring, until all n
 * histories are finished.  Newborns are admitted only while fewer than
 * min(queue_capacity - L, 1.125 L) histories are in flight (L = the
 * launch's threads, at most SMs x 1024), which keeps every ring below
 * queue_capacity: with a capacity of at least 2 L (queue_capacity 0
 * selects 3 x SMs x 1024) no ring can overflow; with a smaller one a ring holding queue_capacity particles
 * when another arrives makes the call return MCG_ERR_OVERFLOW (the
 * reference aborts on a full buffer).  Warps without work poll with
 * growing sleeps and give up with MCG_ERR_TIMEOUT after 2 s in which no
 * history finished; every warp stops at the launch's deadline (30 s plus
 * 2 us per history) with MCG_ERR_TIMEOUT, so the call always returns.  Tallies and
 * counters as the other entry points (equal to the fused tracker's);
 * *h_handoffs (may be NULL) counts the hand-overs.  The rings are kept in
 * the context between calls. */
int mcg_worker_run_async(mcg_context *ctx, const mcg_source *src, int64_t n,
                         int64_t queue_capacity, int64_t *h_handoffs);

/* ---- Batched slabs: thousands of independent slabs in one launch ----
 * Slab s is a Layer(0, 1, 0, n_cells) (dx = 1/n_cells, both faces leak):
 * a slab [0, L] maps onto it exactly by scaling its cross sections by L
 * (sigs = (sigma_a + sigma_s) * L, rates = sigma_a / (sigma_a + sigma_s)).
 * Its histories are particles 0 .. n_histories-1 of the source
 * {seed_mode, isotropic, base_seed, x0 = 0, mu0, w0, cell 0} (mcg_source).
 * Tallies are per slab and cell, concatenated in slab order. */
typedef struct mcg_slab {
  int32_t n_cells;
  int32_t seed_mode;
  int32_t isotropic;
  int32_t reserved;
  uint64_t base_seed;
  int64_t n_histories;
  float mu0, w0;
} mcg_slab;
/* h_sigs/h_rates: sum of n_cells entries, slab after slab.  Resets the
 * batch tally. */
int mcg_batch_set(mcg_context *ctx, int32_t n_slabs, const mcg_slab *h_slabs, const float *h_sigs,
                  const float *h_rates, float particle_min_weight);
/* Every history of every slab in one persistent launch, replayed from a
 * CUDA graph (the graph is rebuilt when the launch shape changes).
 * Accumulates into the batch tally; counters as mcg_counters_read. */
int mcg_batch_run(mcg_context *ctx);
/* The same work as one ordinary tracker launch per slab (the plain form),
 * for comparison. */
int mcg_batch_run_per_slab(mcg_context *ctx);
int mcg_batch_tally_reset(mcg_context *ctx);
int mcg_batch_tally_read(mcg_context *ctx, int64_t *h_q, double *h_f64);
/* Launch shape of mcg_batch_run: threads per block (256, 512 or 1024),
 * histories per work item (a block takes one item at a time), tally mode
 * (as mcg_set_tally_mode). 0 keeps the current value. */
int mcg_batch_set_launch(mcg_context *ctx, int32_t block, int64_t item_histories,
                         int32_t tally_mode);
/* Deferral of the full step in mcg_batch_run (0 off, the default; 1..32
 * on): a lane whose step is not a certain crossing waits while the warp's
 * other lanes keep crossing, and the waiting lanes complete their steps
 * together once at least `defer` of them wait (or no other lane can step),
 * instead of the warp running the full step once for every step any of its
 * lanes needs it; lanes refill when two have ended their histories.  Same
 * results for every value. */
int mcg_batch_set_deferral(mcg_context *ctx, int32_t defer);
/* Autotuner: times every candidate on a sample of each slab's histories
 * (fraction in (0, 1], raised so that the sample holds at least four times
 * the event engine's drain size, or the whole run): the history-based
 * launch shapes (block, histories per work item, tally privatisation,
 * deferral of the full step) and the event-based form at 4 and 16 events
 * per pass, and keeps the one with the least time per history.  Reports the choice and its sample time; the
 * batch tally and counters are reset afterwards. */
typedef struct mcg_batch_tuning {
  int32_t block;
  int32_t tally_mode;
  int64_t item_histories;
  float sample_ms;
  int32_t candidates;
  int32_t algorithm;      /* MCG_ALGO_HISTORY or MCG_ALGO_EVENT */
  int32_t steps_per_pass; /* event mode: events per pass */
  int32_t defer;          /* history mode: waiting lanes of the deferred full step, 0 off */
} mcg_batch_tuning;
int mcg_batch_autotune(mcg_context *ctx, double sample_fraction, mcg_batch_tuning *out);

/* History-based (default: the persistent launch above) or event-based
 * batched runs: all slabs' particles in one structure-of-arrays bank, K
 * events per pass (0: 8).  Identical tallies. */
int mcg_batch_set_algorithm(mcg_context *ctx, int32_t algorithm, int32_t steps_per_pass);

/* ---- Differentiation: forward tally + adjoint gradients of a tally loss ----
 * Loss F = sum_c w_c a_c over the chain cells, a_c the weight absorbed in
 * cell c per history.  Gradients with respect to sig_a[c] = sigs*rates and
 * sig_s[c] = sigs*(1 - rates) of every chain cell: sig_a only attenuates the
 * weight (pathwise derivative along the history), sig_s sets the flight
 * distribution (likelihood-ratio score 1/sig_s - l for a collision, -l for a
 * crossing, times the loss deposited from that step on).  Each history is
 * run forward and then replayed from its source index; no path is stored.
 * A slab [0, L] mapped onto [0, 1] by scaling sigma by L has
 * dF/dsigma_physical = L * dF/dsig. */
int mcg_adjoint_set_weights(mcg_context *ctx, const float *h_w);
int mcg_adjoint_reset(mcg_context *ctx); /* also resets the tally */
/* Histories first .. first+n-1 of the source; with_gradient 0 runs the
 * forward pass only (tally + loss).  Accumulates. */
int mcg_adjoint_run(mcg_context *ctx, const mcg_source *src, int64_t first, int64_t n,
                    int32_t with_gradient);
/* Means per history since the last reset; any pointer may be NULL. */
int mcg_adjoint_read(mcg_context *ctx, double *h_loss, double *h_grad_sig_a, double *h_grad_sig_s);

/* ---- Batched inverse fit of absorption cross sections ----
 * Slabs as mcg_batch_set (n_histories = histories per slab and step), with
 * starting sig_a, fixed sig_s (per cell, slab order, the step's two cross
 * sections) and measured tallies h_target (weight absorbed per history, per
 * cell).  mcg_fit_run performs Adam steps on L = sum_c (a_c - t_c)^2: each
 * step is one batched forward+adjoint launch over all slabs (fast
 * arithmetic; loss weights 2 (a - t) from the previous step's tally),
 * followed by the Adam update, all replayed from one CUDA graph, each step on
 * fresh histories.  At most max_steps steps in total per mcg_fit_set. */
int mcg_fit_set(mcg_context *ctx, int32_t n_slabs, const mcg_slab *h_slabs, const float *h_sig_a0,
                const float *h_sig_s, const double *h_target, float particle_min_weight,
                int32_t max_steps);
int mcg_fit_run(mcg_context *ctx, int32_t n_steps, float lr, float beta1, float beta2, float eps,
                float sig_min);
/* sig_a of every cell, loss of every step so far (max_steps entries), steps done. */
int mcg_fit_read(mcg_context *ctx, float *h_sig_a, double *h_loss_hist, int32_t *h_steps);
int mcg_fit_release(mcg_context *ctx);
/* Testing aid: one forward + adjoint launch of the fit's kernel at the
 * current sig_a with loss weights h_weights (per cell) instead of
 * 2 (a - t), on the histories the next step would run; h_tally = weight
 * absorbed per history, h_grad = dF/dsig_a per history for
 * F = sum_c w_c a_c (compare mcg_adjoint_read).  Leaves the fit's state as
 * it was. */
int mcg_fit_gradient(mcg_context *ctx, const double *h_weights, double *h_tally, double *h_grad);

/* Fast tracker that allocates no device memory (no counterpart in the
 * reference; this library's addition for callers that may not call
 * cudaMalloc, such as host codes whose own allocator reserves the GPU's
 * memory at start-up and forbids allocation afterwards).  Equivalent to a
 * fast-mode context with mcg_set_layers + mcg_set_tally_scale(log2_scale) +
 * mcg_simulate_device + mcg_tally_read: the caller passes the layers and
 * cross sections (host arrays, as mcg_set_layers), the particles (device,
 * 8-byte aligned, updated in place), an optional device result array and the
 * device output d_tally_q[total cells], which is overwritten with the
 * fixed-point tally.  Everything else lives in one statically sized device
 * array inside the library (about 384 KiB, held by every GPU that loads the
 * library until the process exits), which holds chains of at most
 * MCG_NOALLOC_MAX_CELLS cells (larger chains are rejected with MCG_ERR_ARG
 * before any device work).  Every call looks up that array's device address
 * (cudaGetSymbolAddress) on the current device, so a device reset between
 * calls is harmless.  The array is shared by all calls on a device and keeps
 * the last call's contents; each call clears what must start at zero.  Calls
 * from several host threads of one process are serialised by a lock inside
 * the library; calls that overlap on the GPU from other processes use their
 * own copies.  Runs on the legacy default stream of the current device and
 * returns when done, so it must not be called while any stream of the
 * device is being captured into a CUDA graph. */
#define MCG_NOALLOC_MAX_CELLS 16384
int mcg_simulate_fast_noalloc(int n_layers, const int32_t *h_index_start, const int32_t *h_m,
                              const float *h_dx, const float *h_sigs, const float *h_rates,
                              float particle_min_weight, int32_t log2_scale,
                              mcg_particle *d_particles, int64_t n, int32_t *d_results,
                              int64_t *d_tally_q);

/* Throughput of the int <-> float conversions on this GPU (testing aid for
 * the roofline; no counterpart in the reference), conversions per second:
 * h_rates[0] u64 -> f32, [1] f32 -> s64 (both on the FP64 pipe of a GB300),
 * [2] u32 -> f32, [3] f32 -> u32; CUDA events around a launch of four
 * independent conversion chains per thread on 8 x SMs x 256 threads. */
int mcg_measure_conversion_rates(mcg_context *ctx, double *h_rates);

/* Testing aid (no counterpart in the reference): the after-th next device
 * allocation of the geometry set-up (mcg_set_layers, mcg_set_layers_xs,
 * mcg_set_slab, mcg_batch_set; 0 = the next one) reports
 * cudaErrorMemoryAllocation without being attempted, so tests can check that
 * a failed set-up leaves the context with no geometry (later launches and
 * reads return MCG_ERR_STATE) and that a new set-up recovers it.  A negative
 * value disables it.  Process-wide. */
int mcg_testing_fail_allocation(int32_t after);

/* One rnd_real step on n device seeds (src/curandom.cu:7-14). */
int mcg_rnd_real_device(mcg_context *ctx, uint64_t *d_seeds, float *d_reals, int64_t n);

/* Strict-mode libm on the GPU for n arguments (testing aid): fn 0 logf on
 * [0, 1], fn 1 expf on [-17.5, 89) (other arguments give NaN); fn 2 the
 * hardware 2^x of the strict tracker's certain-crossing test; fn 3 expf
 * like fn 1 but through the evaluator's general path for every argument;
 * fn 4 the hardware log2, fn 5 the fast arithmetic's collision probability
 * 1 - e^-tau of a flight of optical depth tau >= 0, fn 6 the fast
 * arithmetic's log2 of the flight sample whose state has top 32 bits t
 * (t passed as the argument's bit pattern). */
int mcg_libm_eval_device(mcg_context *ctx, int fn, const float *d_in, float *d_out, int64_t n);

/* Check of the strict tracker's division by a cached reciprocal against the
 * IEEE quotient (testing aid): mode 0 every pair of significands (2^46
 * pairs, about half a minute), mode 1 n pseudo-random pairs over the
 * tracker's exponent range.  Returns the pairs checked, the mismatches and
 * one mismatching pair's bits (a << 32 | b, 0 if none). */
int mcg_verify_division(mcg_context *ctx, int mode, uint64_t n, uint64_t *checked,
                        uint64_t *mismatches, uint64_t *example);

#ifdef __cplusplus
}
#endif
#endif /* MCGB300_H */
