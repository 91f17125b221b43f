/*
 * mcoracle.h - CPU oracle for the mc-mpi particle-history path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * Layer::simulate path (src/layer.cpp, src/random.cpp of lkskstlr/mc-mpi),
 * used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
 * the checker.  Nothing in the product library links or calls it.
 *
 * Parity pins (tests/test_oracle_golden.py):
 *   - data/test_layer_target_WA.out (100 cells, 100 particles) byte for byte;
 *   - the rnd_seed/rnd_real chain of src/test_curandom.cu (start 30061994);
 *   - the Particle wire layout hash of src/test_async_serialization.cpp;
 *   - per particle, bit for bit, against the reference's own layer.cpp and
 *     random.cpp compiled from source (oracle/_ref, where available).
 */
#ifndef MCORACLE_H
#define MCORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* include/types/particle.hpp:7-17 - 24-byte POD */
typedef struct orc_particle {
  uint64_t seed;
  float x, mu, wmc;
  int32_t index;
} orc_particle;

/* One layer (sub-domain) as built by Layer::Layer (src/layer.cpp:44-69). */
typedef struct orc_layer {
  float x_min, x_max, dx;
  int32_t index_start, m;
  int32_t left_border, right_border;
} orc_layer;

/* Per-particle record of one history (or one layer visit). */
typedef struct orc_trace {
  int32_t result;   /* -1 left, +1 right, 0 killed (weight below minimum) */
  int32_t pad;
  int64_t steps;    /* particle_step calls */
  int64_t scatters; /* steps that stayed in the cell and redrew mu */
} orc_trace;

float orc_rnd_real(uint64_t *seed);
uint64_t orc_rnd_seed(uint64_t *seed);

/* LCG jump-ahead: state after n steps of rnd_seed (a=1) / rnd_real (a=0). */
uint64_t orc_lcg_skip(uint64_t seed, uint64_t n, int seed_chain);

void orc_decompose(float x_min, float x_max, int nb_cells, int world_size, int rank,
                   orc_layer *out);
void orc_layer_make(float x_min, float x_max, int index_start, int m, orc_layer *out);
void orc_default_sigs(const orc_layer *L, float *sigs, float *rates);

/* create_particles(x_ini, wmc, n, seed) on layer L (src/layer.cpp:71-121). */
int orc_create_particles(const orc_layer *L, float x_ini, float wmc, int n, uint64_t seed,
                         orc_particle *out);

/* One history inside one layer; sigs/rates indexed by LOCAL cell. */
int orc_simulate_particle(const orc_layer *L, const float *sigs, const float *rates,
                          float min_w, orc_particle *p, float *tally_f32, int64_t *tally_q,
                          double *tally_f64, float q_scale, orc_trace *tr);

/* Layer::simulate(n) for one call: processes particles[n_total-1] down to
 * particles[n_total-n], in that order, single-threaded.  results[i] is the
 * result of the i-th PROCESSED particle.  Tallies accumulate. */
void orc_layer_simulate(const orc_layer *L, const float *sigs, const float *rates, float min_w,
                        orc_particle *particles, int n_total, int n, int32_t *results,
                        float *tally_f32, int64_t *tally_q, double *tally_f64, float q_scale,
                        orc_trace *traces);

/* Whole histories across a chain of layers (the decomposed slab): each
 * particle starts in the layer holding its index and is handed to the
 * neighbour layer whenever it leaves one, exactly as the workers do.  sigs
 * and rates are indexed by GLOBAL cell.  Results: -1 left border, +1 right
 * border, 0 killed; traces accumulate over layer visits; handoffs counts
 * layer-to-layer transfers.  Tallies indexed by global cell. */
void orc_simulate_histories(const orc_layer *layers, int n_layers, const float *sigs,
                            const float *rates, float min_w, orc_particle *particles, int n,
                            int64_t *tally_q, double *tally_f64, float q_scale,
                            orc_trace *traces, int64_t *handoffs, int nthreads);

/* Layer::dump_WA text (src/layer.cpp:363-380) into buf; returns length. */
int orc_format_wa(const orc_layer *L, const float *tally_f32, char *buf, int cap);

/* FP64 restatement (statistical oracle): same physics in double precision,
 * dw = -expm1(-sig_a * d) * w, h = s * 2^-63 in double.  Per-cell tallies,
 * per-history sums for standard errors. */
void orc_fp64_histories(const orc_layer *layers, int n_layers, const float *sigs,
                        const float *rates, double min_w, const orc_particle *particles, int n,
                        double *tally, double *tally_sq_hist, double *leak, int nthreads);

/* FP64 adjoint estimator: sums over n histories of the loss G = sum_k w dep_k
 * and of its gradients with respect to sig_a and sig_s (global cells). */
void orc_fp64_adjoint(const orc_layer *layers, int n_layers, const double *sig_a,
                      const double *sig_s, const double *w, double min_w,
                      const orc_particle *particles, int n, double *loss_sum, double *grad_a_sum,
                      double *grad_s_sum, int nthreads);

/* Host C library logf (fn 0) / expf (fn 1) over an array. */
void orc_libm_array(int fn, const float *in, float *out, long long n);

#ifdef __cplusplus
}
#endif
#endif
