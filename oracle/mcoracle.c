/*
 * mcoracle.c - CPU oracle for the mc-mpi particle-history path.
 *
 * TEST INFRASTRUCTURE ONLY (tests/, __graft_entry__.smoke(), bench.py's CPU
 * baseline).  A plain-C restatement of lkskstlr/mc-mpi's src/layer.cpp and
 * src/random.cpp; each function cites the lines it follows.  Compiled with
 * -O2 -ffp-contract=off so every float operation rounds exactly where the
 * reference's does (the reference is built in ISO C++11 mode, where GCC does
 * not contract).  logf/expf are the host C library's, as in the reference.
 */
#include "mcoracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_EPS 1e-4F /* EPS_PRECISION, include/types/types.hpp:15 */

/* ---- src/random.cpp:8-29 ---- */
static const uint64_t RNG_G = 6364136223846793005ull;
static const uint64_t RNG_C = 1442695040888963407ull;
static const uint64_t RNGS_G = 5177284530976225183ull;
static const uint64_t RNGS_C = 2096348467109453893ull;
static const uint64_t MASK63 = (1ull << 63) - 1ull; /* % 2^63 */

/* rnd_real: s <- (G s + C) mod 2^63, return (float)s * (1/(float)2^63)
 * (src/random.cpp:12-16).  (float)s rounds to nearest; the scale is exact. */
float orc_rnd_real(uint64_t *seed)
{
  const float inv = (float)1 / (float)(1ull << 63);
  *seed = (RNG_G * *seed + RNG_C) & MASK63;
  return (float)(*seed) * inv;
}

/* rnd_seed: second LCG deriving per-particle seeds (src/random.cpp:24-29). */
uint64_t orc_rnd_seed(uint64_t *seed)
{
  *seed = (RNGS_G * *seed + RNGS_C) & MASK63;
  return *seed;
}

/* n-fold composition of the affine map s -> (a s + c) mod 2^63. */
uint64_t orc_lcg_skip(uint64_t seed, uint64_t n, int seed_chain)
{
  uint64_t a = seed_chain ? RNGS_G : RNG_G, c = seed_chain ? RNGS_C : RNG_C;
  uint64_t A = 1, C = 0; /* accumulated map */
  while (n) {
    if (n & 1) {
      A = A * a;
      C = C * a + c;
    }
    c = c * a + c;
    a = a * a;
    n >>= 1;
  }
  return (A * seed + C) & MASK63;
}

/* ---- Layer::Layer (src/layer.cpp:44-69) ---- */
void orc_layer_make(float x_min, float x_max, int index_start, int m, orc_layer *L)
{
  L->x_min = x_min;
  L->x_max = x_max;
  L->index_start = index_start;
  L->m = m;
  L->dx = (x_max - x_min) / (float)m;
  L->left_border = fabsf(x_min) < ORC_EPS;
  L->right_border = fabs((double)x_max - 1.0) < (double)ORC_EPS;
}

/* sigs[i] = expf(-x_mid), x_mid = x_min + i*dx + 0.5*dx (double, then float);
 * absorption_rates = 0.5 (src/layer.cpp:54-63). */
void orc_default_sigs(const orc_layer *L, float *sigs, float *rates)
{
  for (int i = 0; i < L->m; ++i) {
    float x_mid = (float)((double)(L->x_min + (float)i * L->dx) + 0.5 * (double)L->dx);
    sigs[i] = expf(-x_mid);
    rates[i] = 0.5f;
  }
}

/* ---- decompose_domain (src/layer.cpp:17-42) ---- */
void orc_decompose(float x_min, float x_max, int nb_cells, int world_size, int rank,
                   orc_layer *out)
{
  int cells_per_layer = nb_cells / world_size;
  int num_with_extra = nb_cells % world_size;
  int nb_my_cells = cells_per_layer + (rank < num_with_extra);
  int start_index = rank * cells_per_layer + (rank < num_with_extra ? rank : num_with_extra);
  float dx = (x_max - x_min) / ((float)nb_cells);
  orc_layer_make(x_min + (float)start_index * dx, x_min + (float)(start_index + nb_my_cells) * dx,
                 start_index, nb_my_cells, out);
}

/* ---- Layer::create_particles (src/layer.cpp:71-121), all at once ---- */
int orc_create_particles(const orc_layer *L, float x_ini, float wmc, int n, uint64_t seed,
                         orc_particle *out)
{
  if (!(x_ini > L->x_min && x_ini < L->x_max))
    return 0;
  orc_particle p;
  memset(&p, 0, sizeof(p));
  p.x = x_ini;
  p.wmc = wmc;
  p.index = (int32_t)(x_ini / L->dx);
  for (int i = 0; i < n; ++i) {
    p.seed = orc_rnd_seed(&seed);
    p.mu = 2 * orc_rnd_real(&p.seed) - 1;
    out[i] = p;
  }
  return n;
}

/* ---- Layer::particle_step (src/layer.cpp:123-190) ---- */
static inline void orc_particle_step(const orc_layer *L, const float *sigs, const float *rates,
                                     orc_particle *p, float *tally_f32, int64_t *tally_q,
                                     double *tally_f64, float q_scale, orc_trace *tr)
{
  const int il = p->index - L->index_start;
  const float interaction_rate = (float)(1.0 - (double)rates[il]);
  const float sig_a = sigs[il] * rates[il];
  const float sig_i = sigs[il] * interaction_rate;

  const float h = orc_rnd_real(&p->seed);
  float di = sig_i > ORC_EPS ? -logf(h) / sig_i : FLT_MAX;

  int index_new;
  float x_new_edge;
  if (p->mu < 0) {
    index_new = p->index - 1;
    x_new_edge = (float)p->index * L->dx;
  } else {
    index_new = p->index + 1;
    x_new_edge = (float)(p->index + 1) * L->dx;
  }
  float di_edge = FLT_MAX;
  if (p->mu < -ORC_EPS || ORC_EPS < p->mu)
    di_edge = (x_new_edge - p->x) / p->mu;

  if (di < di_edge) {
    index_new = p->index;
    p->x += di * p->mu;
    p->mu = 2 * orc_rnd_real(&p->seed) - 1;
    if (tr)
      tr->scatters++;
  } else {
    di = di_edge;
    p->x = x_new_edge;
  }
  const float dw = (1 - expf(-sig_a * di)) * p->wmc;
  p->wmc -= dw;
  if (tally_f32)
    tally_f32[il] += dw;
  if (tally_q)
    tally_q[il] += llrintf(dw * q_scale);
  if (tally_f64)
    tally_f64[il] += (double)dw;
  p->index = index_new;
  if (tr)
    tr->steps++;
}

/* ---- Layer::simulate_particle (src/layer.cpp:192-218) ---- */
int orc_simulate_particle(const orc_layer *L, const float *sigs, const float *rates,
                          float min_w, orc_particle *p, float *tally_f32, int64_t *tally_q,
                          double *tally_f64, float q_scale, orc_trace *tr)
{
  const int start = L->index_start, end = L->index_start + L->m;
  while ((p->wmc >= min_w) && (p->index < end) && (p->index >= start))
    orc_particle_step(L, sigs, rates, p, tally_f32, tally_q, tally_f64, q_scale, tr);
  int r;
  if (p->index == start - 1)
    r = -1;
  else if (p->index == end)
    r = +1;
  else if (p->wmc < min_w)
    r = 0;
  else
    r = -1;
  if (tr)
    tr->result = r;
  return r;
}

/* ---- Layer::simulate, one call, single thread (src/layer.cpp:239-361) ----
 * The reference takes particles from the back (particles[size-1-i]) into a
 * zeroed thread-local float tally and then adds it into weights_absorbed. */
void orc_layer_simulate(const orc_layer *L, const float *sigs, const float *rates, float min_w,
                        orc_particle *particles, int n_total, int n, int32_t *results,
                        float *tally_f32, int64_t *tally_q, double *tally_f64, float q_scale,
                        orc_trace *traces)
{
  float *local = (float *)calloc((size_t)L->m, sizeof(float));
  for (int i = 0; i < n; ++i) {
    orc_trace *tr = traces ? &traces[i] : NULL;
    if (tr)
      memset(tr, 0, sizeof(*tr));
    results[i] = orc_simulate_particle(L, sigs, rates, min_w, &particles[n_total - 1 - i], local,
                                       tally_q, tally_f64, q_scale, tr);
  }
  if (tally_f32)
    for (int j = 0; j < L->m; ++j)
      tally_f32[j] += local[j];
  free(local);
}

/* Whole histories through a chain of layers: the handoff of the workers
 * (src/worker_sync.cpp:41-109, src/worker_async.cpp:39-53) moves a leaver to
 * the neighbour layer, where Layer::simulate continues it; border layers drop
 * leavers as disabled (src/layer.cpp:350-360). */
void orc_simulate_histories(const orc_layer *layers, int n_layers, const float *sigs,
                            const float *rates, float min_w, orc_particle *particles, int n,
                            int64_t *tally_q, double *tally_f64, float q_scale,
                            orc_trace *traces, int64_t *handoffs, int nthreads)
{
  int total_cells = layers[n_layers - 1].index_start + layers[n_layers - 1].m;
#ifdef _OPENMP
  if (nthreads > 0)
    omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  int64_t hand_total = 0;
#pragma omp parallel reduction(+ : hand_total)
  {
    int64_t *tq = tally_q ? (int64_t *)calloc((size_t)total_cells, sizeof(int64_t)) : NULL;
    double *tf = tally_f64 ? (double *)calloc((size_t)total_cells, sizeof(double)) : NULL;
#pragma omp for schedule(dynamic, 64)
    for (int i = 0; i < n; ++i) {
      orc_particle *p = &particles[i];
      orc_trace tr;
      memset(&tr, 0, sizeof(tr));
      int k = 0;
      while (k < n_layers - 1 && p->index >= layers[k].index_start + layers[k].m)
        ++k;
      for (;;) {
        const orc_layer *L = &layers[k];
        const int s = L->index_start;
        int r = orc_simulate_particle(L, sigs + s, rates + s, min_w, p, NULL, tq ? tq + s : NULL,
                                      tf ? tf + s : NULL, q_scale, &tr);
        if (r == -1 && !L->left_border && k > 0) {
          --k;
          hand_total++;
          continue;
        }
        if (r == +1 && !L->right_border && k < n_layers - 1) {
          ++k;
          hand_total++;
          continue;
        }
        tr.result = r;
        break;
      }
      if (traces)
        traces[i] = tr;
    }
#pragma omp critical
    {
      for (int c = 0; c < total_cells; ++c) {
        if (tq)
          tally_q[c] += tq[c];
        if (tf)
          tally_f64[c] += tf[c];
      }
    }
    free(tq);
    free(tf);
  }
  if (handoffs)
    *handoffs = hand_total;
}

/* ---- Layer::dump_WA (src/layer.cpp:363-380) ---- */
int orc_format_wa(const orc_layer *L, const float *tally_f32, char *buf, int cap)
{
  int off = 0;
  for (int i = 0; i < L->m; ++i) {
    double x = (double)(L->x_min + (float)i * L->dx) + 0.5 * (double)L->dx;
    int w = snprintf(buf + off, (size_t)(cap - off), "%.4e %.3e\n", x,
                     (double)(tally_f32[i] / L->dx));
    if (w < 0 || off + w >= cap)
      return -1;
    off += w;
  }
  return off;
}

/* ---- FP64 statistical restatement ----
 * The reference's problem (float cross sections, float cell faces
 * (float)index * dx) with its physics evaluated in double: continuous
 * flight samples h = s 2^-63, log and expm1 in double, double positions and
 * weights.  The float faces matter: a face's rounding moves it by up to an
 * ulp of x, which on a 10,000-cell slab changes a cell's width, hence its
 * absorbed weight, by up to 2e-4 relative, about one standard error at 1e8
 * histories. */
void orc_fp64_histories(const orc_layer *layers, int n_layers, const float *sigs,
                        const float *rates, double min_w, const orc_particle *particles, int n,
                        double *tally, double *tally_sq_hist, double *leak, int nthreads)
{
  int total = layers[n_layers - 1].index_start + layers[n_layers - 1].m;
#ifdef _OPENMP
  if (nthreads > 0)
    omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  double lk0 = 0.0, lk1 = 0.0;
#pragma omp parallel reduction(+ : lk0, lk1)
  {
    double *t = (double *)calloc((size_t)total, sizeof(double));
    double *t2 = (double *)calloc((size_t)total, sizeof(double));
    double *hist = (double *)calloc((size_t)total, sizeof(double));
    int *touched = (int *)malloc(sizeof(int) * (size_t)total);
    int *mark = (int *)calloc((size_t)total, sizeof(int));
#pragma omp for schedule(dynamic, 64)
    for (int i = 0; i < n; ++i) {
      uint64_t s = particles[i].seed;
      double x = particles[i].x, mu = particles[i].mu, w = particles[i].wmc;
      int idx = particles[i].index, nt = 0;
      int k = 0;
      while (k < n_layers - 1 && idx >= layers[k].index_start + layers[k].m)
        ++k;
      for (;;) {
        const orc_layer *L = &layers[k];
        if (!(w >= min_w))
          break;
        if (idx < L->index_start) {
          if (L->left_border || k == 0) { lk0 += w; break; }
          --k;
          continue;
        }
        if (idx >= L->index_start + L->m) {
          if (L->right_border || k == n_layers - 1) { lk1 += w; break; }
          ++k;
          continue;
        }
        double sig = sigs[idx], rate = rates[idx];
        double sa = sig * rate, si = sig * (1.0 - rate);
        s = (RNG_G * s + RNG_C) & MASK63;
        double h = (double)s * 0x1p-63;
        double di = si > ORC_EPS ? -log(h) / si : DBL_MAX;
        /* the problem's cell faces are the reference's float values
         * (float)index * dx (src/layer.cpp:146,150); only the physics runs
         * in double */
        double edge = mu < 0 ? (double)((float)idx * L->dx) : (double)((float)(idx + 1) * L->dx);
        double de = (mu < -ORC_EPS || ORC_EPS < mu) ? (edge - x) / mu : DBL_MAX;
        int nidx = mu < 0 ? idx - 1 : idx + 1;
        if (di < de) {
          nidx = idx;
          x += di * mu;
          s = (RNG_G * s + RNG_C) & MASK63;
          mu = 2.0 * ((double)s * 0x1p-63) - 1.0;
        } else {
          di = de;
          x = edge;
        }
        double dw = -expm1(-sa * di) * w;
        w -= dw;
        if (mark[idx] != i + 1) {
          mark[idx] = i + 1;
          touched[nt++] = idx;
        }
        hist[idx] += dw;
        idx = nidx;
      }
      for (int j = 0; j < nt; ++j) {
        int c = touched[j];
        t[c] += hist[c];
        t2[c] += hist[c] * hist[c];
        hist[c] = 0.0;
      }
    }
#pragma omp critical
    {
      for (int c = 0; c < total; ++c) {
        tally[c] += t[c];
        if (tally_sq_hist)
          tally_sq_hist[c] += t2[c];
      }
    }
    free(t);
    free(t2);
    free(hist);
    free(touched);
    free(mark);
  }
  if (leak) {
    leak[0] += lk0;
    leak[1] += lk1;
  }
}

/* The host C library's logf (fn 0) or expf (fn 1) over an array: the values
 * the reference's particle_step obtains (src/layer.cpp:137, :175). */
void orc_libm_array(int fn, const float *in, float *out, long long n)
{
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < n; ++i)
    out[i] = fn == 0 ? logf(in[i]) : expf(in[i]);
}

/* FP64 adjoint estimator (statistical oracle of the GPU adjoint): per history
 * a forward pass in double computing G = sum_k w_{c_k} dep_k, then a replay
 * from the same seed accumulating
 *   dG/dsig_a[c] += l_k (w_c W_k - (G - P_k))          (pathwise)
 *   dG/dsig_s[c] += (1{collision}/sig_s - l_k) (G - P_{k-1})   (score)
 * sig_a/sig_s/w indexed by global cell; sums over the n histories. */
static int fp64_walk(const orc_layer *layers, int n_layers, const double *sa, const double *ss,
                     const double *w, double min_w, const orc_particle *p0, double G,
                     double *grad_a, double *grad_s, double *G_out)
{
  uint64_t s = p0->seed;
  double x = p0->x, mu = p0->mu, W = p0->wmc, Gacc = 0.0, P = 0.0;
  int idx = p0->index, k = 0;
  while (k < n_layers - 1 && idx >= layers[k].index_start + layers[k].m)
    ++k;
  for (;;) {
    const orc_layer *L = &layers[k];
    if (!(W >= min_w))
      break;
    if (idx < L->index_start) {
      if (L->left_border || k == 0)
        break;
      --k;
      continue;
    }
    if (idx >= L->index_start + L->m) {
      if (L->right_border || k == n_layers - 1)
        break;
      ++k;
      continue;
    }
    s = (RNG_G * s + RNG_C) & MASK63;
    double h = (double)s * 0x1p-63;
    double di = ss[idx] > ORC_EPS ? -log(h) / ss[idx] : DBL_MAX;
    /* the reference's float cell faces, as in orc_fp64_histories */
    double edge = mu < 0 ? (double)((float)idx * L->dx) : (double)((float)(idx + 1) * L->dx);
    double de = (mu < -ORC_EPS || ORC_EPS < mu) ? (edge - x) / mu : DBL_MAX;
    int nidx = mu < 0 ? idx - 1 : idx + 1;
    int coll = di < de;
    double l;
    if (coll) {
      nidx = idx;
      l = di;
      x += di * mu;
      s = (RNG_G * s + RNG_C) & MASK63;
      mu = 2.0 * ((double)s * 0x1p-63) - 1.0;
    } else {
      l = de;
      x = edge;
    }
    double Wn = W * exp(-sa[idx] * l);
    double g = w[idx] * (W - Wn);
    if (grad_a) {
      double vb = G - P;
      P += g;
      double va = G - P;
      grad_a[idx] += l * (w[idx] * Wn - va);
      grad_s[idx] += ((coll ? 1.0 / ss[idx] : 0.0) - l) * vb;
    }
    Gacc += g;
    W = Wn;
    idx = nidx;
  }
  if (G_out)
    *G_out = Gacc;
  return 0;
}

void orc_fp64_adjoint(const orc_layer *layers, int n_layers, const double *sig_a,
                      const double *sig_s, const double *w, double min_w,
                      const orc_particle *particles, int n, double *loss_sum, double *grad_a_sum,
                      double *grad_s_sum, int nthreads)
{
  int total = layers[n_layers - 1].index_start + layers[n_layers - 1].m;
#ifdef _OPENMP
  if (nthreads > 0)
    omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  double loss = 0.0;
#pragma omp parallel reduction(+ : loss)
  {
    double *ga = (double *)calloc((size_t)total, sizeof(double));
    double *gs = (double *)calloc((size_t)total, sizeof(double));
#pragma omp for schedule(dynamic, 64)
    for (int i = 0; i < n; ++i) {
      double G = 0.0;
      fp64_walk(layers, n_layers, sig_a, sig_s, w, min_w, &particles[i], 0.0, NULL, NULL, &G);
      if (grad_a_sum)
        fp64_walk(layers, n_layers, sig_a, sig_s, w, min_w, &particles[i], G, ga, gs, NULL);
      loss += G;
    }
#pragma omp critical
    {
      if (grad_a_sum)
        for (int c = 0; c < total; ++c) {
          grad_a_sum[c] += ga[c];
          grad_s_sum[c] += gs[c];
        }
    }
    free(ga);
    free(gs);
  }
  *loss_sum += loss;
}
