/*
 * ref_harness.cpp - C entry points around the REFERENCE's own Layer code.
 *
 * TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile together with the
 * unmodified src/layer.cpp and src/random.cpp of lkskstlr/mc-mpi, read in
 * place from the reference checkout (never copied), into oracle/_ref/.  Used
 * to pin the C restatement (mcoracle.c) per particle and as the reference CPU
 * baseline where it can be built.  MPI is absent, so the multi-layer driver
 * below restates WorkerSync's cycle (src/worker_sync.cpp:31-120) with
 * in-process hand-over instead of MPI_Sendrecv; every particle step runs in
 * the reference's Layer::simulate.
 */
#include "layer.hpp"
#include "particle.hpp"
#include "random.hpp"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <omp.h>
#include <unistd.h>

extern "C" {

struct ref_trace {
  int32_t result, pad;
  int64_t steps, scatters;
};

/* Per-particle histories on one layer through the public particle_step, with
 * the loop condition of simulate_particle (src/layer.cpp:195-197).  The layer
 * spans [x_min, x_max] with cells [index_start, index_start+m); sigs/rates
 * replace the constructor's defaults through the public members. */
void ref_trace_particles(float x_min, float x_max, int index_start, int m, float min_w,
                         const float *sigs, const float *rates, Particle *particles, int n,
                         ref_trace *traces)
{
  Layer layer(x_min, x_max, index_start, m, min_w);
  if (sigs)
    layer.sigs.assign(sigs, sigs + m);
  if (rates)
    layer.absorption_rates.assign(rates, rates + m);
  std::vector<real_t> local(m, 0.0f);
  for (int i = 0; i < n; ++i) {
    Particle &p = particles[i];
    ref_trace tr = {0, 0, 0, 0};
    while ((p.wmc >= layer.particle_min_weight) && (p.index < index_start + m) &&
           (p.index >= index_start)) {
      int before = p.index;
      int after = layer.particle_step(p, local);
      tr.steps++;
      if (after == before)
        tr.scatters++;
    }
    Particle q = p;
    /* result classification exactly as simulate_particle */
    std::vector<real_t> dummy(m, 0.0f);
    tr.result = layer.simulate_particle(q, dummy);
    traces[i] = tr;
  }
}

/* Layer::simulate(n, nthread) on injected particles; returns counts and the
 * processed particles' leaver lists; tallies are the reference's float sums. */
void ref_layer_simulate(float x_min, float x_max, int index_start, int m, float min_w,
                        const float *sigs, const float *rates, const Particle *particles,
                        int n_total, int n, int nthread, float *tally, Particle *left,
                        int *n_left, Particle *right, int *n_right, int *nb_disabled)
{
  Layer layer(x_min, x_max, index_start, m, min_w);
  if (sigs)
    layer.sigs.assign(sigs, sigs + m);
  if (rates)
    layer.absorption_rates.assign(rates, rates + m);
  layer.particles.assign(particles, particles + n_total);
  layer.simulate(n, nthread);
  for (int j = 0; j < m; ++j)
    tally[j] = layer.weights_absorbed[j];
  *n_left = (int)layer.particles_left.size();
  *n_right = (int)layer.particles_right.size();
  if (left)
    std::memcpy(left, layer.particles_left.data(), sizeof(Particle) * layer.particles_left.size());
  if (right)
    std::memcpy(right, layer.particles_right.data(),
                sizeof(Particle) * layer.particles_right.size());
  *nb_disabled = layer.nb_disabled;
}

/* src/test_layer.cpp:41-56: the golden-file case.  Writes WA.out text into
 * buf (Layer::dump_WA writes ./WA.out, so run in a scratch directory). */
int ref_test_layer_wa(const char *scratch_dir, char *buf, int cap, int nthread)
{
  char cwd[4096];
  if (!getcwd(cwd, sizeof(cwd)) || chdir(scratch_dir) != 0)
    return -1;
  const real_t x_ini = sqrtf(2.0) / 2.0;
  Layer layer(decompose_domain(0.0, 1.0, x_ini, 1, 0, 100, 100, 0.0));
  layer.simulate(-1, nthread);
  layer.dump_WA();
  FILE *f = fopen("WA.out", "r");
  int len = f ? (int)fread(buf, 1, cap - 1, f) : -1;
  if (f)
    fclose(f);
  if (len >= 0)
    buf[len] = 0;
  remove("WA.out");
  if (chdir(cwd) != 0)
    return -1;
  return len;
}

/* Decomposed slab without MPI: P layers from decompose_domain, particles
 * injected into the layers holding their index, then WorkerSync's cycle:
 * every layer simulates up to per_cycle particles (layers in parallel, one
 * thread each, as one MPI rank per layer would), leavers are appended to the
 * neighbours' particle vectors, until every particle is disabled.
 * sigs/rates indexed by global cell.  Returns the number of cycles. */
int ref_decomposed(float x_min, float x_max, int nb_cells, int P, float min_w, const float *sigs,
                   const float *rates, const Particle *particles, int n, int per_cycle,
                   int nthreads, double *tally_out)
{
  std::vector<Layer> layers;
  std::vector<int> starts;
  layers.reserve(P);
  for (int r = 0; r < P; ++r) {
    /* x_ini outside every layer: no particles created by the constructor */
    layers.push_back(decompose_domain(x_min, x_max, -1.0f, P, r, nb_cells, n, min_w));
  }
  int acc = 0;
  for (int r = 0; r < P; ++r) {
    starts.push_back(acc);
    acc += (int)layers[r].weights_absorbed.size();
  }
  for (int r = 0; r < P; ++r) {
    int m = (int)layers[r].weights_absorbed.size();
    layers[r].sigs.assign(sigs + starts[r], sigs + starts[r] + m);
    layers[r].absorption_rates.assign(rates + starts[r], rates + starts[r] + m);
  }
  for (int i = 0; i < n; ++i) {
    int r = 0;
    while (r < P - 1 && particles[i].index >= starts[r + 1])
      ++r;
    layers[r].particles.push_back(particles[i]);
  }
  if (nthreads > 0)
    omp_set_num_threads(nthreads);
  int cycles = 0;
  for (;;) {
    ++cycles;
#pragma omp parallel for schedule(dynamic, 1)
    for (int r = 0; r < P; ++r)
      layers[r].simulate(per_cycle, 1);
    long long disabled = 0;
    for (int r = 0; r < P; ++r) {
      if (r > 0) {
        auto &v = layers[r].particles_left;
        layers[r - 1].particles.insert(layers[r - 1].particles.end(), v.begin(), v.end());
        v.clear();
      }
      if (r < P - 1) {
        auto &v = layers[r].particles_right;
        layers[r + 1].particles.insert(layers[r + 1].particles.end(), v.begin(), v.end());
        v.clear();
      }
    }
    for (int r = 0; r < P; ++r)
      disabled += layers[r].nb_disabled;
    if (disabled == n)
      break;
  }
  for (int r = 0; r < P; ++r) {
    int m = (int)layers[r].weights_absorbed.size();
    for (int j = 0; j < m; ++j)
      tally_out[starts[r] + j] = layers[r].weights_absorbed[j];
  }
  return cycles;
}

/* rnd_seed chain and one rnd_real step per seed, with the reference's own
 * src/random.cpp (the CPU half of src/test_curandom.cu:23-37). */
void ref_rng_chain(uint64_t start, int n, uint64_t *seeds_out, uint64_t *seeds_after, float *reals)
{
  seed_t s = start;
  for (int i = 0; i < n; ++i) {
    seeds_out[i] = rnd_seed(&s);
    seed_t t = seeds_out[i];
    reals[i] = rnd_real(&t);
    seeds_after[i] = t;
  }
}

/* src/test_async_serialization.cpp:6-31: FNV-1a over the bytes of the test
 * particle, as the reference's struct lays them out. */
int ref_particle_hash(void)
{
  Particle p{5127801, 0.172634512365276, 123.12342351, -1231.123486123, 2134512};
  const char *data = (const char *)&p;
  unsigned int hash = 0x811c9dc5, prime = 16777619;
  for (int i = 0; i < (int)sizeof(p); ++i) {
    hash = hash ^ data[i];
    hash = hash * prime;
  }
  int res;
  memcpy(&res, &hash, sizeof(res));
  return res;
}

} /* extern "C" */
