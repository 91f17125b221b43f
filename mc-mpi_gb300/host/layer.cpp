/*
 * layer.cpp - Layer and decompose_domain of the mc-mpi API on libmcgb300
 * (the reference's src/layer.cpp behaviour, histories on the GPU).
 */
#include "layer.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "mcgb300.h"
#include "random.hpp"

#define MAX_PARTICLES_VECTOR 1000000 /* src/layer.cpp:15 */

static void die(const char *what)
{
  fprintf(stderr, "%s: %s\n", what, mcg_last_error());
  exit(EXIT_FAILURE);
}

static mcg_context *new_context()
{
  mcg_context *c = nullptr;
  if (mcg_create(0, MCG_MODE_STRICT, &c) != MCG_OK)
    die("Layer: mcg_create");
  return c;
}

/* src/layer.cpp:44-69 */
Layer::Layer(real_t x_min, real_t x_max, int index_start, int m, real_t particle_min_weight)
    : x_min(x_min), x_max(x_max), m(m), index_start(index_start), ctx_(new_context()),
      dx((x_max - x_min) / m), left_border(fabsf(x_min) < EPS_PRECISION),
      right_border(fabs(x_max - 1.0) < EPS_PRECISION), particle_min_weight(particle_min_weight)
{
  sigs.reserve(m);
  for (int i = 0; i < m; ++i) {
    const real_t x_mid = (real_t)((double)(x_min + (real_t)i * dx) + 0.5 * (double)dx);
    sigs.push_back(expf(-x_mid));
  }
  absorption_rates.assign(m, 0.5f);
  weights_absorbed.assign(m, 0.0f);
}

Layer::Layer(const Layer &o)
    : x_min(o.x_min), x_max(o.x_max), m(o.m), index_start(o.index_start), ctx_(new_context()),
      created_(o.created_), weights_absorbed(o.weights_absorbed), particles(o.particles),
      particles_left(o.particles_left), particles_right(o.particles_right), dx(o.dx),
      nb_disabled(o.nb_disabled), left_border(o.left_border), right_border(o.right_border),
      sigs(o.sigs), absorption_rates(o.absorption_rates),
      particle_min_weight(o.particle_min_weight), seed(o.seed), x_ini(o.x_ini), wmc(o.wmc),
      nb_particles_create(o.nb_particles_create)
{
}

Layer::~Layer() { mcg_destroy(ctx_); }

void Layer::upload()
{
  if (sigs == uploaded_sigs_ && absorption_rates == uploaded_rates_)
    return;
  if ((int)sigs.size() != m || (int)absorption_rates.size() != m) {
    fprintf(stderr, "Layer: sigs/absorption_rates must have %d entries\n", m);
    exit(EXIT_FAILURE);
  }
  const int32_t st = index_start, mm = m;
  const float d = dx;
  if (mcg_set_layers(ctx_, 1, &st, &mm, &d, sigs.data(), absorption_rates.data(),
                     particle_min_weight) != MCG_OK)
    die("Layer: mcg_set_layers");
  uploaded_sigs_ = sigs;
  uploaded_rates_ = absorption_rates;
}

int Layer::run(Particle *p, int n, int32_t *results, int64_t max_steps, std::vector<double> *tally)
{
  upload();
  if (mcg_tally_reset(ctx_) != MCG_OK || mcg_set_step_limit(ctx_, max_steps) != MCG_OK)
    die("Layer");
  const int rc = mcg_simulate(ctx_, reinterpret_cast<mcg_particle *>(p), n, results, nullptr, nullptr);
  if (rc != MCG_OK && !(rc == MCG_ERR_LIMIT && max_steps == 1))
    die("Layer::simulate");
  tally->assign(m, 0.0);
  if (mcg_tally_read(ctx_, nullptr, tally->data()) != MCG_OK)
    die("Layer: mcg_tally_read");
  return rc;
}

void Layer::create_particles(real_t x_ini_, real_t wmc_, int n, seed_t seed_)
{
  if (x_ini_ > x_min && x_ini_ < x_max) {
    x_ini = x_ini_;
    wmc = wmc_;
    nb_particles_create = n;
    seed = seed_;
    created_ = 0;
    create_particles(MAX_PARTICLES_VECTOR);
  }
}

int Layer::nb_active() const { return (int)particles.size() + nb_particles_create; }

/* src/layer.cpp:89-121: particles created_ .. of the rnd_seed chain, isotropic
 * mu from each particle's own stream, made on the GPU */
void Layer::create_particles(int n)
{
  if (nb_particles_create <= 0)
    return;
  const int best = MAX_PARTICLES_VECTOR - (int)particles.size();
  n = best > n ? best : n;
  n = nb_particles_create < n ? nb_particles_create : n;
  nb_particles_create -= n;
  mcg_source src = {0, 1, seed, x_ini, 0.0f, wmc, (int32_t)(x_ini / dx)};
  const size_t old = particles.size();
  particles.resize(old + n);
  if (mcg_create_particles(ctx_, &src, created_, n,
                           reinterpret_cast<mcg_particle *>(particles.data() + old)) != MCG_OK)
    die("Layer::create_particles");
  created_ += n;
}

void Layer::simulate_helper(int nb_particles, int nthread, bool use_gpu)
{
  if (nb_particles == -1)
    while (particles.size() > 0 || nb_particles_create > 0)
      simulate(MAX_PARTICLES_VECTOR, nthread, use_gpu);
  while (nb_particles > 0 && (particles.size() > 0 || nb_particles_create > 0)) {
    const int k = nb_particles < MAX_PARTICLES_VECTOR ? nb_particles : MAX_PARTICLES_VECTOR;
    simulate(k, nthread, use_gpu);
    nb_particles -= k;
  }
}

/* src/layer.cpp:239-361 */
void Layer::simulate(int nb_particles, int nthread, bool use_gpu)
{
  if (nb_particles == -1 || nb_particles > MAX_PARTICLES_VECTOR)
    simulate_helper(nb_particles, nthread, use_gpu);
  if ((int)particles.size() < nb_particles && nb_particles_create > 0)
    create_particles(nb_particles);
  const int size = (int)particles.size();
  const int nb = size < nb_particles ? size : nb_particles;
  if (nb <= 0)
    return;
  std::vector<Particle> batch(particles.rbegin(), particles.rbegin() + nb); /* processing order */
  std::vector<int32_t> result(nb);
  std::vector<double> tally;
  run(batch.data(), nb, result.data(), 1ll << 28, &tally);
  for (int j = 0; j < m; ++j)
    weights_absorbed[j] += (real_t)tally[j];
  for (int i = 0; i < nb; ++i) {
    if (result[i] == -1)
      particles_left.push_back(batch[i]);
    else if (result[i] == 1)
      particles_right.push_back(batch[i]);
    else
      nb_disabled++;
  }
  particles.resize(size - nb);
  if (left_border) {
    nb_disabled += (int)particles_left.size();
    particles_left.clear();
  }
  if (right_border) {
    nb_disabled += (int)particles_right.size();
    particles_right.clear();
  }
}

int Layer::simulate_particle(Particle &particle, std::vector<real_t> &weights_absorbed_local)
{
  int32_t r = 0;
  std::vector<double> tally;
  run(&particle, 1, &r, 1ll << 28, &tally);
  for (int j = 0; j < m && j < (int)weights_absorbed_local.size(); ++j)
    weights_absorbed_local[j] += (real_t)tally[j];
  return r;
}

int Layer::particle_step(Particle &particle, std::vector<real_t> &weights_absorbed_local)
{
  int32_t r = 0;
  std::vector<double> tally;
  run(&particle, 1, &r, 1, &tally);
  for (int j = 0; j < m && j < (int)weights_absorbed_local.size(); ++j)
    weights_absorbed_local[j] += (real_t)tally[j];
  return particle.index;
}

/* src/layer.cpp:363-380 */
void Layer::dump_WA()
{
  FILE *file = fopen("WA.out", "w");
  if (!file) {
    fprintf(stderr, "Couldn't open file WA.out for writing.\n");
    exit(1);
  }
  for (int i = 0; i < (int)weights_absorbed.size(); ++i)
    fprintf(file, "%.4e %.3e\n", x_min + (i * dx) + 0.5 * dx, weights_absorbed[i] / dx);
  fclose(file);
}

/* src/layer.cpp:17-42 */
Layer decompose_domain(real_t x_min, real_t x_max, real_t x_ini, int world_size, int world_rank,
                       int nb_cells, int nb_particles, real_t particle_min_weight)
{
  const int cells_per_layer = nb_cells / world_size;
  const int num_with_extra = nb_cells % world_size;
  const int nb_my_cells = cells_per_layer + (world_rank < num_with_extra);
  const int start_index =
      world_rank * cells_per_layer + (world_rank < num_with_extra ? world_rank : num_with_extra);
  const real_t dx = (x_max - x_min) / ((float)nb_cells);
  const int cell_ini = (int)((x_ini - x_min) / dx);
  Layer layer(x_min + start_index * dx, x_min + (start_index + nb_my_cells) * dx, start_index,
              nb_my_cells, particle_min_weight);
  if (cell_ini >= start_index && cell_ini < start_index + nb_my_cells)
    layer.create_particles(x_ini, 1.0 / nb_particles, nb_particles, 5127801);
  return layer;
}
