/*
 * layer.hpp - the Layer of the mc-mpi API (include/layer/layer.hpp of the
 * reference) with its histories run on the GPU by libmcgb300.
 *
 * Same constructor, methods and public members with the same meaning:
 * simulate(n) consumes up to n particles from the back of `particles`
 * (creating them lazily from the source of create_particles), accumulates the
 * absorbed weight into weights_absorbed, appends leavers to particles_left /
 * particles_right in processing order (border layers count them in
 * nb_disabled instead) and counts killed particles in nb_disabled.  sigs and
 * absorption_rates may be changed between calls.  The arithmetic is the
 * strict mode: every particle ends exactly as the reference's CPU code would
 * leave it.  nthread and use_gpu are accepted for compatibility; there is no
 * CPU path.  Errors print mcg_last_error() and exit, as the reference does.
 */
#ifndef MCG_LAYER_HPP
#define MCG_LAYER_HPP

#include <vector>

#include "particle.hpp"
#include "types.hpp"

class Layer
{
public:
  Layer(real_t x_min, real_t x_max, int index_start, int m, real_t particle_min_weight);
  Layer(const Layer &other);
  Layer &operator=(const Layer &) = delete;
  ~Layer();

  void create_particles(real_t x_ini, real_t wmc, int n, seed_t seed);
  void simulate(int nb_particles, int nthread = -1, bool use_gpu = false);
  void dump_WA();
  int nb_active() const;

  void create_particles(int n);
  /* One history inside this layer (src/layer.cpp:192-218): -1 left, +1
   * right, 0 below the minimum weight; deposits into weights_absorbed_local. */
  int simulate_particle(Particle &particle, std::vector<real_t> &weights_absorbed_local);
  /* One step (src/layer.cpp:123-190); returns the new cell index. */
  int particle_step(Particle &particle, std::vector<real_t> &weights_absorbed_local);
  void simulate_helper(int nb_particles, int nthread, bool use_gpu);

  const real_t x_min, x_max;

private:
  const int m;
  const int index_start;
  mcg_context *ctx_;
  std::vector<real_t> uploaded_sigs_, uploaded_rates_;
  int run(Particle *p, int n, int32_t *results, int64_t max_steps, std::vector<double> *tally);
  void upload();
  int64_t created_ = 0;

public:
  std::vector<real_t> weights_absorbed;
  std::vector<Particle> particles;
  std::vector<Particle> particles_left;
  std::vector<Particle> particles_right;
  const real_t dx;
  int nb_disabled = 0;

  const bool left_border, right_border;

  std::vector<real_t> sigs;
  std::vector<real_t> absorption_rates;
  const real_t particle_min_weight;

  seed_t seed = 0;
  real_t x_ini = 0, wmc = 0;
  int nb_particles_create = 0;
};

Layer decompose_domain(real_t x_min, real_t x_max, real_t x_ini, int world_size, int world_rank,
                       int nb_cells, int nb_particles, real_t particle_min_weight);

#endif
