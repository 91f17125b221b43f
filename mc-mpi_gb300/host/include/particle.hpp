/*
 * particle.hpp - the 24-byte particle of the mc-mpi API
 * (include/types/particle.hpp:7-17 of the reference), byte-compatible with
 * mcg_particle of mcgb300.h.
 */
#ifndef MCG_PARTICLE_HPP
#define MCG_PARTICLE_HPP

#include "mcgb300.h"
#include "types.hpp"

typedef struct particle_tag {
public:
  seed_t seed;
  real_t x;
  real_t mu;
  real_t wmc;
  int index; /* cell index, authoritative over x */
} Particle;

static_assert(sizeof(Particle) == sizeof(mcg_particle), "Particle must be 24 bytes");

#endif
