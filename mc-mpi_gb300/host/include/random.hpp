/*
 * random.hpp - the per-particle generators of the mc-mpi API
 * (include/random/random.hpp, src/random.cpp:8-29 of the reference), for
 * callers that build particles on the host.
 */
#ifndef MCG_RANDOM_HPP
#define MCG_RANDOM_HPP

#include "types.hpp"

/* s <- (6364136223846793005 s + 1442695040888963407) mod 2^63;
 * returns (float)s / 2^63 in [0, 1]. */
real_t rnd_real(seed_t *seed);
/* s <- (5177284530976225183 s + 2096348467109453893) mod 2^63; returns s. */
seed_t rnd_seed(seed_t *seed);

#endif
