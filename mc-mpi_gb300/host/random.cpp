/* random.cpp - the reference's two LCGs (src/random.cpp:8-29) for host code. */
#include "random.hpp"

real_t rnd_real(seed_t *seed)
{
  const real_t inv = (real_t)1 / (real_t)((seed_t)1 << 63);
  *seed = (6364136223846793005ull * *seed + 1442695040888963407ull) & (((seed_t)1 << 63) - 1);
  return (real_t)(*seed) * inv;
}

seed_t rnd_seed(seed_t *seed)
{
  *seed = (5177284530976225183ull * *seed + 2096348467109453893ull) & (((seed_t)1 << 63) - 1);
  return *seed;
}
