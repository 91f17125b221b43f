/*
 * culayer.hpp - the GPU seam of the mc-mpi API (include/culayer/culayer.hpp
 * of the reference) on libmcgb300: every particle's final state is written
 * back and the deposits are added to weights_absorbed (local cell order).
 */
#ifndef MCG_CULAYER_HPP
#define MCG_CULAYER_HPP

#include "particle.hpp"

inline void cusimulate(int n, Particle *particles, float const *const sigs,
                       float const *const absorption_rates, float *const weights_absorbed,
                       int min_index, int max_index, float dx)
{
  ::cusimulate(n, reinterpret_cast<mcg_particle *>(particles), sigs, absorption_rates,
               weights_absorbed, min_index, max_index, dx);
}

#endif
