/*
 * types.hpp - scalar types of the mc-mpi API (include/types/types.hpp of the
 * reference): single precision reals, 64-bit seeds.
 */
#ifndef MCG_TYPES_HPP
#define MCG_TYPES_HPP

#include <limits>

typedef unsigned long long seed_t;
typedef float real_t;
constexpr real_t MAXREAL = std::numeric_limits<real_t>::max();
#define EPS_PRECISION 1e-4F

#endif
