/* Layer::particle_step applied until the particle leaves the layer ends in
 * the same state, with the same deposits, as one Layer::simulate_particle
 * (src/layer.cpp:123-218), for 200 particles of the reference's source. */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "layer.hpp"

int main()
{
  Layer layer(decompose_domain(0.0, 1.0, sqrtf(2.0) / 2.0, 1, 0, 50, 200, 1e-12f));
  std::vector<real_t> a(50, 0.0f), b(50, 0.0f);
  int bad = 0;
  long long steps = 0;
  for (int i = 0; i < 200; ++i) {
    Particle p = layer.particles[i], q = layer.particles[i];
    const int r = layer.simulate_particle(p, a);
    while (q.wmc >= layer.particle_min_weight && q.index >= 0 && q.index < 50) {
      layer.particle_step(q, b);
      ++steps;
    }
    const int rq = q.index == -1 ? -1 : q.index == 50 ? 1 : 0;
    if (memcmp(&p, &q, sizeof(Particle)) != 0 || r != rq)
      ++bad;
  }
  double da = 0, db = 0, dmax = 0;
  for (int j = 0; j < 50; ++j) {
    da += a[j];
    db += b[j];
    dmax = fmax(dmax, fabs(a[j] - b[j]));
  }
  printf("%d mismatched particles, %lld single steps, tallies %.9g %.9g (max diff %.3g)\n", bad,
         steps, da, db, dmax);
  return (bad == 0 && dmax < 1e-6) ? 0 : EXIT_FAILURE;
}
