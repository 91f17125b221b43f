/* Reads a config.yaml with options_from_config (the reference's
 * src/worker.cpp:315-333 over src/yaml_loader.cpp) and prints the options,
 * one `key value` per line.  Needs no GPU. */
#include <cstdio>
#include <cstdlib>

#include "worker.hpp"

int main(int argc, char **argv)
{
  if (argc < 3)
    return 2;
  const MCMPIOptions o = options_from_config(argv[1], std::atoi(argv[2]));
  printf("world_size %d\n", o.world_size);
  printf("nb_cells %d\n", o.nb_cells);
  printf("x_min %.9e\n", (double)o.x_min);
  printf("x_max %.9e\n", (double)o.x_max);
  printf("x_ini %.9e\n", (double)o.x_ini);
  printf("particle_min_weight %.9e\n", (double)o.particle_min_weight);
  printf("nb_particles %zu\n", o.nb_particles);
  printf("cycle_time %.17e\n", o.cycle_time);
  printf("nb_particles_per_cycle %d\n", o.nb_particles_per_cycle);
  printf("nthread %d\n", o.nthread);
  printf("statistics_cycle_time %.17e\n", o.statistics_cycle_time);
  return 0;
}
