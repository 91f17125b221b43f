/* The golden-file check of src/test_layer.cpp through this library's C++
 * Layer: 100 cells, 100 particles from x_ini = sqrt(2)/2, minimum weight 0,
 * simulate(-1), dump_WA, byte comparison with the golden WA.out (argv[1]). */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>

#include "layer.hpp"

static std::string slurp(const char *path)
{
  std::ifstream f(path);
  std::stringstream s;
  s << f.rdbuf();
  return s.str();
}

int main(int argc, char **argv)
{
  if (argc != 2) {
    fprintf(stderr, "usage: %s golden_WA.out\n", argv[0]);
    return 2;
  }
  const real_t x_ini = sqrtf(2.0) / 2.0;
  Layer layer(decompose_domain(0.0, 1.0, x_ini, 1, 0, 100, 100, 0.0));
  layer.simulate(-1);
  layer.dump_WA();
  const std::string got = slurp("WA.out"), want = slurp(argv[1]);
  remove("WA.out");
  if (got != want || got.empty()) {
    printf("ERROR: Output files are not identical!\n");
    return EXIT_FAILURE;
  }
  printf("WA.out identical, nb_disabled = %d\n", layer.nb_disabled);
  return layer.nb_disabled == 100 ? 0 : EXIT_FAILURE;
}
