/* The Worker of the mc-mpi API on one GPU: config file in the reference's
 * format (argv[1]) with 8 sub-domains, spin(), dump().  Prints the total
 * absorbed weight and the cycles; the files are checked by the caller. */
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "worker.hpp"

int main(int argc, char **argv)
{
  if (argc != 2) {
    fprintf(stderr, "usage: %s config.yaml\n", argv[0]);
    return 2;
  }
  MCMPIOptions opt = options_from_config(argv[1], 8);
  WorkerSync worker(0, opt);
  worker.spin();
  worker.dump();
  double total = 0;
  for (real_t w : worker.weights_absorbed())
    total += w;
  printf("total %.9f cycles %lld handoffs %lld\n", total, worker.cycles, worker.handoffs);
  /* the asynchronous workers on the same problem: the same weights */
  WorkerAsync wa(0, opt);
  wa.spin();
  const std::vector<real_t> a = wa.weights_absorbed(), s = worker.weights_absorbed();
  if (a != s) {
    fprintf(stderr, "WorkerAsync and WorkerSync weights differ\n");
    return EXIT_FAILURE;
  }
  printf("async handoffs %lld\n", wa.handoffs);
  return total > 0 ? 0 : EXIT_FAILURE;
}
