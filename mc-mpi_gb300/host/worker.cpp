/* worker.cpp - Worker of the mc-mpi API with all sub-domains on one GPU. */
#include "worker.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sys/stat.h>
#include <time.h>
#include <unistd.h>

static void die(const char *what)
{
  fprintf(stderr, "%s: %s\n", what, mcg_last_error());
  exit(EXIT_FAILURE);
}

/* Wall clock in seconds, the time base of the reference's timer stamps
 * (MPI_Wtime shifted to CLOCK_REALTIME, src/timer.cpp:7-24). */
static double wall_seconds()
{
  struct timespec t;
  clock_gettime(CLOCK_REALTIME, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

MCMPIOptions options_from_config(std::string filepath, int world_size)
{
  std::ifstream in(filepath);
  if (!in) {
    fprintf(stderr, "Couldn't open Yaml File %s.\n", filepath.c_str());
    exit(1);
  }
  std::map<std::string, std::string> v;
  std::string line;
  while (std::getline(in, line)) {
    const size_t n = line.find(':');
    if (n == std::string::npos) {
      fprintf(stderr, "Yaml File %s was not correctly formatted.\n", filepath.c_str());
      exit(1);
    }
    /* the first line with a key wins (src/yaml_loader.cpp:27 emplaces) */
    v.emplace(line.substr(0, n), line.substr(n + 1));
  }
  auto get = [&](const char *k) -> std::string {
    auto it = v.find(k);
    if (it == v.end()) {
      fprintf(stderr, "Yaml File %s has no key %s.\n", filepath.c_str(), k);
      exit(1);
    }
    return it->second;
  };
  MCMPIOptions o;
  memset(&o, 0, sizeof(o));
  o.world_size = world_size;
  o.nb_cells = std::stoi(get("nb_cells"));
  o.x_min = (real_t)std::stod(get("x_min"));
  o.x_max = (real_t)std::stod(get("x_max"));
  o.x_ini = (real_t)std::stod(get("x_ini"));
  o.particle_min_weight = (real_t)std::stod(get("particle_min_weight"));
  o.nb_particles = (size_t)std::stoi(get("nb_particles"));
  o.cycle_time = std::stod(get("cycle_time"));
  o.nb_particles_per_cycle = std::stoi(get("nb_particles_per_cycle"));
  o.nthread = std::stoi(get("nthread"));
  o.statistics_cycle_time = std::stod(get("statistics_cycle_time"));
  return o;
}

Worker::Worker(int world_rank, const MCMPIOptions &options) : world_rank(world_rank), options(options)
{
  const char *slurm = getenv("SLURM_JOB_ID");
  foldername = slurm ? std::string("../out/") + slurm : std::string("out");
  if (mcg_create(0, MCG_MODE_STRICT, &ctx_) != MCG_OK)
    die("Worker: mcg_create");
  /* decompose_domain for every sub-domain (src/layer.cpp:17-42) */
  const int P = options.world_size, M = options.nb_cells;
  const int cpl = M / P, extra = M % P;
  const real_t gdx = (options.x_max - options.x_min) / ((float)M);
  std::vector<float> sigs, rates;
  for (int r = 0; r < P; ++r) {
    const int m = cpl + (r < extra), s = r * cpl + (r < extra ? r : extra);
    const real_t lx0 = options.x_min + s * gdx, lx1 = options.x_min + (s + m) * gdx;
    const real_t dx = (lx1 - lx0) / m;
    start_.push_back(s);
    m_.push_back(m);
    dx_.push_back(dx);
    x0_.push_back(lx0);
    for (int i = 0; i < m; ++i) {
      const real_t x_mid = (real_t)((double)(lx0 + (real_t)i * dx) + 0.5 * (double)dx);
      sigs.push_back(expf(-x_mid)); /* the Layer constructor's physics (src/layer.cpp:54-63) */
      rates.push_back(0.5f);
    }
  }
  if (mcg_set_layers(ctx_, P, start_.data(), m_.data(), dx_.data(), sigs.data(), rates.data(),
                     options.particle_min_weight) != MCG_OK)
    die("Worker: mcg_set_layers");
}

Worker::~Worker() { mcg_destroy(ctx_); }

void Worker::spin()
{
  const real_t dx = (options.x_max - options.x_min) / ((float)options.nb_cells);
  const int cell_ini = (int)((options.x_ini - options.x_min) / dx);
  int src_layer = 0;
  for (size_t l = 0; l < start_.size(); ++l)
    if (cell_ini >= start_[l] && cell_ini < start_[l] + m_[l])
      src_layer = (int)l;
  /* Layer::create_particles of the source layer: index = x_ini / its dx */
  mcg_source src = {0, 1, 5127801, options.x_ini, 0.0f, (float)(1.0 / options.nb_particles),
                    (int32_t)(options.x_ini / dx_[src_layer])};
  int64_t cyc = 0, hand = 0;
  starttime = wall_seconds();
  if (async_) {
    /* the library's default ring capacity, which never overflows */
    if (mcg_worker_run_async(ctx_, &src, (int64_t)options.nb_particles, 0, &hand) != MCG_OK)
      die("WorkerAsync::spin");
  } else {
    const int64_t cap = (int64_t)options.nb_particles + 1;
    if (mcg_worker_run(ctx_, &src, (int64_t)options.nb_particles,
                       options.nb_particles_per_cycle > 0 ? options.nb_particles_per_cycle : 65536,
                       cap, &cyc, &hand) != MCG_OK)
      die("WorkerSync::spin");
  }
  endtime = wall_seconds();
  cycles = cyc;
  handoffs = hand;
  mcg_last_kernel_ms(ctx_, &seconds);
  seconds /= 1e3f;
  tally_.assign(options.nb_cells, 0.0);
  if (mcg_tally_read(ctx_, nullptr, tally_.data()) != MCG_OK)
    die("Worker: mcg_tally_read");
}

std::vector<real_t> Worker::weights_absorbed()
{
  std::vector<real_t> w(tally_.size());
  for (size_t i = 0; i < w.size(); ++i)
    w[i] = (real_t)tally_[i];
  return w;
}

void Worker::dump()
{
  mkdir(foldername.c_str(), S_IRWXU | S_IRWXG | S_IRWXO);
  const std::vector<real_t> w = weights_absorbed();
  /* out/config.yaml (src/worker.cpp:218-241) */
  FILE *f = fopen((foldername + "/config.yaml").c_str(), "w");
  if (!f)
    die("Worker::dump");
  fprintf(f, "# Read from config\n");
  fprintf(f, "nb_cells: %d\n", options.nb_cells);
  fprintf(f, "x_min: %.18e\n", (double)options.x_min);
  fprintf(f, "x_max: %.18e\n", (double)options.x_max);
  fprintf(f, "x_ini: %.18e\n", (double)options.x_ini);
  fprintf(f, "particle_min_weight: %.18e\n", (double)options.particle_min_weight);
  fprintf(f, "nb_particles: %d\n", (int)options.nb_particles);
  fprintf(f, "buffer_size: %d\n", (int)options.buffer_size);
  fprintf(f, "cycle_time: %.18e\n", options.cycle_time);
  fprintf(f, "nb_particles_per_cycle: %d\n", options.nb_particles_per_cycle);
  fprintf(f, "nthread: %d\n", options.nthread);
  fprintf(f, "statistics_cycle_time: %.18e\n", options.statistics_cycle_time);
  fprintf(f, "\n# Other values\n");
  fprintf(f, "world_size: %d\n", options.world_size);
  char host[1000] = {0};
  gethostname(host, sizeof(host) - 1);
  fprintf(f, "hostname: %s\n", host);
  fclose(f);
  /* out/weights.csv (src/worker.cpp:287-313): rank 0's dx, as the reference */
  f = fopen((foldername + "/weights.csv").c_str(), "w");
  if (!f)
    die("Worker::dump");
  fprintf(f, "proc, x, weight\n");
  int proc = 0;
  for (int i = 0; i < (int)w.size(); ++i) {
    if (proc < options.world_size - 1 && start_[proc + 1] == i)
      proc++;
    fprintf(f, "%d, %.18e, %.18e\n", proc, dx_[0] * (i + 0.5), w[i] / dx_[0]);
  }
  fclose(f);
  /* out/stats.csv (src/worker.cpp:63-181) with WorkerSync's columns: one
   * timer state per sub-domain (the whole spin), no message counts */
  f = fopen((foldername + "/stats.csv").c_str(), "w");
  if (!f)
    die("Worker::dump");
  fprintf(f, "rank, starttime, endtime, time_comp, time_send, time_recv, time_idle, "
             "nb_cycles, \n");
  for (int r = 0; r < options.world_size; ++r)
    fprintf(f, "%d, %.18e, %.18e, %.18e, %.18e, %.18e, %.18e, %d, \n", r, starttime, endtime,
            (double)seconds, 0.0, 0.0, 0.0, (int)cycles);
  fclose(f);
  /* WA.out of rank 0's layer (Layer::dump_WA) */
  f = fopen("WA.out", "w");
  if (!f)
    die("Worker::dump");
  for (int i = 0; i < m_[0]; ++i)
    fprintf(f, "%.4e %.3e\n", x0_[0] + (i * dx_[0]) + 0.5 * dx_[0], w[i] / dx_[0]);
  fclose(f);
}
