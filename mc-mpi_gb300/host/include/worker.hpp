/*
 * worker.hpp - the Worker of the mc-mpi API (include/mcmpi/worker.hpp,
 * include/mcmpi/mcmpi_options.hpp of the reference) for a GPU holding every
 * sub-domain.
 *
 * The reference runs one Worker per MPI rank; here one Worker holds all
 * options.world_size sub-domains (the layers of decompose_domain) on the GPU.
 * WorkerSync::spin() runs the workers' cycle with on-device hand-over queues
 * (mcg_worker_run): each cycle every sub-domain simulates up to
 * nb_particles_per_cycle particles, leavers join the neighbour's queue, and
 * the loop ends when all nb_particles histories are finished.
 * WorkerAsync::spin() and WorkerRma::spin() run the asynchronous form
 * (mcg_worker_run_async): one persistent launch, leavers handed to the
 * neighbour's bounded ring and taken by whichever warp is idle, as
 * AsyncComm/RmaComm let ranks proceed without a cycle barrier.  All three
 * give the same tallies.  dump() writes out/config.yaml,
 * out/weights.csv, out/stats.csv and WA.out in the reference's formats
 * (src/worker.cpp:36-61, 63-181, 218-241, 287-313; src/layer.cpp:363-380).
 * stats.csv has WorkerSync's columns (the timer's, no message counts: the
 * hand-over is part of the GPU cycle, so its send, receive and idle times
 * are zero and the computation time is the GPU time of spin()), one row per
 * sub-domain.
 */
#ifndef MCG_WORKER_HPP
#define MCG_WORKER_HPP

#include <stddef.h>

#include <string>
#include <vector>

#include "layer.hpp"
#include "mcgb300.h"

typedef struct mcmpi_options_tag {
  enum Tag : int { Particle = 0, State, STATE_COUNT };
  int world_size; /* number of sub-domains */
  int nb_cells;
  real_t x_min, x_max, x_ini;
  real_t particle_min_weight;
  size_t nb_particles;
  size_t buffer_size;
  double cycle_time;
  int nb_particles_per_cycle;
  int nthread;
  double statistics_cycle_time;
} MCMPIOptions;

/* The `key: value` file of the reference (config.yaml; src/worker.cpp:315-333). */
MCMPIOptions options_from_config(std::string filepath, int world_size);

class Worker
{
public:
  Worker(int world_rank, const MCMPIOptions &options);
  virtual ~Worker();
  virtual void spin();
  void dump();
  std::vector<real_t> weights_absorbed();

  const int world_rank;
  const MCMPIOptions options;
  long long cycles = 0, handoffs = 0; /* of the last spin() */
  float seconds = 0.f;                /* GPU time of the last spin() */
  double starttime = 0.0, endtime = 0.0; /* wall clock (CLOCK_REALTIME) around spin() */

protected:
  bool async_ = false; /* spin() through mcg_worker_run_async */

private:
  mcg_context *ctx_ = nullptr;
  std::vector<int32_t> start_, m_;
  std::vector<float> dx_, x0_;
  std::vector<double> tally_;
  std::string foldername;
};

/* src/worker_sync.cpp: cycles with a hand-over barrier */
class WorkerSync : public Worker
{
public:
  using Worker::Worker;
};

/* src/worker_async.cpp: no cycle barrier (mcg_worker_run_async) */
class WorkerAsync : public Worker
{
public:
  WorkerAsync(int world_rank, const MCMPIOptions &options) : Worker(world_rank, options)
  {
    async_ = true;
  }
};

/* src/worker_rma.cpp: one-sided puts into the neighbour's buffer are the same
 * rings on one GPU */
class WorkerRma : public WorkerAsync
{
public:
  using WorkerAsync::WorkerAsync;
};

#endif
