/*
 * mcg_worker.cu - the workers' cycle with on-device hand-over queues.
 *
 * Restates WorkerSync/WorkerAsync::spin (src/worker_sync.cpp:31-131,
 * src/worker_async.cpp:19-105) for sub-domains that all live on one GPU:
 *  - sub-domain L owns a ring queue of particles (its Layer::particles);
 *  - each cycle, every sub-domain simulates up to `per_cycle` particles of
 *    its queue (the source sub-domain also takes newborn particles from the
 *    source, as Layer::create_particles feeds Layer::simulate) until they
 *    leave the sub-domain or fall below the minimum weight, with its own cell
 *    table and tally in shared memory;
 *  - a particle leaving to the left/right is appended to the neighbour's
 *    queue (one atomic per warp and destination reserves the slots): the
 *    MPI_Sendrecv / AsyncComm::send / RmaComm::send of the reference; at the
 *    slab's borders it is disabled (src/layer.cpp:350-360);
 *  - termination: a device counter of finished histories reaching N (the
 *    Allreduce of src/worker_sync.cpp:113-120 / StateComm's vote).
 * A queue that would overflow its capacity sets an error flag (the reference
 * aborts on a full buffer, src/async_comm.cpp:27-36).  Per-particle
 * trajectories, hence tallies, equal the fused tracker's.
 */
#include <algorithm>
#include <cstring>
#include <vector>

#include "mcg_internal.h"
#include "mcg_track.cuh"

struct mcg_worker_layer {
  int32_t lo, hi;               /* cell range */
  unsigned long long take;      /* particles of the queue processed this cycle */
  unsigned long long from_src;  /* newborns taken from the source this cycle */
  unsigned long long head;      /* queue head at the cycle start */
  unsigned long long cursor;    /* work counter of this cycle */
  unsigned long long tail;      /* queue tail (appends) */
};

struct mcg_worker_params {
  const float4 *cells;
  int32_t n_layers, cell_lo, src_layer, left_border, right_border;
  mcg_worker_layer *layers;
  mcg_particle *queues; /* n_layers x cap */
  unsigned long long cap;
  mcg_source src;
  unsigned long long *src_next;
  unsigned long long src_total;
  int32_t per_cycle;
  float min_w;
  int32_t q_log2;
  unsigned long long *tally, *counters, *done, *handoffs;
  mcg_libm_dev libm;
  const mcg_libm_tab *libm_tab;
  uint32_t max_steps;
};

/* Cycle start (one thread per sub-domain): how many queued particles and
 * newborns each sub-domain takes this cycle. */
__global__ void mcg_worker_prepare(mcg_worker_params P)
{
  const int L = blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= P.n_layers)
    return;
  mcg_worker_layer &W = P.layers[L];
  W.head += W.take; /* consume last cycle's share */
  const unsigned long long queued = W.tail - W.head;
  W.take = min(queued, (unsigned long long)P.per_cycle);
  W.from_src = 0;
  if (L == P.src_layer) {
    const unsigned long long left = P.src_total - *P.src_next;
    W.from_src = min(left, (unsigned long long)P.per_cycle - W.take);
    *P.src_next += W.from_src;
  }
  W.cursor = 0;
}

template <bool STRICT>
__global__ void __launch_bounds__(256) mcg_worker_cycle(mcg_worker_params P, int blocks_per_layer)
{
  extern __shared__ __align__(16) unsigned char smem[];
  mcg_libm_tab *T = reinterpret_cast<mcg_libm_tab *>(smem);
  unsigned long long *s_tally = reinterpret_cast<unsigned long long *>(smem + sizeof(mcg_libm_tab));
  const int L = blockIdx.x / blocks_per_layer, tid = threadIdx.x, lane = tid & 31;
  mcg_worker_layer &W = P.layers[L];
  const int lo = W.lo, hi = W.hi, m = hi - lo;
  if (STRICT)
    for (int i = tid; i < (int)(sizeof(mcg_libm_tab) / 4); i += blockDim.x)
      reinterpret_cast<float *>(T)[i] = reinterpret_cast<const float *>(P.libm_tab)[i];
  for (int i = tid; i < m; i += blockDim.x)
    s_tally[i] = 0ull;
  __syncthreads();
  const unsigned long long take = W.take, total = take + W.from_src, head = W.head;
  const unsigned long long src_first = *P.src_next - W.from_src;
  const float min_w = P.min_w;
  unsigned long long n_done = 0, n_hand = 0, steps = 0, scat = 0;
  const float4 *cells = P.cells + (lo - P.cell_lo);
  for (;;) {
    unsigned long long k = 0;
    if (lane == 0)
      k = atomicAdd(&W.cursor, 32ull);
    k = __shfl_sync(0xffffffffu, k, 0) + lane;
    if (__all_sync(0xffffffffu, k >= total))
      break;
    bool have = k < total;
    uint64_t seed = 0;
    float x = 0.f, mu = 0.f, wmc = 0.f, inv_mu = 0.f;
    int idx = lo;
    uint32_t nsc = 0, nst = 0;
    if (have) {
      if (k < take) {
        const mcg_particle p = P.queues[(size_t)L * P.cap + (head + k) % P.cap];
        seed = p.seed, x = p.x, mu = p.mu, wmc = p.wmc, idx = p.index;
      } else {
        mcg_source_particle(P.src, (int64_t)(src_first + (k - take)), seed, x, mu, wmc, idx);
      }
      inv_mu = mcg_flight_rcp(mu);
      /* Layer::simulate_particle within this sub-domain */
      while ((wmc >= min_w) && (idx < hi) && (idx >= lo) && nst < P.max_steps) {
        mcg_step<STRICT, MCG_TALLY_SMEM32>(seed, x, mu, wmc, inv_mu, idx, nsc, __ldg(cells + (idx - lo)),
                                           &s_tally[idx - lo], P.q_log2, T, P.libm);
        ++nst;
      }
      steps += nst;
      scat += nsc;
    }
    /* hand-over: dir -1 left, +1 right, 0 finished here */
    int dir = 0;
    if (have) {
      if (nst >= P.max_steps && (wmc >= min_w) && (idx < hi) && (idx >= lo)) {
        atomicOr(&P.counters[MCG_CNT_ERR], 1ull);
      } else if (idx == lo - 1) {
        dir = (L == 0 && P.left_border) ? 0 : -1;
      } else if (idx == hi) {
        dir = (L == P.n_layers - 1 && P.right_border) ? 0 : 1;
      }
      if (dir == 0)
        ++n_done;
      else
        ++n_hand;
    }
    for (int d = -1; d <= 1; d += 2) {
      const unsigned want = __ballot_sync(0xffffffffu, have && dir == d);
      if (!want)
        continue;
      const int dst = L + d;
      unsigned long long base = 0;
      if (lane == 0)
        base = atomicAdd(&P.layers[dst].tail, (unsigned long long)__popc(want));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (have && dir == d) {
        const unsigned long long slot = base + __popc(want & lanemask_lt());
        /* the destination's head at this cycle's start bounds its queue */
        if (slot - P.layers[dst].head >= P.cap) {
          atomicOr(&P.counters[MCG_CNT_ERR], 2ull);
        } else {
          mcg_particle o;
          o.seed = seed, o.x = x, o.mu = mu, o.wmc = wmc, o.index = idx;
          P.queues[(size_t)dst * P.cap + slot % P.cap] = o;
        }
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    n_done += __shfl_down_sync(0xffffffffu, n_done, o);
    n_hand += __shfl_down_sync(0xffffffffu, n_hand, o);
    steps += __shfl_down_sync(0xffffffffu, steps, o);
    scat += __shfl_down_sync(0xffffffffu, scat, o);
  }
  if (lane == 0) {
    if (n_done)
      atomicAdd(P.done, n_done);
    if (n_hand)
      atomicAdd(P.handoffs, n_hand);
    atomicAdd(&P.counters[MCG_CNT_STEPS], steps);
    atomicAdd(&P.counters[MCG_CNT_SCAT], scat);
  }
  __syncthreads();
  for (int i = tid; i < m; i += blockDim.x)
    if (s_tally[i])
      atomicAdd(&P.tally[lo - P.cell_lo + i], s_tally[i]);
}

extern "C" int mcg_worker_run(mcg_context *ctx, const mcg_source *src, int64_t n,
                              int32_t per_cycle, int64_t queue_capacity, int64_t *h_cycles,
                              int64_t *h_handoffs)
{
  if (!ctx || !src || n < 0 || per_cycle <= 0 || queue_capacity <= 0)
    return mcg_fail(MCG_ERR_ARG, "mcg_worker_run: bad arguments");
  if (!ctx->d_tally)
    return mcg_fail(MCG_ERR_STATE, "mcg_worker_run: no layers set");
  cudaSetDevice(ctx->device);
  const bool strict = ctx->mode == MCG_MODE_STRICT;
  if (strict && !ctx->libm_loaded) {
    int rc = mcg_load_libm(ctx);
    if (rc != MCG_OK)
      return rc;
  }
  const int P_ = ctx->n_layers;
  int maxm = 0, src_layer = -1;
  std::vector<mcg_worker_layer> lay(P_);
  for (int l = 0; l < P_; ++l) {
    memset(&lay[l], 0, sizeof(lay[l]));
    lay[l].lo = ctx->layer_start[l];
    lay[l].hi = ctx->layer_start[l] + ctx->layer_m[l];
    maxm = std::max(maxm, ctx->layer_m[l]);
    if (src->cell0 >= lay[l].lo && src->cell0 < lay[l].hi)
      src_layer = l;
  }
  if (src_layer < 0)
    return mcg_fail(MCG_ERR_ARG, "mcg_worker_run: the source cell %d is outside the chain", src->cell0);
  const size_t smem = sizeof(mcg_libm_tab) + (size_t)maxm * 8;
  if (smem > (size_t)ctx->smem_optin)
    return mcg_fail(MCG_ERR_ARG, "mcg_worker_run: a sub-domain of %d cells is too large", maxm);
  /* device state: layers, queues, counters (freed at the end of the call) */
  void *d_lay = nullptr, *d_q = nullptr, *d_c = nullptr;
  cudaError_t e;
  if ((e = cudaMalloc(&d_lay, P_ * sizeof(mcg_worker_layer))) != cudaSuccess ||
      (e = cudaMalloc(&d_q, (size_t)P_ * queue_capacity * sizeof(mcg_particle))) != cudaSuccess ||
      (e = cudaMalloc(&d_c, 64)) != cudaSuccess) {
    cudaFree(d_lay);
    cudaFree(d_q);
    return mcg_cuda_fail(e, "mcg_worker_run: cudaMalloc");
  }
  unsigned long long *cnt = static_cast<unsigned long long *>(d_c); /* src_next, done, handoffs */
  cudaMemcpy(d_lay, lay.data(), P_ * sizeof(mcg_worker_layer), cudaMemcpyHostToDevice);
  cudaMemset(d_c, 0, 64);
  mcg_worker_params W;
  memset(&W, 0, sizeof(W));
  W.cells = strict ? ctx->d_cells_strict : ctx->d_cells_fast;
  W.n_layers = P_;
  W.cell_lo = ctx->cell_lo;
  W.src_layer = src_layer;
  /* the chain's end layers leak to the outside (src/layer.cpp:47-48) */
  W.left_border = 1;
  W.right_border = 1;
  W.layers = static_cast<mcg_worker_layer *>(d_lay);
  W.queues = static_cast<mcg_particle *>(d_q);
  W.cap = (unsigned long long)queue_capacity;
  W.src = *src;
  W.src_next = cnt;
  W.src_total = (unsigned long long)n;
  W.per_cycle = per_cycle;
  W.min_w = ctx->min_w;
  W.q_log2 = ctx->log2_scale;
  W.tally = ctx->d_tally;
  W.counters = ctx->d_counters;
  W.done = cnt + 1;
  W.handoffs = cnt + 2;
  W.libm = ctx->libm;
  W.libm_tab = ctx->libm_tab;
  W.max_steps = ctx->max_steps;
  const int bpl = std::max(1, std::min(8, (int)((per_cycle + 255) / 256)));
  auto kern = strict ? mcg_worker_cycle<true> : mcg_worker_cycle<false>;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int64_t cycles = 0;
  unsigned long long host[3] = {0, 0, 0};
  int rc = MCG_OK;
  cudaEventRecord(ctx->ev0, ctx->stream);
  while (e == cudaSuccess) {
    for (int g = 0; g < 8; ++g, ++cycles) {
      mcg_worker_prepare<<<(P_ + 127) / 128, 128, 0, ctx->stream>>>(W);
      kern<<<P_ * bpl, 256, smem, ctx->stream>>>(W, bpl);
      ctx->launches += 2;
    }
    if ((e = cudaGetLastError()) != cudaSuccess)
      break;
    if ((e = cudaMemcpyAsync(host, cnt, sizeof(host), cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess)
      break;
    unsigned long long err = 0;
    cudaMemcpy(&err, ctx->d_counters + MCG_CNT_ERR, 8, cudaMemcpyDeviceToHost);
    if (err) {
      rc = mcg_fail((err & 2) ? MCG_ERR_OVERFLOW : MCG_ERR_LIMIT,
                    (err & 2) ? "mcg_worker_run: a hand-over queue overflowed (capacity %lld)"
                              : "mcg_worker_run: a history exceeded the step limit",
                    (long long)queue_capacity);
      break;
    }
    if (host[1] >= (unsigned long long)n)
      break;
    if (cycles > (int64_t)1 << 40) {
      rc = mcg_fail(MCG_ERR_LIMIT, "mcg_worker_run: no termination");
      break;
    }
  }
  cudaEventRecord(ctx->ev1, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  cudaEventElapsedTime(&ctx->last_ms, ctx->ev0, ctx->ev1);
  cudaFree(d_lay);
  cudaFree(d_q);
  cudaFree(d_c);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_worker_run");
  if (rc != MCG_OK)
    return rc;
  /* histories finished = n; counters in the context */
  unsigned long long hcount = (unsigned long long)n;
  cudaMemcpy(ctx->d_counters + MCG_CNT_HIST, &hcount, 8, cudaMemcpyHostToDevice);
  if (h_cycles)
    *h_cycles = cycles;
  if (h_handoffs)
    *h_handoffs = (int64_t)host[2];
  return MCG_OK;
}
