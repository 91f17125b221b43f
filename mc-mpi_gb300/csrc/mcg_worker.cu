/*
 * mcg_worker.cu - the workers' cycle with on-device hand-over queues.
 *
 * Restates WorkerSync/WorkerAsync::spin (src/worker_sync.cpp:31-131,
 * src/worker_async.cpp:19-105) for sub-domains that all live on one GPU:
 *  - sub-domain L owns a ring queue of particles (its Layer::particles);
 *  - each cycle, every sub-domain takes up to `per_cycle` particles of its
 *    queue (the source sub-domain also takes newborn particles from the
 *    source, as Layer::create_particles feeds Layer::simulate) and simulates
 *    each until it leaves the sub-domain or falls below the minimum weight;
 *  - a particle leaving to the left/right is appended to the neighbour's
 *    queue: the MPI_Sendrecv / AsyncComm::send / RmaComm::send of the
 *    reference; at the slab's borders it is disabled (src/layer.cpp:350-360);
 *  - termination: a device counter of finished histories reaching N (the
 *    Allreduce of src/worker_sync.cpp:113-120 / StateComm's vote).
 * One kernel launch is one cycle.  The cycle's particles of all sub-domains
 * form one list (sub-domain by sub-domain), split evenly over a full grid;
 * lanes of a block refill from the block's share, so a busy sub-domain uses
 * as many lanes as its particles need.  Each block keeps the chain's tally in
 * shared memory and clears and flushes only the cells of the sub-domains its
 * share covers.  A queue that would overflow its capacity sets an error flag
 * (the reference aborts on a full buffer, src/async_comm.cpp:27-36).
 * Per-particle trajectories, hence tallies, equal the fused tracker's.
 */
#include <algorithm>
#include <cstring>
#include <vector>

#include "mcg_internal.h"
#include "mcg_track.cuh"

struct mcg_worker_layer {
  int32_t lo, hi;               /* cell range (global indices) */
  unsigned long long take;      /* particles of the queue processed this cycle */
  unsigned long long from_src;  /* newborns taken from the source this cycle */
  unsigned long long head;      /* queue head at the cycle start */
  unsigned long long tail;      /* queue tail (appends) */
  unsigned long long item0;     /* first item of this sub-domain in the cycle's list */
};

struct mcg_worker_params {
  const float4 *cells;
  int32_t n_layers, cell_lo, n_cells, src_layer;
  mcg_worker_layer *layers;
  mcg_particle *queues; /* n_layers x cap */
  unsigned long long cap;
  mcg_source src;
  unsigned long long *src_next;  /* newborns handed out so far */
  unsigned long long *items;     /* [0] items of this cycle, [1] first newborn of this cycle */
  unsigned long long *cycles;    /* cycles that had particles to simulate */
  unsigned long long src_total;
  int32_t per_cycle, refill_steps;
  float min_w;
  int32_t q_log2;
  unsigned long long *tally, *counters, *done, *handoffs;
  mcg_libm_dev libm;
  const mcg_libm_tab *libm_tab;
  uint32_t max_steps;
};

/* Cycle start (one block): each sub-domain's share of this cycle (queued
 * particles, and newborns for the source sub-domain) and the offsets of the
 * shares in the cycle's item list. */
__global__ void mcg_worker_prepare(mcg_worker_params P)
{
  for (int L = threadIdx.x; L < P.n_layers; L += blockDim.x) {
    mcg_worker_layer &W = P.layers[L];
    W.head += W.take; /* consume last cycle's share */
    const unsigned long long queued = W.tail - W.head;
    W.take = min(queued, (unsigned long long)P.per_cycle);
    W.from_src = 0;
    if (L == P.src_layer) {
      const unsigned long long left = P.src_total - *P.src_next;
      W.from_src = min(left, (unsigned long long)P.per_cycle - W.take);
      P.items[1] = *P.src_next;
      *P.src_next += W.from_src;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long off = 0;
    for (int L = 0; L < P.n_layers; ++L) {
      P.layers[L].item0 = off;
      off += P.layers[L].take + P.layers[L].from_src;
    }
    P.items[0] = off;
    if (off)
      ++*P.cycles;
  }
}

/* Sub-domain of item k: the last L with item0 <= k (item0 is ascending). */
__device__ __forceinline__ int mcg_worker_layer_of(const mcg_worker_layer *lay, int n, unsigned long long k)
{
  int a = 0, b = n - 1;
  while (a < b) {
    const int mid = (a + b + 1) >> 1;
    if (lay[mid].item0 <= k)
      a = mid;
    else
      b = mid - 1;
  }
  return a;
}

/* One cycle.  SMEM: the chain's tally in shared memory (else global
 * atomics, for chains too long for it). */
template <bool STRICT, bool SMEM>
__global__ void __launch_bounds__(1024) mcg_worker_cycle(mcg_worker_params P)
{
  extern __shared__ __align__(16) unsigned char smem[];
  mcg_libm_tab *T = reinterpret_cast<mcg_libm_tab *>(smem);
  unsigned long long *s_next = reinterpret_cast<unsigned long long *>(smem + sizeof(mcg_libm_tab));
  unsigned long long *s_tally = s_next + 4; /* chain-local cells */
  const int tid = threadIdx.x, lane = tid & 31;
  const unsigned long long total = P.items[0], src_first = P.items[1];
  const unsigned long long q = total / gridDim.x, r = total % gridDim.x;
  const unsigned long long beg = q * blockIdx.x + min((unsigned long long)blockIdx.x, r);
  const unsigned long long end = beg + q + (blockIdx.x < r ? 1ull : 0ull);
  if (beg >= end)
    return; /* the whole block: nothing of this cycle is its share */
  /* cells of the sub-domains this block's share covers */
  const int clo = P.layers[mcg_worker_layer_of(P.layers, P.n_layers, beg)].lo - P.cell_lo;
  const int chi = P.layers[mcg_worker_layer_of(P.layers, P.n_layers, end - 1)].hi - P.cell_lo;
  if (STRICT)
    for (int i = tid; i < (int)(sizeof(mcg_libm_tab) / 4); i += blockDim.x)
      reinterpret_cast<float *>(T)[i] = reinterpret_cast<const float *>(P.libm_tab)[i];
  if (tid == 0)
    s_next[0] = beg;
  if (SMEM)
    for (int i = clo + tid; i < chi; i += blockDim.x)
      s_tally[i] = 0ull;
  __syncthreads();
  unsigned long long *tally = SMEM ? s_tally : P.tally;
  const float min_w = P.min_w;
  const int qs = P.q_log2;

  uint64_t seed = 0;
  float x = 0.f, mu = 0.f, wmc = 0.f, inv_mu = 0.f;
  int idx = 0, L = 0, llo = 0, lhi = 0; /* chain-local cell index and sub-domain range */
  uint32_t nst = 0, nsc = 0;
  bool active = false, drained = false;
  unsigned long long pool_next = 0, pool_end = 0;
  unsigned long long n_done = 0, n_hand = 0, steps = 0, scat = 0;
  for (;;) {
    const unsigned need = __ballot_sync(0xffffffffu, !active);
    if (need) {
      /* idle lanes take the next items of the block's share, 32 at a time */
      const int cnt = __popc(need), rank = __popc(need & lanemask_lt());
      const unsigned long long avail = pool_end - pool_next;
      unsigned long long my = ~0ull;
      if ((unsigned long long)rank < avail)
        my = pool_next + rank;
      if ((unsigned long long)cnt > avail && !drained) {
        unsigned long long base = 0;
        if (lane == 0)
          base = atomicAdd(s_next, 32ull);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= end) {
          drained = true;
          pool_next = pool_end = 0;
        } else {
          const unsigned long long e = min(base + 32ull, end);
          const unsigned long long r2 = (unsigned long long)rank - avail;
          if ((unsigned long long)rank >= avail && r2 < e - base)
            my = base + r2;
          pool_next = min(base + (unsigned long long)(cnt - avail), e);
          pool_end = e;
        }
      } else {
        pool_next += min((unsigned long long)cnt, avail);
      }
      if (!active && my != ~0ull) {
        L = mcg_worker_layer_of(P.layers, P.n_layers, my);
        const mcg_worker_layer &W = P.layers[L];
        const unsigned long long j = my - W.item0;
        if (j < W.take) {
          const mcg_particle q = P.queues[(size_t)L * P.cap + (W.head + j) % P.cap];
          seed = q.seed, x = q.x, mu = q.mu, wmc = q.wmc, idx = q.index;
        } else {
          mcg_source_particle(P.src, (int64_t)(src_first + (j - W.take)), seed, x, mu, wmc, idx);
        }
        idx -= P.cell_lo;
        llo = W.lo - P.cell_lo;
        lhi = W.hi - P.cell_lo;
        inv_mu = mcg_flight_rcp(mu);
        nst = nsc = 0;
        active = true;
      }
    }
    if (!__any_sync(0xffffffffu, active))
      break;
    int dir = 0;
    bool finished = false;
    if (active) {
      /* Layer::simulate_particle within the sub-domain: up to refill_steps
       * steps, never past the step limit */
      const int kmax = (int)min((uint32_t)P.refill_steps, P.max_steps - nst);
      int k = 0;
      bool going = true;
      for (; k < kmax; ++k) {
        if (!((wmc >= min_w) & ((unsigned)(idx - llo) < (unsigned)(lhi - llo)))) {
          going = false;
          break;
        }
        mcg_step<STRICT, SMEM ? MCG_TALLY_SMEM32 : MCG_TALLY_GLOBAL>(
            seed, x, mu, wmc, inv_mu, idx, nsc, __ldg(P.cells + idx), &tally[idx], qs, T, P.libm);
      }
      nst += (uint32_t)k;
      if (!going || nst >= P.max_steps) {
        /* hand-over: -1 left, +1 right, 0 finished here */
        if ((wmc >= min_w) && ((unsigned)(idx - llo) < (unsigned)(lhi - llo)))
          atomicOr(&P.counters[MCG_CNT_ERR], 1ull); /* the step limit */
        else if (idx == llo - 1)
          dir = L == 0 ? 0 : -1; /* the chain's ends leak (src/layer.cpp:47-48) */
        else if (idx == lhi)
          dir = L == P.n_layers - 1 ? 0 : 1;
        steps += nst;
        scat += nsc;
        finished = true;
        active = false;
      }
    }
    /* leavers join the neighbour's queue: one atomic per destination and warp */
    const unsigned movers = __ballot_sync(0xffffffffu, finished && dir != 0);
    if (finished && dir == 0)
      ++n_done;
    if (finished && dir != 0) {
      const int dst = L + dir;
      const unsigned peers = __match_any_sync(movers, dst);
      const int leader = __ffs(peers) - 1;
      unsigned long long base = 0;
      if (lane == leader)
        base = atomicAdd(&P.layers[dst].tail, (unsigned long long)__popc(peers));
      base = __shfl_sync(peers, base, leader);
      const unsigned long long slot = base + __popc(peers & lanemask_lt());
      /* the destination's head at this cycle's start bounds its queue */
      if (slot - P.layers[dst].head >= P.cap) {
        atomicOr(&P.counters[MCG_CNT_ERR], 2ull);
      } else {
        mcg_particle o;
        o.seed = seed, o.x = x, o.mu = mu, o.wmc = wmc, o.index = idx + P.cell_lo;
        P.queues[(size_t)dst * P.cap + slot % P.cap] = o;
      }
      ++n_hand;
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
  if (SMEM) {
    __syncthreads();
    for (int i = clo + tid; i < chi; i += blockDim.x)
      if (s_tally[i])
        atomicAdd(&P.tally[i], s_tally[i]);
  }
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
  int src_layer = -1;
  std::vector<mcg_worker_layer> lay(P_);
  for (int l = 0; l < P_; ++l) {
    memset(&lay[l], 0, sizeof(lay[l]));
    lay[l].lo = ctx->layer_start[l];
    lay[l].hi = ctx->layer_start[l] + ctx->layer_m[l];
    if (src->cell0 >= lay[l].lo && src->cell0 < lay[l].hi)
      src_layer = l;
  }
  if (src_layer < 0)
    return mcg_fail(MCG_ERR_ARG, "mcg_worker_run: the source cell %d is outside the chain", src->cell0);
  /* the chain's tally in shared memory when it fits, else global atomics */
  const size_t smem_base = sizeof(mcg_libm_tab) + 4 * sizeof(unsigned long long);
  const bool use_smem = smem_base + (size_t)ctx->n_cells * 8 <= (size_t)ctx->smem_optin;
  const size_t smem = smem_base + (use_smem ? (size_t)ctx->n_cells * 8 : 0);
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
  /* src_next, done, handoffs, cycles with work, items of the cycle, first newborn of it */
  unsigned long long *cnt = static_cast<unsigned long long *>(d_c);
  cudaMemcpy(d_lay, lay.data(), P_ * sizeof(mcg_worker_layer), cudaMemcpyHostToDevice);
  cudaMemset(d_c, 0, 64);
  mcg_worker_params W;
  memset(&W, 0, sizeof(W));
  W.cells = strict ? ctx->d_cells_strict : ctx->d_cells_fast;
  W.n_layers = P_;
  W.cell_lo = ctx->cell_lo;
  W.n_cells = ctx->n_cells;
  W.src_layer = src_layer;
  W.layers = static_cast<mcg_worker_layer *>(d_lay);
  W.queues = static_cast<mcg_particle *>(d_q);
  W.cap = (unsigned long long)queue_capacity;
  W.src = *src;
  W.src_next = cnt;
  W.src_total = (unsigned long long)n;
  W.items = cnt + 4;
  W.cycles = cnt + 3;
  W.per_cycle = per_cycle;
  W.refill_steps = ctx->refill;
  W.min_w = ctx->min_w;
  W.q_log2 = ctx->log2_scale;
  W.tally = ctx->d_tally;
  W.counters = ctx->d_counters;
  W.done = cnt + 1;
  W.handoffs = cnt + 2;
  W.libm = ctx->libm;
  W.libm_tab = ctx->libm_tab;
  W.max_steps = ctx->max_steps;
  auto kern = strict ? (use_smem ? mcg_worker_cycle<true, true> : mcg_worker_cycle<true, false>)
                     : (use_smem ? mcg_worker_cycle<false, true> : mcg_worker_cycle<false, false>);
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int bps = 1;
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, 1024, smem);
  const int grid = ctx->sm_count * std::max(bps, 1);
  int64_t cycles = 0;
  unsigned long long host[4] = {0, 0, 0, 0}; /* src_next, done, handoffs, cycles with work */
  int rc = MCG_OK;
  cudaEventRecord(ctx->ev0, ctx->stream);
  while (e == cudaSuccess) {
    for (int g = 0; g < 8; ++g, ++cycles) {
      mcg_worker_prepare<<<1, 256, 0, ctx->stream>>>(W);
      kern<<<grid, 1024, smem, ctx->stream>>>(W);
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
    *h_cycles = (int64_t)host[3]; /* launched cycles past the last one with work ran empty */
  if (h_handoffs)
    *h_handoffs = (int64_t)host[2];
  return MCG_OK;
}
