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
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <thread>
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
template <bool STRICT, bool SMEM, bool THIN>
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
        mcg_step<STRICT, SMEM ? MCG_TALLY_SMEM32 : MCG_TALLY_GLOBAL, THIN>(
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

static size_t worker_align(size_t b)
{
  return (b + 255) & ~(size_t)255;
}

/* The context's worker buffer, at least `bytes` long. */
static int worker_buffer(mcg_context *ctx, size_t bytes, unsigned char **out)
{
  if (!ctx->ext)
    ctx->ext = new mcg_ext();
  mcg_worker_state &W = ctx->ext->worker;
  if (W.bytes < bytes) {
    if (W.dev)
      cudaFree(W.dev);
    W.dev = nullptr;
    W.bytes = 0;
    cudaError_t e = cudaMalloc(&W.dev, bytes);
    if (e != cudaSuccess)
      return mcg_cuda_fail(e, "workers: cudaMalloc(queues)");
    W.bytes = bytes;
  }
  *out = static_cast<unsigned char *>(W.dev);
  return MCG_OK;
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
  /* device state: layers, queues, counters, in the context's worker
   * buffer (allocated once, grown when a call needs more) */
  const size_t o_lay = 0, o_c = worker_align(P_ * sizeof(mcg_worker_layer));
  const size_t o_q = o_c + 256;
  unsigned char *wb = nullptr;
  int rcb = worker_buffer(ctx, o_q + (size_t)P_ * queue_capacity * sizeof(mcg_particle), &wb);
  if (rcb != MCG_OK)
    return rcb;
  void *d_lay = wb + o_lay, *d_q = wb + o_q, *d_c = wb + o_c;
  cudaError_t e;
  /* src_next, done, handoffs, cycles with work, items of the cycle, first newborn of it */
  unsigned long long *cnt = static_cast<unsigned long long *>(d_c);
  if ((e = cudaMemcpy(d_lay, lay.data(), P_ * sizeof(mcg_worker_layer), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemset(d_c, 0, 64)) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_worker_run: set-up");
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
  /* the strict thin-cell step (mcg_step THIN) on chains where it applies */
  auto kern = strict ? (mcg_strict_thin(ctx) ? (use_smem ? mcg_worker_cycle<true, true, true>
                                              : mcg_worker_cycle<true, false, true>)
                                  : (use_smem ? mcg_worker_cycle<true, true, false>
                                              : mcg_worker_cycle<true, false, false>))
                     : (use_smem ? mcg_worker_cycle<false, true, false>
                                 : mcg_worker_cycle<false, false, false>);
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, ctx->smem_optin);
  int bps = 1;
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, 1024, smem);
  const int grid = ctx->sm_count * std::max(bps, 1);
  int64_t cycles = 0;
  /* Termination bound: every cycle with work takes at least one step of some
   * history, and every history ends within max_steps steps of each of its
   * visits to a sub-domain, one visit per hand-over, so the loop needs at
   * most n * max_steps cycles with work; a check every 8 cycles that finds
   * no work while histories are unfinished is an inconsistency, reported as
   * MCG_ERR_STATE rather than looped on. */
  const double max_cycles = (double)std::max<int64_t>(n, 1) * (double)ctx->max_steps + 8.0;
  unsigned long long last_work_cycles = 0;
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
    if (host[3] == last_work_cycles) {
      rc = mcg_fail(MCG_ERR_STATE, "mcg_worker_run: %llu of %lld histories finished and no "
                    "particle left to simulate", host[1], (long long)n);
      break;
    }
    last_work_cycles = host[3];
    if ((double)cycles > max_cycles) {
      rc = mcg_fail(MCG_ERR_LIMIT, "mcg_worker_run: more cycles than n * max_steps");
      break;
    }
  }
  cudaEventRecord(ctx->ev1, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  cudaEventElapsedTime(&ctx->last_ms, ctx->ev0, ctx->ev1);
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

/* ---------------------------------------------------------------------------
 * The asynchronous form (WorkerAsync / WorkerRma, src/worker_async.cpp:19-105,
 * src/async_comm.cpp, src/rma_comm.cpp): no cycles.  One persistent launch;
 * every warp takes work for its idle lanes from the sub-domains' queues (or
 * newborns from the source), simulates each particle inside its sub-domain
 * and appends leavers to the neighbour's queue, until the device counter of
 * finished histories reaches N.  The queues are bounded multi-producer
 * multi-consumer rings with a publication word per slot: slot s of a ring
 * of capacity C is free for ticket t when seq[s] == t and holds ticket t
 * when seq[s] == t + 1; a producer takes a ticket with one atomic and
 * writes the particle and then seq = t + 1, a consumer claims a run of
 * published tickets with one compare-and-swap on the ring's head and, after
 * reading, frees the slots for the next lap (seq = t + C).  Nothing waits on
 * a slot: a producer that finds its slot still occupied (the ring holds C
 * particles) sets the overflow flag, as the reference aborts on a full
 * buffer.  Newborns are admitted only while fewer than `inflight` histories
 * are born and unfinished, which bounds every ring's content: with a
 * capacity of the grid's lanes plus `inflight` no ring can overflow.
 *
 * Idle warps must not crowd the rings: a global count of published,
 * unclaimed particles (a hint, exact once every producer and consumer has
 * updated it) is all an idle warp polls, with an exponential back-off sleep
 * (up to 32 us); only when it is positive does the warp look at the rings,
 * each lane one or two rings at once, and try to claim from at most four.
 * The grid is no larger than the work needs (one 1024-thread block per 1024
 * histories).  Every loop of the kernel is bounded: a warp gives up with
 * MCG_ERR_TIMEOUT after `idle_limit_ns` in which no history finished, and
 * every warp, busy or not, stops at the launch's deadline (`budget_ns` after
 * its start), recording how far the run got, so a run can fail but never
 * hang.  Every particle follows the trajectory of the fused tracker, so the
 * tally equals it.
 * ------------------------------------------------------------------------- */
struct mcg_aq_ring {
  int32_t lo, hi;           /* cell range of the sub-domain (global indices) */
  unsigned long long enq;   /* tickets handed to producers */
  unsigned long long deq;   /* tickets claimed by consumers */
  unsigned long long pad[5];
};

/* Run state of the asynchronous workers (one 256-byte block of counters). */
enum { MCG_AQ_SRC_NEXT = 0, MCG_AQ_DONE, MCG_AQ_HANDOFFS, MCG_AQ_PENDING, MCG_AQ_DEADLINE_HITS,
       MCG_AQ_ABORT, MCG_AQ_ITERS, MCG_AQ_EXITED, MCG_AQ_N };

struct mcg_async_params {
  const float4 *cells;
  int32_t n_layers, cell_lo, n_cells, src_layer;
  mcg_aq_ring *rings;
  mcg_particle *slots;          /* n_layers x cap */
  unsigned long long *seq;      /* n_layers x cap publication words */
  unsigned long long cap;
  mcg_source src;
  unsigned long long *state;    /* MCG_AQ_* counters */
  unsigned long long src_total;
  int32_t refill_steps;
  float min_w;
  int32_t q_log2;
  unsigned long long *tally, *counters;
  mcg_libm_dev libm;
  const mcg_libm_tab *libm_tab;
  uint32_t max_steps;
  unsigned long long idle_limit_ns, budget_ns;
  unsigned long long inflight; /* born and unfinished histories admitted */
};

__device__ __forceinline__ unsigned long long mcg_ld_acquire(const unsigned long long *p)
{
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long mcg_ld_relaxed(const unsigned long long *p)
{
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void mcg_st_release(unsigned long long *p, unsigned long long v)
{
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned long long mcg_globaltimer()
{
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

/* The block's own ring in shared memory: a leaver goes there while the
 * ring holds at most MCG_LQ - 1024 particles (then at most 1024 more can be
 * reserved by the block's lanes at once, so it never overfills), else to the
 * destination's global ring; idle lanes take from it first. */
#define MCG_LQ 2048
#define MCG_LQ_BYTES (16 + MCG_LQ * (4 + 4 + (int)sizeof(mcg_particle)))

/* Rounds of the asynchronous workers: steps per lane between two warp
 * votes, lanes without a particle that end a round, longest round */
#define MCG_AQ_WINDOW 16
#define MCG_AQ_ROUND_IDLE 4
#define MCG_AQ_ROUND_CAP 256

template <bool STRICT, bool SMEM, bool THIN>
__global__ void __launch_bounds__(1024) mcg_worker_async(mcg_async_params P)
{
  extern __shared__ __align__(16) unsigned char smem[];
  mcg_libm_tab *T = reinterpret_cast<mcg_libm_tab *>(smem);
  /* local ring: head and tail tickets, publication words, sub-domain and
   * particle of every slot */
  unsigned *lq_ctl = reinterpret_cast<unsigned *>(smem + sizeof(mcg_libm_tab));
  unsigned *lq_seq = lq_ctl + 4;
  int *lq_L = reinterpret_cast<int *>(lq_seq + MCG_LQ);
  mcg_particle *lq_part = reinterpret_cast<mcg_particle *>(lq_L + MCG_LQ);
  int2 *s_rng = reinterpret_cast<int2 *>(smem + sizeof(mcg_libm_tab) + MCG_LQ_BYTES); /* [n_layers] lo, hi local */
  unsigned long long *s_tally =
      reinterpret_cast<unsigned long long *>(s_rng + ((P.n_layers + 1) & ~1));
  const int tid = threadIdx.x, lane = tid & 31;
  const int gwarp = (int)((blockIdx.x * blockDim.x + tid) >> 5);
  if (STRICT)
    for (int i = tid; i < (int)(sizeof(mcg_libm_tab) / 4); i += blockDim.x)
      reinterpret_cast<float *>(T)[i] = reinterpret_cast<const float *>(P.libm_tab)[i];
  for (int l = tid; l < P.n_layers; l += blockDim.x)
    s_rng[l] = make_int2(P.rings[l].lo - P.cell_lo, P.rings[l].hi - P.cell_lo);
  if (SMEM)
    for (int i = tid; i < P.n_cells; i += blockDim.x)
      s_tally[i] = 0ull;
  for (int i = tid; i < MCG_LQ; i += blockDim.x)
    lq_seq[i] = (unsigned)i; /* free for its first-lap ticket */
  if (tid < 4)
    lq_ctl[tid] = 0u;
  __syncthreads();
  unsigned long long *tally = SMEM ? s_tally : P.tally;
  const float min_w = P.min_w;
  const int qs = P.q_log2;
  const unsigned long long cap = P.cap;
  const int nl = P.n_layers;
  unsigned long long *const src_next = P.state + MCG_AQ_SRC_NEXT;
  unsigned long long *const done = P.state + MCG_AQ_DONE;
  long long *const pending = reinterpret_cast<long long *>(P.state + MCG_AQ_PENDING);

  uint64_t seed = 0;
  float x = 0.f, mu = 0.f, wmc = 0.f, inv_mu = 0.f;
  int idx = 0, L = 0, llo = 0, lhi = 0;
  uint32_t nst = 0, nsc = 0;
  bool active = false;
  unsigned long long n_hand = 0, steps = 0, scat = 0;
  unsigned long long seen_done = 0, seen_t = 0;
  /* every decision that steers the warp's control flow is taken on lane
   * 0's value, broadcast, so the lanes can never disagree */
  const unsigned long long t_start = __shfl_sync(0xffffffffu, mcg_globaltimer(), 0);
  unsigned long long iters = 0;
  int scan = gwarp % nl;
  unsigned sleep_ns = 128;
  unsigned long long stop = 0; /* 4: idle limit, 8: deadline */

  for (;;) {
    unsigned need = __ballot_sync(0xffffffffu, !active);
    if (need) {
      /* 0. the block's own hand-overs: claim the leading published run */
      {
        unsigned h = 0, e = 0;
        if (lane == 0) {
          h = *(volatile unsigned *)&lq_ctl[0];
          e = *(volatile unsigned *)&lq_ctl[1];
        }
        h = __shfl_sync(0xffffffffu, h, 0);
        e = __shfl_sync(0xffffffffu, e, 0);
        if ((int)(e - h) > 0) {
          const unsigned want = min((unsigned)__popc(need), e - h);
          const bool pub = (unsigned)lane < want &&
                           *(volatile unsigned *)&lq_seq[(h + lane) % MCG_LQ] == h + lane + 1u;
          const unsigned pm = __ballot_sync(0xffffffffu, pub);
          const int m = pm == 0xffffffffu ? 32 : __ffs(~pm) - 1;
          if (m > 0) {
            unsigned got = 0;
            if (lane == 0)
              got = atomicCAS(&lq_ctl[0], h, h + (unsigned)m);
            got = __shfl_sync(0xffffffffu, got, 0);
            if (got == h) {
              const int rank = __popc(need & lanemask_lt());
              if (((need >> lane) & 1u) && rank < m) {
                const unsigned t = h + (unsigned)rank, sl = t % MCG_LQ;
                int polls = 0;
                while (*(volatile unsigned *)&lq_seq[sl] != t + 1u && ++polls < (1 << 16))
                  ;
                if (polls >= (1 << 16))
                  atomicOr(&P.counters[MCG_CNT_ERR], 16ull);
                __threadfence_block();
                const mcg_particle q = lq_part[sl];
                const int ql = lq_L[sl];
                __threadfence_block();
                *(volatile unsigned *)&lq_seq[sl] = t + (unsigned)MCG_LQ; /* next lap */
                seed = q.seed, x = q.x, mu = q.mu, wmc = q.wmc, idx = q.index - P.cell_lo;
                L = ql;
                llo = s_rng[ql].x;
                lhi = s_rng[ql].y;
                inv_mu = mcg_flight_rcp(mu);
                nst = nsc = 0;
                active = true;
              }
              need = __ballot_sync(0xffffffffu, !active);
            }
          }
        }
      }
      /* (the global words below are read only while lanes are still idle:
       * the block's ring usually serves them all) */
      /* 1. queued particles, when the published count says there are some:
       * each lane looks at one or two rings from this warp's rotating
       * start; the warp tries to claim a run of published tickets from at
       * most four of the non-empty ones */
      long long pend = 0;
      if (lane == 0 && need)
        pend = (long long)mcg_ld_relaxed(reinterpret_cast<unsigned long long *>(pending));
      pend = __shfl_sync(0xffffffffu, pend, 0);
      if (pend > 0) {
        const int r0 = (scan + lane) % nl, r1 = (scan + lane + 32) % nl;
        const bool ne0 = lane < nl && mcg_ld_relaxed(&P.rings[r0].enq) > mcg_ld_relaxed(&P.rings[r0].deq);
        const bool ne1 = lane + 32 < nl && mcg_ld_relaxed(&P.rings[r1].enq) > mcg_ld_relaxed(&P.rings[r1].deq);
        unsigned long long cand = ((unsigned long long)__ballot_sync(0xffffffffu, ne1) << 32) |
                                  __ballot_sync(0xffffffffu, ne0);
        for (int tries = 0; tries < 4 && cand && need; ++tries) {
          const int j = __ffsll((long long)cand) - 1;
          cand &= cand - 1;
          const int l = (scan + j) % nl;
          mcg_aq_ring *R = &P.rings[l];
          unsigned long long h = 0, e = 0;
          if (lane == 0) {
            h = mcg_ld_relaxed(&R->deq);
            e = mcg_ld_relaxed(&R->enq);
          }
          h = __shfl_sync(0xffffffffu, h, 0);
          e = __shfl_sync(0xffffffffu, e, 0);
          if (e <= h)
            continue;
          const unsigned long long want = min((unsigned long long)__popc(need), e - h);
          const bool pub = (unsigned long long)lane < want &&
                           mcg_ld_relaxed(&P.seq[(size_t)l * cap + (h + lane) % cap]) == h + lane + 1;
          const unsigned pubmask = __ballot_sync(0xffffffffu, pub);
          const int m = pubmask == 0xffffffffu ? 32 : __ffs(~pubmask) - 1; /* leading run */
          if (m <= 0)
            continue;
          unsigned long long got = 0;
          if (lane == 0)
            got = atomicCAS(&R->deq, h, h + (unsigned long long)m);
          got = __shfl_sync(0xffffffffu, got, 0);
          if (got != h)
            continue; /* another warp claimed first */
          if (lane == 0)
            atomicAdd(reinterpret_cast<unsigned long long *>(pending), (unsigned long long)(-(long long)m));
          const int rank = __popc(need & lanemask_lt());
          if (((need >> lane) & 1u) && rank < m) {
            const unsigned long long t = h + rank;
            const size_t s = (size_t)l * cap + t % cap;
            /* the reading lane acquires the publication itself (another lane
             * saw it published, so this returns at once; bounded anyway) */
            int polls = 0;
            while (mcg_ld_acquire(&P.seq[s]) != t + 1 && ++polls < (1 << 16))
              __nanosleep(64);
            if (polls >= (1 << 16))
              atomicOr(&P.counters[MCG_CNT_ERR], 16ull);
            const mcg_particle q = P.slots[s];
            mcg_st_release(&P.seq[s], t + cap); /* free for the next lap */
            seed = q.seed, x = q.x, mu = q.mu, wmc = q.wmc, idx = q.index - P.cell_lo;
            L = l;
            llo = s_rng[l].x;
            lhi = s_rng[l].y;
            inv_mu = mcg_flight_rcp(mu);
            nst = nsc = 0;
            active = true;
          }
          need = __ballot_sync(0xffffffffu, !active);
        }
      }
      /* 2. newborns for the lanes still idle, while fewer than `inflight`
       * histories are born and unfinished: every ring entry is such a
       * history, and warps that pass this check together add at most 32
       * each, so no ring ever holds more than inflight + the grid's lanes
       * (the capacity the host sizes `inflight` from) */
      unsigned long long sn = 0, dn = 0;
      if (lane == 0 && need) {
        sn = mcg_ld_relaxed(src_next);
        dn = mcg_ld_relaxed(done);
      }
      sn = __shfl_sync(0xffffffffu, sn, 0);
      dn = __shfl_sync(0xffffffffu, dn, 0);
      if (need && sn < P.src_total && sn - dn < P.inflight) {
        unsigned long long base = 0;
        if (lane == 0)
          base = atomicAdd(src_next, (unsigned long long)__popc(need));
        base = __shfl_sync(0xffffffffu, base, 0);
        const int rank = __popc(need & lanemask_lt());
        if (((need >> lane) & 1u) && base + rank < P.src_total) {
          mcg_source_particle(P.src, (int64_t)(base + rank), seed, x, mu, wmc, idx);
          idx -= P.cell_lo;
          L = P.src_layer;
          llo = s_rng[L].x;
          lhi = s_rng[L].y;
          inv_mu = mcg_flight_rcp(mu);
          nst = nsc = 0;
          active = true;
        }
      }
      scan = (scan + 1) % nl;
    }
    ++iters;
    /* the deadline, the abort word and the error word: every 32 rounds of a
     * busy warp (three global reads), every round of an idle one */
    const bool idle = !__any_sync(0xffffffffu, active);
    unsigned long long now = 0, errw = 0;
    if (idle || (iters & 31u) == 0) {
      if (lane == 0) {
        now = mcg_globaltimer();
        errw = mcg_ld_relaxed(&P.counters[MCG_CNT_ERR]) | mcg_ld_relaxed(&P.state[MCG_AQ_ABORT]);
      }
      now = __shfl_sync(0xffffffffu, now, 0);
      errw = __shfl_sync(0xffffffffu, errw, 0);
    } else {
      now = t_start;
    }
    if (now - t_start > P.budget_ns || (errw & 32ull)) {
      /* the launch's deadline, or the host's abort: abandon what this warp
       * holds */
      stop = 8;
      break;
    }
    if (errw & 30ull)
      break; /* a full ring, or another warp gave up */
    if (idle) {
      /* nothing to do: finished, or wait (backing off) for hand-overs */
      unsigned long long d = 0;
      if (lane == 0)
        d = mcg_ld_relaxed(done);
      d = __shfl_sync(0xffffffffu, d, 0);
      if (d >= P.src_total)
        break;
      if (errw & 30ull)
        break; /* a full ring, or another warp gave up */
      if (d != seen_done || seen_t == 0) {
        seen_done = d;
        seen_t = now;
      } else if (now - seen_t > P.idle_limit_ns) {
        stop = 4;
        break;
      }
      __nanosleep(sleep_ns);
      sleep_ns = min(sleep_ns * 2u, 32768u);
      continue;
    }
    sleep_ns = 128;
    int dir = 0;
    bool finished = false;
    int k = 0;
    {
      /* the round: MCG_AQ_WINDOW steps per lane between two warp votes,
       * until MCG_AQ_ROUND_IDLE lanes are without a particle to step, one of
       * them newly (its particle left the sub-domain, ended, or reached the
       * round's cap), or no lane can step: the queues are visited when
       * there is something to hand over or to take, not every few steps */
      const uint32_t kcap = active ? min((uint32_t)MCG_AQ_ROUND_CAP, P.max_steps - nst) : 0u;
      for (;;) {
        bool go = ((uint32_t)k < kcap) & (wmc >= min_w) &
                  ((unsigned)(idx - llo) < (unsigned)(lhi - llo));
        for (int j = 0; go & (j < MCG_AQ_WINDOW); ++j) {
          mcg_step<STRICT, SMEM ? MCG_TALLY_SMEM32 : MCG_TALLY_GLOBAL, THIN>(
              seed, x, mu, wmc, inv_mu, idx, nsc, __ldg(P.cells + idx), &tally[idx], qs, T,
              P.libm);
          ++k;
          go = ((uint32_t)k < kcap) & (wmc >= min_w) &
               ((unsigned)(idx - llo) < (unsigned)(lhi - llo));
        }
        const unsigned gb = __ballot_sync(0xffffffffu, go);
        const unsigned fb = __ballot_sync(0xffffffffu, active & !go);
        if (!gb || (fb && __popc(~gb) >= MCG_AQ_ROUND_IDLE))
          break;
      }
    }
    if (active) {
      nst += (uint32_t)k;
      const bool going = (wmc >= min_w) & ((unsigned)(idx - llo) < (unsigned)(lhi - llo));
      if (!going || nst >= P.max_steps) {
        if (going)
          atomicOr(&P.counters[MCG_CNT_ERR], 1ull); /* the step limit */
        else if (idx == llo - 1)
          dir = L == 0 ? 0 : -1; /* the chain's ends leak (src/layer.cpp:47-48) */
        else if (idx == lhi)
          dir = L == nl - 1 ? 0 : 1;
        steps += nst;
        scat += nsc;
        finished = true;
        active = false;
      }
    }
    /* hand-over: to the block's ring while it has room (one shared atomic
     * per warp), else to the destination's global ring (one atomic per
     * destination and warp) */
    const unsigned movers = __ballot_sync(0xffffffffu, finished && dir != 0);
    bool published = false;
    bool local = false;
    if (movers) {
      unsigned h = 0, e = 0;
      if (lane == 0) {
        h = *(volatile unsigned *)&lq_ctl[0];
        e = *(volatile unsigned *)&lq_ctl[1];
      }
      h = __shfl_sync(0xffffffffu, h, 0);
      e = __shfl_sync(0xffffffffu, e, 0);
      local = e - h <= (unsigned)(MCG_LQ - 1024);
    }
    if (local && finished && dir != 0) {
      const int leader = __ffs(movers) - 1;
      unsigned base = 0;
      if (lane == leader)
        base = atomicAdd(&lq_ctl[1], (unsigned)__popc(movers));
      base = __shfl_sync(movers, base, leader);
      const unsigned t = base + __popc(movers & lanemask_lt()), sl = t % MCG_LQ;
      /* the slot's previous occupant is claimed; its reader frees it at once */
      int polls = 0;
      while (*(volatile unsigned *)&lq_seq[sl] != t && ++polls < (1 << 16))
        ;
      if (polls >= (1 << 16)) {
        atomicOr(&P.counters[MCG_CNT_ERR], 16ull);
      } else {
        mcg_particle o;
        o.seed = seed, o.x = x, o.mu = mu, o.wmc = wmc, o.index = idx + P.cell_lo;
        lq_part[sl] = o;
        lq_L[sl] = L + dir;
        __threadfence_block();
        *(volatile unsigned *)&lq_seq[sl] = t + 1u; /* publish */
      }
      ++n_hand;
    }
    if (!local && finished && dir != 0) {
      const int dst = L + dir;
      const unsigned peers = __match_any_sync(movers, dst);
      const int leader = __ffs(peers) - 1;
      unsigned long long base = 0;
      if (lane == leader)
        base = atomicAdd(&P.rings[dst].enq, (unsigned long long)__popc(peers));
      base = __shfl_sync(peers, base, leader);
      const unsigned long long t = base + __popc(peers & lanemask_lt());
      const size_t s = (size_t)dst * cap + t % cap;
      if (mcg_ld_acquire(&P.seq[s]) != t) {
        atomicOr(&P.counters[MCG_CNT_ERR], 2ull); /* the ring is full */
      } else {
        mcg_particle o;
        o.seed = seed, o.x = x, o.mu = mu, o.wmc = wmc, o.index = idx + P.cell_lo;
        P.slots[s] = o;
        mcg_st_release(&P.seq[s], t + 1); /* publish */
        published = true;
      }
      ++n_hand;
    }
    /* the published count and the finished histories, once per warp */
    const unsigned npub = __popc(__ballot_sync(0xffffffffu, published));
    const unsigned nfin = __popc(__ballot_sync(0xffffffffu, finished && dir == 0));
    if (lane == 0) {
      if (npub)
        atomicAdd(reinterpret_cast<unsigned long long *>(pending), (unsigned long long)npub);
      if (nfin)
        atomicAdd(done, (unsigned long long)nfin);
    }
  }
  if (lane == 0) {
    if (stop)
      atomicOr(&P.counters[MCG_CNT_ERR], stop);
    if (stop == 8)
      atomicAdd(&P.state[MCG_AQ_DEADLINE_HITS], 1ull);
    atomicMax(&P.state[MCG_AQ_ITERS], iters);
    atomicAdd(&P.state[MCG_AQ_EXITED], 1ull);
  }
  for (int o = 16; o > 0; o >>= 1) {
    n_hand += __shfl_down_sync(0xffffffffu, n_hand, o);
    steps += __shfl_down_sync(0xffffffffu, steps, o);
    scat += __shfl_down_sync(0xffffffffu, scat, o);
  }
  if (lane == 0) {
    if (n_hand)
      atomicAdd(&P.state[MCG_AQ_HANDOFFS], n_hand);
    atomicAdd(&P.counters[MCG_CNT_STEPS], steps);
    atomicAdd(&P.counters[MCG_CNT_SCAT], scat);
  }
  if (SMEM) {
    __syncthreads();
    for (int i = tid; i < P.n_cells; i += blockDim.x)
      if (s_tally[i])
        atomicAdd(&P.tally[i], s_tally[i]);
  }
}

/* Every slot free for its first-lap ticket: seq[l * cap + s] = s. */
__global__ void mcg_aq_init(unsigned long long *seq, unsigned long long total, unsigned long long cap)
{
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < total;
       i += (unsigned long long)gridDim.x * blockDim.x)
    seq[i] = i % cap;
}

extern "C" int mcg_worker_run_async(mcg_context *ctx, const mcg_source *src, int64_t n,
                                    int64_t queue_capacity, int64_t *h_handoffs)
{
  if (!ctx || !src || n < 0 || queue_capacity < 0)
    return mcg_fail(MCG_ERR_ARG, "mcg_worker_run_async: bad arguments");
  if (queue_capacity == 0) /* three times the resident threads: never overflows */
    queue_capacity = 3LL * 1024 * ctx->sm_count;
  if (!ctx->d_tally)
    return mcg_fail(MCG_ERR_STATE, "mcg_worker_run_async: no layers set");
  cudaSetDevice(ctx->device);
  const bool strict = ctx->mode == MCG_MODE_STRICT;
  if (strict && !ctx->libm_loaded) {
    int rc = mcg_load_libm(ctx);
    if (rc != MCG_OK)
      return rc;
  }
  const int P_ = ctx->n_layers;
  int src_layer = -1;
  std::vector<mcg_aq_ring> rings(P_);
  for (int l = 0; l < P_; ++l) {
    memset(&rings[l], 0, sizeof(rings[l]));
    rings[l].lo = ctx->layer_start[l];
    rings[l].hi = ctx->layer_start[l] + ctx->layer_m[l];
    if (src->cell0 >= rings[l].lo && src->cell0 < rings[l].hi)
      src_layer = l;
  }
  if (src_layer < 0)
    return mcg_fail(MCG_ERR_ARG, "mcg_worker_run_async: the source cell %d is outside the chain",
                    src->cell0);
  const unsigned long long cap = (unsigned long long)queue_capacity;
  const size_t o_rings = 0, o_c = worker_align(P_ * sizeof(mcg_aq_ring));
  const size_t o_seq = o_c + 256, o_slots = o_seq + worker_align((size_t)P_ * cap * 8);
  unsigned char *wb = nullptr;
  int rc = worker_buffer(ctx, o_slots + (size_t)P_ * cap * sizeof(mcg_particle), &wb);
  if (rc != MCG_OK)
    return rc;
  unsigned long long *state = reinterpret_cast<unsigned long long *>(wb + o_c);
  cudaError_t e;
  if ((e = cudaMemcpyAsync(wb + o_rings, rings.data(), P_ * sizeof(mcg_aq_ring),
                           cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess ||
      (e = cudaMemsetAsync(state, 0, 256, ctx->stream)) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_worker_run_async: set-up");
  mcg_aq_init<<<ctx->sm_count * 4, 256, 0, ctx->stream>>>(
      reinterpret_cast<unsigned long long *>(wb + o_seq), (unsigned long long)P_ * cap, cap);

  const size_t smem_base =
      sizeof(mcg_libm_tab) + MCG_LQ_BYTES + (size_t)((P_ + 1) & ~1) * sizeof(int2);
  const bool use_smem = smem_base + (size_t)ctx->n_cells * 8 <= (size_t)ctx->smem_optin;
  const size_t smem = smem_base + (use_smem ? (size_t)ctx->n_cells * 8 : 0);
  if (smem > (size_t)ctx->smem_optin)
    return mcg_fail(MCG_ERR_ARG, "mcg_worker_run_async: %d sub-domains too many", P_);
  mcg_async_params A;
  memset(&A, 0, sizeof(A));
  A.cells = strict ? ctx->d_cells_strict : ctx->d_cells_fast;
  A.n_layers = P_;
  A.cell_lo = ctx->cell_lo;
  A.n_cells = ctx->n_cells;
  A.src_layer = src_layer;
  A.rings = reinterpret_cast<mcg_aq_ring *>(wb + o_rings);
  A.seq = reinterpret_cast<unsigned long long *>(wb + o_seq);
  A.slots = reinterpret_cast<mcg_particle *>(wb + o_slots);
  A.cap = cap;
  A.src = *src;
  A.state = state;
  A.src_total = (unsigned long long)n;
  A.refill_steps = ctx->refill;
  A.min_w = ctx->min_w;
  A.q_log2 = ctx->log2_scale;
  A.tally = ctx->d_tally;
  A.counters = ctx->d_counters;
  A.libm = ctx->libm;
  A.libm_tab = ctx->libm_tab;
  A.max_steps = ctx->max_steps;
  A.idle_limit_ns = 2000000000ull; /* 2 s without any history finishing */
  /* the launch's deadline: 30 s plus 2 us per history (the benchmark slab
   * runs a history in about 40 ns of GPU time) */
  A.budget_ns = 30000000000ull + 2000ull * (unsigned long long)n;
  auto kern = strict ? (mcg_strict_thin(ctx) ? (use_smem ? mcg_worker_async<true, true, true>
                                              : mcg_worker_async<true, false, true>)
                                  : (use_smem ? mcg_worker_async<true, true, false>
                                              : mcg_worker_async<true, false, false>))
                     : (use_smem ? mcg_worker_async<false, true, false>
                                 : mcg_worker_async<false, false, false>);
  int bps = 1;
  if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                ctx->smem_optin)) != cudaSuccess ||
      (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, 1024, smem)) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_worker_run_async: launch set-up");
  /* no more blocks than the histories need (idle warps only poll) */
  const long long want = std::max<long long>(1, (n + 1023) / 1024);
  const int grid = (int)std::min<long long>((long long)ctx->sm_count * std::max(bps, 1), want);
  /* admission: a ring holds at most inflight + the grid's lanes particles,
   * so capacity - lanes histories in flight can never overflow a ring (a
   * smaller capacity still admits 32, and may overflow) */
  const long long lanes = (long long)grid * 1024;
  /* about one history per lane plus an eighth in transit: more would only
   * wait in the rings (and spill from the blocks' own rings to the global
   * ones) */
  A.inflight = (unsigned long long)std::max<long long>(
      32, std::min<long long>((long long)cap - lanes, lanes + lanes / 8));
  mcg_worker_state &WS = ctx->ext->worker;
  if (!WS.monitor && (e = cudaStreamCreateWithFlags(&WS.monitor, cudaStreamNonBlocking)) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_worker_run_async: monitor stream");
  cudaEventRecord(ctx->ev0, ctx->stream);
  kern<<<grid, 1024, smem, ctx->stream>>>(A);
  e = cudaGetLastError();
  cudaEventRecord(ctx->ev1, ctx->stream);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_worker_async launch");
  ctx->launches++;
  /* Host watchdog: the kernel stops itself at its deadline; if it has not
   * ended 10 s after that, the host raises the abort word (read by every
   * warp each round) from a second stream, and gives up 10 s later.  With
   * MCG_WORKER_TRACE set, progress is printed to stderr every second. */
  unsigned long long host[MCG_AQ_N] = {};
  {
    const bool trace = getenv("MCG_WORKER_TRACE") != nullptr;
    const double limit_s = A.budget_ns * 1e-9 + 10.0;
    const auto t0 = std::chrono::steady_clock::now();
    double next_trace = 1.0;
    bool aborted = false;
    for (;;) {
      e = cudaStreamQuery(ctx->stream);
      if (e != cudaErrorNotReady)
        break;
      std::this_thread::sleep_for(std::chrono::milliseconds(2));
      const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      if (trace && el >= next_trace) {
        next_trace += 1.0;
        if (cudaMemcpyAsync(host, state, sizeof(host), cudaMemcpyDeviceToHost, WS.monitor) == cudaSuccess &&
            cudaStreamSynchronize(WS.monitor) == cudaSuccess)
          fprintf(stderr, "worker_async %.1f s: done %llu born %llu pending %lld handoffs %llu "
                  "warps exited %llu\n", el, host[MCG_AQ_DONE], host[MCG_AQ_SRC_NEXT],
                  (long long)host[MCG_AQ_PENDING], host[MCG_AQ_HANDOFFS], host[MCG_AQ_EXITED]);
      }
      if (!aborted && el > limit_s) {
        static const unsigned long long abort_word = 32ull;
        cudaMemcpyAsync(state + MCG_AQ_ABORT, &abort_word, 8, cudaMemcpyHostToDevice, WS.monitor);
        cudaStreamSynchronize(WS.monitor);
        aborted = true;
      }
      if (el > limit_s + 10.0)
        return mcg_fail(MCG_ERR_TIMEOUT, "mcg_worker_run_async: the launch did not stop after "
                        "its deadline and an abort; the device context should be reset");
    }
  }
  if (e != cudaSuccess ||
      (e = cudaMemcpy(host, state, sizeof(host), cudaMemcpyDeviceToHost)) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_worker_run_async");
  cudaEventElapsedTime(&ctx->last_ms, ctx->ev0, ctx->ev1);
  unsigned long long err = 0;
  if ((e = cudaMemcpy(&err, ctx->d_counters + MCG_CNT_ERR, 8, cudaMemcpyDeviceToHost)) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_worker_run_async: error flags");
  if (err & 2)
    return mcg_fail(MCG_ERR_OVERFLOW, "mcg_worker_run_async: a hand-over ring overflowed "
                    "(capacity %lld)", (long long)queue_capacity);
  if (err & 28)
    return mcg_fail(MCG_ERR_TIMEOUT, "mcg_worker_run_async: %s (%llu of %lld histories done, "
                    "%llu born, %lld published and unclaimed, %llu warps at the deadline)",
                    (err & 8) ? "the launch's deadline passed"
                    : (err & 16) ? "a published particle stayed invisible"
                                 : "no history finished for 2 s",
                    host[MCG_AQ_DONE], (long long)n, host[MCG_AQ_SRC_NEXT],
                    (long long)host[MCG_AQ_PENDING], host[MCG_AQ_DEADLINE_HITS]);
  if (err & 1)
    return mcg_fail(MCG_ERR_LIMIT, "mcg_worker_run_async: a history exceeded the step limit");
  unsigned long long hcount = (unsigned long long)n;
  if ((e = cudaMemcpy(ctx->d_counters + MCG_CNT_HIST, &hcount, 8, cudaMemcpyHostToDevice)) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_worker_run_async: counters");
  if (h_handoffs)
    *h_handoffs = (int64_t)host[MCG_AQ_HANDOFFS];
  return MCG_OK;
}
