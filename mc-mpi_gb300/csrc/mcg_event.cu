/*
 * mcg_event.cu - event-based variant of the tracker.
 *
 * Live particles sit in a structure-of-arrays bank (seed u64; x, mu, wmc
 * f32; cell, history or slab, step and scatter counts i32) of fixed
 * capacity.  One pass:
 *   1. flight kernel: every live particle draws its flight sample; a certain
 *      crossing (the common event of a fine mesh) is completed at once, up to
 *      K of them per pass; a particle whose event is not a certain crossing
 *      is moved into the collision queue, its state advanced to the
 *      flight sample's (which determines the sample); survivors are
 *      compacted into the other bank.  Threads take four consecutive
 *      particles and read each field with one 128-bit load; warp ballots and
 *      popc give every survivor and every queued particle its slot, one
 *      atomic per warp and destination reserves the warp's range;
 *   2. collision kernel: the queued events (scatters, near-ties, the
 *      reference's EPS cases) complete their step from that state in
 *      converged warps and join the bank;
 *   3. newborns from the source top the bank up to its capacity.
 * When the source is exhausted and fewer particles than a full grid remain,
 * one history-based launch finishes them (instead of one pass per event of
 * the longest history).  Particles that end write their result and final
 * state by history index.  Deposits go to the global 64-bit fixed-point
 * tally.  The step is mcg_step_cross + mcg_step_rest (Layer::particle_step,
 * src/layer.cpp:123-190), so results are identical to the history-based
 * tracker's, particle by particle.
 *
 * The engine serves one chain (mcg_set_algorithm) and the batched slabs
 * (mcg_batch_set_algorithm; the bank then carries the slab index).
 * Memory per particle and pass: 40 B read + 40 B written (+ 40 B each way
 * through the queue for a collision).
 */
#include <algorithm>
#include <cstring>

#include "mcg_internal.h"
#include "mcg_track.cuh"

/* 512-thread blocks, two per SM: with a block's 80 KB copy of a 10k-cell
 * tally that is 32 warps per SM (measured 1.36x the events/s of 256-thread
 * blocks at 16 events per pass, despite a few registers spilled) */
#define MCG_EV_BLOCK 512
#define MCG_EV_MIN_BLOCKS 2

struct mcg_ev_params {
  const float4 *cells;          /* chain-local (chain) or slab-concatenated cells */
  unsigned long long *tally;    /* same indexing */
  int32_t n_cells, cell_lo;     /* chain: cells and global index of cell 0 */
  /* slab mode */
  const mcg_batch_slab_dev *slabs;
  const unsigned long long *slab_hist0; /* first history of each slab, ascending */
  int32_t n_slabs;
  /* chain mode: births and outputs by history */
  mcg_track_params tp;
  float min_w;
  int32_t q_log2, steps_per_pass;
  uint32_t max_steps;
  unsigned long long cap;
  mcg_soa in, out, q;
  mcg_ev_ctl *ctl;
  unsigned long long *counters;
  mcg_libm_dev libm;
  const mcg_libm_tab *libm_tab;
};

/* A lane's particle. */
struct mcg_ev_particle {
  uint64_t seed;
  float x, mu, wmc, res; /* res: the fast weight's rounding residue */
  int32_t idx, hid, nst, nsc;
};

__device__ __forceinline__ void mcg_ev_store(const mcg_soa &b, unsigned long long i,
                                             const mcg_ev_particle &p)
{
  b.seed[i] = p.seed;
  b.x[i] = p.x;
  b.mu[i] = p.mu;
  b.wmc[i] = p.wmc;
  b.res[i] = p.res;
  b.idx[i] = p.idx;
  b.hid[i] = p.hid;
  b.nst[i] = p.nst;
  b.nsc[i] = p.nsc;
}

/* Particles 4q..4q+3 of a bank (those below n), 128-bit loads for full quads. */
__device__ __forceinline__ void mcg_ev_load4(const mcg_soa &b, unsigned long long q,
                                             unsigned long long n, mcg_ev_particle p[4],
                                             bool live[4])
{
  const unsigned long long i0 = 4 * q;
  if (i0 + 3 < n) {
    const ulonglong2 s01 = reinterpret_cast<const ulonglong2 *>(b.seed)[2 * q];
    const ulonglong2 s23 = reinterpret_cast<const ulonglong2 *>(b.seed)[2 * q + 1];
    const float4 vx = reinterpret_cast<const float4 *>(b.x)[q];
    const float4 vm = reinterpret_cast<const float4 *>(b.mu)[q];
    const float4 vw = reinterpret_cast<const float4 *>(b.wmc)[q];
    const float4 vr = reinterpret_cast<const float4 *>(b.res)[q];
    const int4 vi = reinterpret_cast<const int4 *>(b.idx)[q];
    const int4 vh = reinterpret_cast<const int4 *>(b.hid)[q];
    const int4 vs = reinterpret_cast<const int4 *>(b.nst)[q];
    const int4 vc = reinterpret_cast<const int4 *>(b.nsc)[q];
    p[0].seed = s01.x, p[1].seed = s01.y, p[2].seed = s23.x, p[3].seed = s23.y;
    p[0].x = vx.x, p[1].x = vx.y, p[2].x = vx.z, p[3].x = vx.w;
    p[0].mu = vm.x, p[1].mu = vm.y, p[2].mu = vm.z, p[3].mu = vm.w;
    p[0].wmc = vw.x, p[1].wmc = vw.y, p[2].wmc = vw.z, p[3].wmc = vw.w;
    p[0].res = vr.x, p[1].res = vr.y, p[2].res = vr.z, p[3].res = vr.w;
    p[0].idx = vi.x, p[1].idx = vi.y, p[2].idx = vi.z, p[3].idx = vi.w;
    p[0].hid = vh.x, p[1].hid = vh.y, p[2].hid = vh.z, p[3].hid = vh.w;
    p[0].nst = vs.x, p[1].nst = vs.y, p[2].nst = vs.z, p[3].nst = vs.w;
    p[0].nsc = vc.x, p[1].nsc = vc.y, p[2].nsc = vc.z, p[3].nsc = vc.w;
#pragma unroll
    for (int j = 0; j < 4; ++j)
      live[j] = true;
  } else {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const unsigned long long i = i0 + j;
      live[j] = i < n;
      if (live[j]) {
        p[j].seed = b.seed[i];
        p[j].x = b.x[i];
        p[j].mu = b.mu[i];
        p[j].wmc = b.wmc[i];
        p[j].res = b.res[i];
        p[j].idx = b.idx[i];
        p[j].hid = b.hid[i];
        p[j].nst = b.nst[i];
        p[j].nsc = b.nsc[i];
      }
    }
  }
}

/* Cells, cell count and tally of a particle's chain or slab. */
template <bool SLABS>
__device__ __forceinline__ void mcg_ev_geometry(const mcg_ev_params &P, const mcg_ev_particle &p,
                                                const float4 *&cells,
                                                unsigned long long *&tally, int &m)
{
  if (SLABS) {
    const mcg_batch_slab_dev sd = P.slabs[p.hid];
    cells = P.cells + sd.cell_off;
    tally = P.tally + sd.cell_off;
    m = sd.m;
  } else {
    cells = P.cells;
    tally = P.tally;
    m = P.n_cells;
  }
}

/* End of a history: outputs by history index (chain mode) and counters. */
template <bool SLABS>
__device__ __forceinline__ void mcg_ev_finish(const mcg_ev_params &P, const mcg_ev_particle &p,
                                              int m, unsigned long long *s_cnt)
{
  const bool in = (p.wmc >= P.min_w) && ((unsigned)p.idx < (unsigned)m);
  const int r = in ? 2 : p.idx == -1 ? -1 : p.idx == m ? 1 : p.wmc < P.min_w ? 0 : -1;
  if (!SLABS) {
    const int h = p.hid;
    if (P.tp.particles) {
      mcg_particle o;
      o.seed = p.seed;
      o.x = p.x;
      o.mu = p.mu;
      o.wmc = p.wmc;
      o.index = p.idx + P.cell_lo;
      P.tp.particles[h] = o;
    }
    if (P.tp.results)
      P.tp.results[h] = r;
    if (P.tp.steps)
      P.tp.steps[h] = p.nst;
    if (P.tp.scatters)
      P.tp.scatters[h] = p.nsc;
  }
  atomicAdd(&s_cnt[MCG_CNT_HIST], 1ull);
  /* the weight with its rounding residue (zero in strict mode) */
  const unsigned long long wq =
      (unsigned long long)(mcg_to_fixed(p.wmc, P.q_log2) + mcg_to_fixed(p.res, P.q_log2));
  if (r == -1) {
    atomicAdd(&s_cnt[MCG_CNT_LEFT], 1ull);
    atomicAdd(&s_cnt[MCG_CNT_WLEFT], wq);
  } else if (r == 1) {
    atomicAdd(&s_cnt[MCG_CNT_RIGHT], 1ull);
    atomicAdd(&s_cnt[MCG_CNT_WRIGHT], wq);
  } else if (r == 0) {
    atomicAdd(&s_cnt[MCG_CNT_KILL], 1ull);
    atomicAdd(&s_cnt[MCG_CNT_WKILL], wq);
  } else {
    atomicOr(&s_cnt[MCG_CNT_ERR], 1ull);
  }
}

/* Block counters -> context counters. */
__device__ __forceinline__ void mcg_ev_flush_counters(const mcg_ev_params &P,
                                                      unsigned long long *s_cnt,
                                                      unsigned long long steps,
                                                      unsigned long long scat)
{
  for (int o = 16; o > 0; o >>= 1) {
    steps += __shfl_down_sync(0xffffffffu, steps, o);
    scat += __shfl_down_sync(0xffffffffu, scat, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&s_cnt[MCG_CNT_STEPS], steps);
    atomicAdd(&s_cnt[MCG_CNT_SCAT], scat);
  }
  __syncthreads();
  if (threadIdx.x < MCG_CNT_N && s_cnt[threadIdx.x]) {
    if (threadIdx.x == MCG_CNT_ERR)
      atomicOr(&P.counters[threadIdx.x], s_cnt[threadIdx.x]);
    else
      atomicAdd(&P.counters[threadIdx.x], s_cnt[threadIdx.x]);
  }
}

/* A block's shared-memory chain tally -> the global tally (after the block
 * synchronisation inside mcg_ev_flush_counters). */
__device__ __forceinline__ void mcg_ev_flush_tally(const mcg_ev_params &P,
                                                   const unsigned long long *s_tally)
{
  for (int i = threadIdx.x; i < P.n_cells; i += blockDim.x)
    if (s_tally[i])
      atomicAdd(&P.tally[i], s_tally[i]);
}

/* Warp-compacted append of the lanes with `want` to a bank; one atomic per
 * warp on *count reserves the warp's range. */
__device__ __forceinline__ void mcg_ev_append(const mcg_soa &b, unsigned long long *count,
                                              bool want, const mcg_ev_particle &p)
{
  const unsigned ball = __ballot_sync(0xffffffffu, want);
  if (!ball)
    return;
  const int lane = threadIdx.x & 31;
  unsigned long long base = 0;
  if (lane == __ffs(ball) - 1)
    base = atomicAdd(count, (unsigned long long)__popc(ball));
  base = __shfl_sync(0xffffffffu, base, __ffs(ball) - 1);
  if (want)
    mcg_ev_store(b, base + __popc(ball & lanemask_lt()), p);
}

/* Pass part 1: certain crossings, up to K per particle; other events go to
 * the collision queue with their state advanced to the flight sample's. */
template <bool STRICT, bool SLABS, bool SMEM>
__global__ void __launch_bounds__(MCG_EV_BLOCK, MCG_EV_MIN_BLOCKS) mcg_ev_flight_kernel(mcg_ev_params P)
{
  __shared__ mcg_libm_tab T;
  __shared__ unsigned long long s_cnt[16];
  extern __shared__ unsigned long long s_tally[]; /* SMEM: the chain's tally */
  const int tid = threadIdx.x;
  if (STRICT)
    for (int i = tid; i < (int)(sizeof(mcg_libm_tab) / 4); i += blockDim.x)
      reinterpret_cast<float *>(&T)[i] = reinterpret_cast<const float *>(P.libm_tab)[i];
  if (tid < 16)
    s_cnt[tid] = 0ull;
  if (SMEM)
    for (int i = tid; i < P.n_cells; i += blockDim.x)
      s_tally[i] = 0ull;
  __syncthreads();
  const unsigned long long n = P.ctl->n_in, n4 = (n + 3) / 4;
  unsigned long long steps = 0;
  /* whole warps iterate together so the ballots see every lane */
  for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x; base < n4;
       base += (unsigned long long)gridDim.x * blockDim.x) {
    mcg_ev_particle p[4];
    bool live[4], queued[4];
    mcg_ev_load4(P.in, base + tid, n, p, live);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      queued[j] = false;
      if (!live[j])
        continue;
      const float4 *cells;
      unsigned long long *tally;
      int m;
      mcg_ev_geometry<SLABS>(P, p[j], cells, tally, m);
      if (SMEM)
        tally = s_tally;
      float inv_mu = mcg_flight_rcp(p[j].mu);
      const int kmax = (int)min((uint32_t)P.steps_per_pass, P.max_steps - (uint32_t)p[j].nst);
      int k = 0;
      bool ended = false;
      for (; k < kmax; ++k) {
        if (!((p[j].wmc >= P.min_w) & ((unsigned)p[j].idx < (unsigned)m))) {
          ended = true;
          break;
        }
        if (!mcg_step_cross<STRICT, SMEM ? MCG_TALLY_SMEM32 : MCG_TALLY_GLOBAL>(p[j].seed, p[j].x, p[j].mu, p[j].wmc,
                                                      inv_mu, p[j].idx, __ldg(cells + p[j].idx),
                                                      &tally[p[j].idx], P.q_log2, &T, P.libm,
                                                      nullptr, nullptr, nullptr,
                                                      STRICT ? nullptr : &p[j].res)) {
          queued[j] = true;
          break;
        }
      }
      p[j].nst += k;
      steps += (unsigned long long)k;
      if (!queued[j] && !ended &&
          (!((p[j].wmc >= P.min_w) & ((unsigned)p[j].idx < (unsigned)m)) ||
           (uint32_t)p[j].nst >= P.max_steps))
        ended = true;
      if (ended) {
        mcg_ev_finish<SLABS>(P, p[j], m, s_cnt);
        live[j] = false;
      } else if (queued[j]) {
        live[j] = false;
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      mcg_ev_append(P.out, &P.ctl->n_out, live[j], p[j]);
      mcg_ev_append(P.q, &P.ctl->n_q, queued[j], p[j]);
    }
  }
  mcg_ev_flush_counters(P, s_cnt, steps, 0ull);
  if (SMEM)
    mcg_ev_flush_tally(P, s_tally);
}

/* Pass part 2: the queued events complete their step from the stored
 * sample; survivors join the bank. */
template <bool STRICT, bool SLABS, bool SMEM>
__global__ void __launch_bounds__(MCG_EV_BLOCK, MCG_EV_MIN_BLOCKS) mcg_ev_collide_kernel(mcg_ev_params P)
{
  __shared__ mcg_libm_tab T;
  __shared__ unsigned long long s_cnt[16];
  extern __shared__ unsigned long long s_tally[]; /* SMEM: the chain's tally */
  const int tid = threadIdx.x;
  if (STRICT)
    for (int i = tid; i < (int)(sizeof(mcg_libm_tab) / 4); i += blockDim.x)
      reinterpret_cast<float *>(&T)[i] = reinterpret_cast<const float *>(P.libm_tab)[i];
  if (tid < 16)
    s_cnt[tid] = 0ull;
  if (SMEM)
    for (int i = tid; i < P.n_cells; i += blockDim.x)
      s_tally[i] = 0ull;
  __syncthreads();
  const unsigned long long n = P.ctl->n_q, n4 = (n + 3) / 4;
  unsigned long long steps = 0, scat = 0;
  for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x; base < n4;
       base += (unsigned long long)gridDim.x * blockDim.x) {
    mcg_ev_particle p[4];
    bool live[4];
    mcg_ev_load4(P.q, base + tid, n, p, live);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (!live[j])
        continue;
      const float4 *cells;
      unsigned long long *tally;
      int m;
      mcg_ev_geometry<SLABS>(P, p[j], cells, tally, m);
      if (SMEM)
        tally = s_tally;
      float inv_mu = mcg_flight_rcp(p[j].mu);
      uint32_t sc = (uint32_t)p[j].nsc;
      mcg_step_rest<STRICT, SMEM ? MCG_TALLY_SMEM32 : MCG_TALLY_GLOBAL>(p[j].seed, p[j].x, p[j].mu, p[j].wmc, inv_mu,
                                              p[j].idx, sc, __ldg(cells + p[j].idx),
                                              &tally[p[j].idx], P.q_log2, &T, P.libm,
                                              nullptr, nullptr, nullptr,
                                              STRICT ? nullptr : &p[j].res);
      scat += sc - (uint32_t)p[j].nsc;
      p[j].nsc = (int)sc;
      ++p[j].nst;
      ++steps;
      if (!((p[j].wmc >= P.min_w) & ((unsigned)p[j].idx < (unsigned)m)) ||
          (uint32_t)p[j].nst >= P.max_steps) {
        mcg_ev_finish<SLABS>(P, p[j], m, s_cnt);
        live[j] = false;
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
      mcg_ev_append(P.out, &P.ctl->n_out, live[j], p[j]);
  }
  mcg_ev_flush_counters(P, s_cnt, steps, scat);
  if (SMEM)
    mcg_ev_flush_tally(P, s_tally);
}

/* Pass part 3 (one thread): this pass's newborns fill the bank up to its
 * capacity; the counters roll over to the next pass. */
__global__ void mcg_ev_birth_ctl_kernel(mcg_ev_ctl *c, unsigned long long cap)
{
  const unsigned long long room = cap - c->n_out, left = c->total - c->next;
  const unsigned long long born = room < left ? room : left;
  c->birth_base = c->n_out;
  c->birth_n = born;
  c->birth_first = c->next;
  c->next += born;
  c->n_in = c->n_out + born;
  c->n_out = 0;
  c->n_q = 0;
  c->passes++;
}

/* Newborn g of the run: particle g of the chain's input (array or source),
 * or history g - hist0[s] of slab s's source. */
template <bool SLABS>
__global__ void mcg_ev_birth_kernel(mcg_ev_params P)
{
  const unsigned long long nb = P.ctl->birth_n, base = P.ctl->birth_base;
  const unsigned long long first = P.ctl->birth_first;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < nb;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long g = first + i;
    mcg_ev_particle p;
    int idx;
    if (SLABS) {
      int a = 0, b = P.n_slabs - 1; /* the last slab with hist0 <= g */
      while (a < b) {
        const int mid = (a + b + 1) >> 1;
        if (P.slab_hist0[mid] <= g)
          a = mid;
        else
          b = mid - 1;
      }
      mcg_source_particle(P.slabs[a].src, (int64_t)(g - P.slab_hist0[a]), p.seed, p.x, p.mu,
                          p.wmc, idx);
      p.hid = a;
    } else {
      mcg_load_particle(P.tp, (int64_t)g, p.seed, p.x, p.mu, p.wmc, idx);
      idx -= P.cell_lo;
      p.hid = (int32_t)g;
    }
    p.idx = idx;
    p.nst = p.nsc = 0;
    p.res = 0.f;
    mcg_ev_store(P.out, base + i, p);
  }
}

/* The last particles of a run, once the source is exhausted and fewer than
 * a full grid remain: one thread carries each to its end. */
template <bool STRICT, bool SLABS, bool SMEM>
__global__ void __launch_bounds__(MCG_EV_BLOCK, MCG_EV_MIN_BLOCKS) mcg_ev_drain_kernel(mcg_ev_params P)
{
  __shared__ mcg_libm_tab T;
  __shared__ unsigned long long s_cnt[16];
  extern __shared__ unsigned long long s_tally[]; /* SMEM: the chain's tally */
  const int tid = threadIdx.x;
  if (STRICT)
    for (int i = tid; i < (int)(sizeof(mcg_libm_tab) / 4); i += blockDim.x)
      reinterpret_cast<float *>(&T)[i] = reinterpret_cast<const float *>(P.libm_tab)[i];
  if (tid < 16)
    s_cnt[tid] = 0ull;
  if (SMEM)
    for (int i = tid; i < P.n_cells; i += blockDim.x)
      s_tally[i] = 0ull;
  __syncthreads();
  const unsigned long long n = P.ctl->n_in;
  unsigned long long steps = 0, scat = 0;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + tid; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    mcg_ev_particle p;
    p.seed = P.in.seed[i];
    p.x = P.in.x[i];
    p.mu = P.in.mu[i];
    p.wmc = P.in.wmc[i];
    p.res = P.in.res[i];
    p.idx = P.in.idx[i];
    p.hid = P.in.hid[i];
    p.nst = P.in.nst[i];
    p.nsc = P.in.nsc[i];
    const float4 *cells;
    unsigned long long *tally;
    int m;
    mcg_ev_geometry<SLABS>(P, p, cells, tally, m);
    if (SMEM)
      tally = s_tally;
    float inv_mu = mcg_flight_rcp(p.mu);
    uint32_t sc = (uint32_t)p.nsc, st = (uint32_t)p.nst;
    const uint32_t st0 = st, sc0 = sc;
    while ((p.wmc >= P.min_w) && ((unsigned)p.idx < (unsigned)m) && st < P.max_steps) {
      mcg_step<STRICT, SMEM ? MCG_TALLY_SMEM32 : MCG_TALLY_GLOBAL>(p.seed, p.x, p.mu, p.wmc,
                                                                  inv_mu, p.idx, sc,
                                         __ldg(cells + p.idx), &tally[p.idx], P.q_log2, &T,
                                         P.libm, nullptr, nullptr, nullptr,
                                         STRICT ? nullptr : &p.res);
      ++st;
    }
    steps += st - st0;
    scat += sc - sc0;
    p.nst = (int)st;
    p.nsc = (int)sc;
    mcg_ev_finish<SLABS>(P, p, m, s_cnt);
  }
  mcg_ev_flush_counters(P, s_cnt, steps, scat);
  if (SMEM)
    mcg_ev_flush_tally(P, s_tally);
}

/* ------------------------------------------------------------ host side */
static int soa_alloc(mcg_soa &s, size_t cap, std::vector<void *> &owned)
{
  void *base = nullptr;
  /* one allocation, each field 256-byte aligned (128-bit loads of quads) */
  const size_t pad = (cap + 63) & ~(size_t)63;
  cudaError_t e = cudaMalloc(&base, pad * (8 + 8 * 4));
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "event buffers");
  owned.push_back(base);
  char *p = static_cast<char *>(base);
  s.seed = reinterpret_cast<unsigned long long *>(p);
  p += pad * 8;
  float **f[4] = {&s.x, &s.mu, &s.wmc, &s.res};
  for (float **q : f) {
    *q = reinterpret_cast<float *>(p);
    p += pad * 4;
  }
  int32_t **ii[4] = {&s.idx, &s.hid, &s.nst, &s.nsc};
  for (int32_t **q : ii) {
    *q = reinterpret_cast<int32_t *>(p);
    p += pad * 4;
  }
  return MCG_OK;
}

static int ev_reserve(mcg_context *ctx, size_t cap)
{
  if (cap <= ctx->event_cap)
    return MCG_OK;
  for (void *p : ctx->event_owned)
    cudaFree(p);
  ctx->event_owned.clear();
  ctx->event_cap = 0;
  ctx->event_ctl = nullptr;
  int rc;
  for (int b = 0; b < 3; ++b)
    if ((rc = soa_alloc(ctx->event_buf[b], cap, ctx->event_owned)) != MCG_OK)
      return rc;
  void *c = nullptr;
  cudaError_t e = cudaMalloc(&c, sizeof(mcg_ev_ctl));
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "event counters");
  ctx->event_owned.push_back(c);
  ctx->event_ctl = static_cast<mcg_ev_ctl *>(c);
  ctx->event_cap = cap;
  return MCG_OK;
}

/* Bank capacity: the whole run when it is small, else 2^24 particles (about
 * 2 GB for the two banks and the queue). */
static size_t ev_capacity(unsigned long long total)
{
  const unsigned long long c = std::min<unsigned long long>(total, 1ull << 24);
  return (size_t)std::max<unsigned long long>(64, (c + 63) & ~63ull);
}

template <bool STRICT, bool SLABS, bool SMEM>
static int ev_run_t(mcg_context *ctx, mcg_ev_params &P, unsigned long long total)
{
  const size_t cap = ev_capacity(total);
  int rc = ev_reserve(ctx, cap);
  if (rc != MCG_OK)
    return rc;
  P.cap = cap;
  P.ctl = ctx->event_ctl;
  if (P.steps_per_pass <= 0)
    P.steps_per_pass = std::max(1, ctx->event_steps);
  mcg_ev_ctl c0;
  memset(&c0, 0, sizeof(c0));
  c0.total = total;
  cudaError_t e = cudaMemcpyAsync(P.ctl, &c0, sizeof(c0), cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "event counters");
  const size_t smem = SMEM ? (size_t)P.n_cells * 8 : 0;
  if (SMEM)
    for (const void *k : {(const void *)mcg_ev_flight_kernel<STRICT, SLABS, SMEM>,
                          (const void *)mcg_ev_drain_kernel<STRICT, SLABS, SMEM>})
      if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
          cudaSuccess)
        return mcg_cuda_fail(e, "event kernels: shared memory");
  int bps = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, mcg_ev_flight_kernel<STRICT, SLABS, SMEM>,
                                                MCG_EV_BLOCK, smem);
  const int grid = ctx->sm_count * std::max(bps, 1);
  const unsigned long long drain_below = mcg_event_drain_below(ctx);
  mcg_soa cur = ctx->event_buf[0], other = ctx->event_buf[1];
  P.q = ctx->event_buf[2];
  cudaEventRecord(ctx->ev0, ctx->stream);
  /* the first newborns */
  P.out = cur;
  mcg_ev_birth_ctl_kernel<<<1, 1, 0, ctx->stream>>>(P.ctl, cap);
  mcg_ev_birth_kernel<SLABS><<<grid, MCG_EV_BLOCK, 0, ctx->stream>>>(P);
  ctx->launches += 2;
  unsigned long long passes = 0;
  const unsigned long long max_passes =
      ((unsigned long long)ctx->max_steps / P.steps_per_pass + 2) * (total / cap + 2);
  for (;;) {
    for (int g = 0; g < 8; ++g, ++passes) {
      P.in = cur;
      P.out = other;
      mcg_ev_flight_kernel<STRICT, SLABS, SMEM><<<grid, MCG_EV_BLOCK, smem, ctx->stream>>>(P);
      /* the queue holds few events, scattered over the chain: global atomics
       * cost less than clearing and flushing a block copy of the tally */
      mcg_ev_collide_kernel<STRICT, SLABS, false><<<grid, MCG_EV_BLOCK, 0, ctx->stream>>>(P);
      mcg_ev_birth_ctl_kernel<<<1, 1, 0, ctx->stream>>>(P.ctl, cap);
      mcg_ev_birth_kernel<SLABS><<<grid, MCG_EV_BLOCK, 0, ctx->stream>>>(P);
      ctx->launches += 4;
      std::swap(cur, other);
    }
    mcg_ev_ctl c;
    if ((e = cudaGetLastError()) != cudaSuccess ||
        (e = cudaMemcpyAsync(&c, P.ctl, sizeof(c), cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess)
      return mcg_cuda_fail(e, "event passes");
    if (c.next == c.total && c.n_in <= drain_below) {
      /* the source is exhausted and the bank no longer fills the GPU */
      P.in = cur;
      if (c.n_in) {
        mcg_ev_drain_kernel<STRICT, SLABS, SMEM><<<grid, MCG_EV_BLOCK, smem, ctx->stream>>>(P);
        ctx->launches++;
      }
      break;
    }
    if (passes > max_passes)
      return mcg_fail(MCG_ERR_LIMIT, "event mode: particles still alive after %llu passes",
                      passes);
  }
  cudaEventRecord(ctx->ev1, ctx->stream);
  if ((e = cudaGetLastError()) != cudaSuccess)
    return mcg_cuda_fail(e, "event drain");
  ctx->last_grid = grid;
  ctx->last_block = 256;
  ctx->event_passes = (int)std::min<unsigned long long>(passes, 0x7fffffff);
  return MCG_OK;
}

/* Chain mode: the histories of one context (mcg_set_algorithm). */
int mcg_event_run(mcg_context *ctx, mcg_track_params &TP)
{
  if (TP.n > 0x7fffffffLL)
    return mcg_fail(MCG_ERR_ARG, "event mode: at most 2^31-1 particles per call");
  if (TP.n == 0)
    return MCG_OK;
  mcg_ev_params P;
  memset(&P, 0, sizeof(P));
  P.cells = TP.cells;
  P.tally = TP.tally;
  P.n_cells = TP.n_cells;
  P.cell_lo = TP.cell_lo;
  P.tp = TP;
  P.min_w = TP.min_w;
  P.q_log2 = TP.q_log2;
  P.max_steps = TP.max_steps;
  P.counters = TP.counters;
  P.libm = TP.libm;
  P.libm_tab = TP.libm_tab;
  /* the chain's tally in shared memory when two blocks' copies fit on an SM
   * (in a fine mesh every block deposits all along the chain: global atomics
   * would contend on the cells the particles stream through together) */
  const unsigned long long n = (unsigned long long)TP.n;
  const bool smem = (size_t)TP.n_cells * 8 + sizeof(mcg_libm_tab) + 256 <= (size_t)ctx->smem_optin / 2;
  if (ctx->mode == MCG_MODE_STRICT)
    return smem ? ev_run_t<true, false, true>(ctx, P, n) : ev_run_t<true, false, false>(ctx, P, n);
  return smem ? ev_run_t<false, false, true>(ctx, P, n) : ev_run_t<false, false, false>(ctx, P, n);
}

/* Slab mode: the batched slabs (mcg_batch_run with the event algorithm). */
int mcg_event_run_slabs(mcg_context *ctx, const float4 *cells, unsigned long long *tally,
                        const void *slabs, const unsigned long long *slab_hist0, int n_slabs,
                        unsigned long long total, float min_w, int steps_per_pass)
{
  if (total == 0)
    return MCG_OK;
  mcg_ev_params P;
  memset(&P, 0, sizeof(P));
  P.cells = cells;
  P.tally = tally;
  P.slabs = static_cast<const mcg_batch_slab_dev *>(slabs);
  P.slab_hist0 = slab_hist0;
  P.n_slabs = n_slabs;
  P.min_w = min_w;
  P.steps_per_pass = steps_per_pass;
  P.q_log2 = ctx->log2_scale;
  P.max_steps = ctx->max_steps;
  P.counters = ctx->d_counters;
  P.libm = ctx->libm;
  P.libm_tab = ctx->libm_tab;
  return ctx->mode == MCG_MODE_STRICT ? ev_run_t<true, true, false>(ctx, P, total)
                                      : ev_run_t<false, true, false>(ctx, P, total);
}

extern "C" int mcg_set_algorithm(mcg_context *ctx, int32_t algorithm, int32_t steps_per_pass)
{
  if (!ctx || (algorithm != MCG_ALGO_HISTORY && algorithm != MCG_ALGO_EVENT) || steps_per_pass < 0)
    return mcg_fail(MCG_ERR_ARG, "mcg_set_algorithm: bad arguments");
  ctx->algorithm = algorithm;
  ctx->event_steps = steps_per_pass ? steps_per_pass : 1;
  return MCG_OK;
}
