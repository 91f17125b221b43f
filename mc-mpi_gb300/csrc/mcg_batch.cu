/*
 * mcg_batch.cu - thousands of independent slabs of uneven size in one
 * persistent launch (the batched form of the tracker).
 *
 * Work is cut into items: up to `item_histories` consecutive histories of
 * one slab.  Items are sorted by expected cost (histories x cells, largest
 * first) and handed out through one global counter.  A block takes one item
 * at a time; when the item's slab differs from the block's current one it
 * flushes its shared-memory tally to the slab's global tally and zeroes it
 * for the new slab (at most max_cells 64-bit counters, 32 KB for 4096 cells).
 * Inside an item the warps refill their lanes from a block-local counter
 * exactly as the single-chain tracker does, so lanes stay busy across
 * histories of different lengths; the block synchronises only between
 * items.  The per-cell step table of every slab lives in HBM (16 B per cell)
 * and is read through L1.  The step is mcg_step (mcg_track.cuh), i.e.
 * Layer::particle_step of src/layer.cpp:123-190; with deferral on, it is
 * split into the certain crossing (mcg_step_cross) and the rest of the step
 * (mcg_step_rest), which a warp runs for its waiting lanes together.
 */
#include <algorithm>
#include <new>
#include <cmath>
#include <cstring>
#include <vector>

/* A warp whose lanes need both exp paths takes the general one for all: it
 * returns the small-argument path's bits wherever that applies.  Measured on
 * the batched kernels: about 0.5-1 % faster; on the single-chain tracker, whose
 * crossings almost all take the small path, 3 % slower, so it keeps the
 * per-lane choice. */
#define MCG_EXP_UNIFORM
#include "mcg_internal.h"
#include "mcg_track.cuh"

struct mcg_batch_item {
  int32_t slab, pad;
  int64_t first, count;
};

struct mcg_batch_params {
  const float4 *cells;
  const mcg_batch_slab_dev *slabs;
  const mcg_batch_item *items;
  int32_t n_items;
  int32_t max_cells;
  unsigned long long *item_next;
  unsigned long long *tally;
  unsigned long long *counters;
  mcg_libm_dev libm;
  const mcg_libm_tab *libm_tab;
  float min_w;
  int32_t q_log2;
  int32_t refill_steps;
  uint32_t max_steps;
  int32_t defer_lanes; /* DEFER: waiting lanes that trigger the full steps */
};

/* DEFER: certain crossings a lane takes between two of the warp's checks,
 * and the idle lanes (history ended) at which the warp refills */
#define MCG_DEFER_WINDOW 4
#define MCG_DEFER_REFILL 2

template <bool STRICT, int TALLY, bool DEFER>
__global__ void __launch_bounds__(1024) mcg_batch_kernel(mcg_batch_params P)
{
  extern __shared__ __align__(16) unsigned char smem[];
  mcg_libm_tab *T = reinterpret_cast<mcg_libm_tab *>(smem);
  unsigned long long *s_cnt = reinterpret_cast<unsigned long long *>(smem + sizeof(mcg_libm_tab));
  long long *s_ctl = reinterpret_cast<long long *>(s_cnt + 16); /* item, local history counter */
  unsigned long long *s_tally = reinterpret_cast<unsigned long long *>(s_ctl + 4);
  const int tid = threadIdx.x, lane = tid & 31;
  /* r-step jumps of the seed chain, s -> (A_r s + C_r) mod 2^63 for
   * r < 32: a warp finds the chain state of the first history of each
   * 32-history chunk it takes with one jump-ahead, run by all its lanes
   * together, and each lane its own from there with one multiply-add */
  __shared__ unsigned long long s_jump[64];
  if (tid < 32) {
    const uint64_t c = mcg_lcg_skip(0ull, (uint64_t)tid, 1);
    s_jump[tid] = (mcg_lcg_skip(1ull, (uint64_t)tid, 1) - c) & MCG_MASK63;
    s_jump[32 + tid] = c;
  }
  if (STRICT) {
    const float *src = reinterpret_cast<const float *>(P.libm_tab);
    float *dst = reinterpret_cast<float *>(T);
    for (int i = tid; i < (int)(sizeof(mcg_libm_tab) / 4); i += blockDim.x)
      dst[i] = src[i];
  }
  if (tid < 16)
    s_cnt[tid] = 0ull;
  const float min_w = P.min_w;
  const int qs = P.q_log2;
  int cur = -1, m = 0;
  const float4 *cells = nullptr;
  unsigned long long *gtally = nullptr;
  unsigned long long tot_steps = 0, tot_scat = 0;

  for (;;) {
    __syncthreads();
    if (tid == 0)
      s_ctl[0] = (long long)atomicAdd(P.item_next, 1ull);
    __syncthreads();
    const long long item = s_ctl[0];
    if (item >= P.n_items)
      break;
    const mcg_batch_item it = P.items[item];
    if (it.slab != cur) {
      if (cur >= 0 && TALLY != MCG_TALLY_GLOBAL)
        for (int i = tid; i < m; i += blockDim.x)
          if (s_tally[i])
            atomicAdd(&gtally[i], s_tally[i]);
      __syncthreads();
      cur = it.slab;
      const mcg_batch_slab_dev sd = P.slabs[cur];
      m = sd.m;
      cells = P.cells + sd.cell_off;
      gtally = P.tally + sd.cell_off;
      if (TALLY != MCG_TALLY_GLOBAL)
        for (int i = tid; i < m; i += blockDim.x)
          s_tally[i] = 0ull;
    }
    if (tid == 0)
      s_ctl[1] = 0;
    __syncthreads();
    const mcg_source S = P.slabs[cur].src;
    unsigned long long *tally = TALLY == MCG_TALLY_GLOBAL ? gtally : s_tally;

    /* lanes refill from the item's histories [0, it.count) */
    uint64_t seed = 0;
    float x = 0.f, mu = 0.f, wmc = 0.f, inv_mu = 0.f;
    float wres = 0.f; /* fast: the weight's rounding residue */
    int idx = 0;
    uint32_t nst = 0, nsc = 0;
    bool active = false;
    bool wait = false; /* DEFER: the lane's step waits for the full step */
    long long pool_next = 0, pool_end = 0;
    /* the chunk the pool lies in: its first history and that history's
     * seed-chain state (seed_mode 0) */
    long long pool_base = 0;
    uint64_t pool_seed = 0;
    bool drained = false;
    for (;;) {
      unsigned need = __ballot_sync(0xffffffffu, !active);
      if (need) {
        int cnt = __popc(need), rank = __popc(need & lanemask_lt());
        long long avail = pool_end - pool_next, my = -1, my_base = pool_base;
        uint64_t my_seed = pool_seed;
        if (rank < avail)
          my = pool_next + rank;
        if (cnt > avail && !drained) {
          long long base = 0;
          if (lane == 0)
            base = (long long)atomicAdd(reinterpret_cast<unsigned long long *>(&s_ctl[1]), 32ull);
          base = __shfl_sync(0xffffffffu, base, 0);
          if (base >= it.count) {
            drained = true;
            pool_next = pool_end = 0;
          } else {
            long long end = min(base + 32, (long long)it.count);
            long long r2 = rank - avail;
            pool_base = base;
            if (S.seed_mode == 0)
              pool_seed = mcg_lcg_skip(S.base_seed, (uint64_t)(it.first + base) + 1, 1);
            if (rank >= avail && r2 < end - base) {
              my = base + r2;
              my_base = base;
              my_seed = pool_seed;
            }
            pool_next = min(base + (cnt - avail), end);
            pool_end = end;
          }
        } else {
          pool_next += min((long long)cnt, avail);
        }
        if (!active && my >= 0) {
          if (S.seed_mode == 0) {
            const int r = (int)(my - my_base); /* 0 <= r < 32: my lies in its chunk */
            mcg_source_particle_at(S, (s_jump[r] * my_seed + s_jump[32 + r]) & MCG_MASK63, seed, x,
                                   mu, wmc, idx);
          } else {
            mcg_source_particle(S, it.first + my, seed, x, mu, wmc, idx);
          }
          inv_mu = mcg_flight_rcp(mu);
          wres = 0.f;
          nst = nsc = 0;
          active = true;
        }
      }
      if (!__any_sync(0xffffffffu, active))
        break;
      int k = 0;
      if (DEFER) {
        /* pooled deferral, run by the whole warp: a lane whose step is not
         * a certain crossing waits (mcg_step_cross has advanced only its
         * seed) while the others keep crossing, and the waiting lanes
         * complete their steps together (mcg_step_rest) once defer_lanes of
         * them wait or no other lane can step, so the long full step runs
         * with many lanes instead of once for every lane that needs it.
         * The round lasts until MCG_DEFER_REFILL lanes have ended their
         * histories (while the item has more) or no lane can step; a lane
         * may still wait when it ends, and its step completes in a later
         * round.  mcg_step_cross + mcg_step_rest perform exactly mcg_step
         * and each lane's steps keep their order: same results.  Every pass
         * steps a lane, makes one wait or completes the waiting steps, and
         * no lane passes its step limit, so the round ends. */
        const uint32_t kcap = active ? P.max_steps - nst : 0u;
        for (;;) {
          bool go = !wait & ((uint32_t)k < kcap) & (wmc >= min_w) & ((unsigned)idx < (unsigned)m);
          for (int j = 0; go & (j < MCG_DEFER_WINDOW); ++j) {
            if (!mcg_step_cross<STRICT, TALLY>(seed, x, mu, wmc, inv_mu, idx,
                                               __ldg(cells + idx), &tally[idx], qs, T, P.libm,
                                               nullptr, nullptr, nullptr,
                                               STRICT ? nullptr : &wres)) {
              wait = true;
              break;
            }
            ++k;
            go = ((uint32_t)k < kcap) & (wmc >= min_w) & ((unsigned)idx < (unsigned)m);
          }
          go &= !wait;
          const unsigned wb = __ballot_sync(0xffffffffu, wait);
          const unsigned gb = __ballot_sync(0xffffffffu, go);
          if (!wb && !gb)
            break;
          if (wb && (!gb || __popc(wb) >= P.defer_lanes)) {
            if (wait) {
              mcg_step_rest<STRICT, TALLY>(seed, x, mu, wmc, inv_mu, idx, nsc,
                                           __ldg(cells + idx), &tally[idx], qs, T, P.libm,
                                           nullptr, nullptr, nullptr, STRICT ? nullptr : &wres);
              ++k;
              wait = false;
            }
          } else if (!drained && __popc(~(wb | gb)) >= MCG_DEFER_REFILL) {
            break;
          }
        }
      } else if (active) {
        /* up to refill_steps steps, never past the step limit; one
         * unsigned compare is the slab's range test */
        const int kmax = (int)min((uint32_t)P.refill_steps, P.max_steps - nst);
        while ((k < kmax) & (wmc >= min_w) & ((unsigned)idx < (unsigned)m)) {
          mcg_step<STRICT, TALLY>(seed, x, mu, wmc, inv_mu, idx, nsc, __ldg(cells + idx),
                                  &tally[idx], qs, T, P.libm, nullptr, nullptr, nullptr,
                                  STRICT ? nullptr : &wres);
          ++k;
        }
      }
      if (active)
        nst += (uint32_t)k;
      if (active && !wait) {
        const bool going = (wmc >= min_w) & ((unsigned)idx < (unsigned)m);
        if (!going || nst >= P.max_steps) {
          /* a history still alive in the slab here has reached the limit */
          const bool in = (wmc >= min_w) && ((unsigned)idx < (unsigned)m);
          int r;
          if (in)
            r = 2;
          else if (idx == -1)
            r = -1;
          else if (idx == m)
            r = 1;
          else if (wmc < min_w)
            r = 0;
          else
            r = -1;
          atomicAdd(&s_cnt[MCG_CNT_HIST], 1ull);
          const unsigned long long wq =
              (unsigned long long)(mcg_to_fixed(wmc, qs) + (STRICT ? 0ll : mcg_to_fixed(wres, qs)));
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
          tot_steps += nst;
          tot_scat += nsc;
          active = false;
        }
      }
    }
  }
  if (cur >= 0 && TALLY != MCG_TALLY_GLOBAL)
    for (int i = tid; i < m; i += blockDim.x)
      if (s_tally[i])
        atomicAdd(&gtally[i], s_tally[i]);
  for (int o = 16; o > 0; o >>= 1) {
    tot_steps += __shfl_down_sync(0xffffffffu, tot_steps, o);
    tot_scat += __shfl_down_sync(0xffffffffu, tot_scat, o);
  }
  if (lane == 0) {
    atomicAdd(&s_cnt[MCG_CNT_STEPS], tot_steps);
    atomicAdd(&s_cnt[MCG_CNT_SCAT], tot_scat);
  }
  __syncthreads();
  if (tid < MCG_CNT_N && s_cnt[tid]) {
    if (tid == MCG_CNT_ERR)
      atomicOr(&P.counters[tid], s_cnt[tid]);
    else
      atomicAdd(&P.counters[tid], s_cnt[tid]);
  }
}

/* ------------------------------------------------------------ host side */
static mcg_batch_state *batch_of(mcg_context *ctx)
{
  if (!ctx->ext)
    ctx->ext = new mcg_ext();
  return &ctx->ext->batch;
}

static void batch_free(mcg_batch_state *B)
{
  for (void *p : {B->d_slabs, B->d_items, (void *)B->d_cells_strict, (void *)B->d_cells_fast,
                  (void *)B->d_tally, (void *)B->d_item_next, (void *)B->d_hist0})
    if (p)
      cudaFree(p);
  if (B->graph)
    cudaGraphExecDestroy(B->graph);
  *B = mcg_batch_state();
}

void mcg_adjoint_release(mcg_adj_state *A);

void mcg_ext_destroy(mcg_context *ctx)
{
  if (!ctx->ext)
    return;
  batch_free(&ctx->ext->batch);
  mcg_adjoint_release(&ctx->ext->adj);
  if (ctx->ext->worker.dev)
    cudaFree(ctx->ext->worker.dev);
  if (ctx->ext->worker.monitor)
    cudaStreamDestroy(ctx->ext->worker.monitor);
  delete ctx->ext;
  ctx->ext = nullptr;
}

extern "C" int mcg_batch_set(mcg_context *ctx, int32_t n_slabs, const mcg_slab *h_slabs,
                             const float *h_sigs, const float *h_rates, float particle_min_weight)
{
  if (!ctx || n_slabs <= 0 || !h_slabs || !h_sigs || !h_rates)
    return mcg_fail(MCG_ERR_ARG, "mcg_batch_set: bad arguments");
  int64_t total = 0, hist = 0;
  int maxc = 0;
  for (int s = 0; s < n_slabs; ++s) {
    const mcg_slab &sl = h_slabs[s];
    if (sl.n_cells <= 0 || sl.n_histories < 0 || sl.seed_mode < 0 || sl.seed_mode > 1 ||
        sl.isotropic < 0 || sl.isotropic > 2)
      return mcg_fail(MCG_ERR_ARG, "mcg_batch_set: bad slab %d", s);
    total += sl.n_cells;
    hist += sl.n_histories;
    maxc = std::max(maxc, sl.n_cells);
  }
  const size_t smem_need = sizeof(mcg_libm_tab) + 16 * 8 + 4 * 8 + (size_t)maxc * 8;
  if (total > INT32_MAX || smem_need > (size_t)ctx->smem_optin)
    return mcg_fail(MCG_ERR_ARG, "mcg_batch_set: %lld cells / largest slab %d cells too large",
                    (long long)total, maxc);
  std::vector<float4> cs, cf;
  std::vector<mcg_batch_slab_dev> sd;
  try {
    cs.resize(total);
    cf.resize(total);
    sd.resize(n_slabs);
  } catch (const std::bad_alloc &) {
    return mcg_fail(MCG_ERR_ARG, "mcg_batch_set: no host memory for %lld cells", (long long)total);
  }
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  mcg_batch_state *B = batch_of(ctx);
  const int keep_block = B->block, keep_tm = B->tally_mode;
  const int keep_defer = B->defer;
  const int64_t keep_item = B->item_histories;
  batch_free(B);
  B->block = keep_block;
  B->tally_mode = keep_tm;
  B->defer = keep_defer;
  B->item_histories = keep_item;
  B->n_slabs = n_slabs;
  B->total_cells = (int)total;
  B->max_cells = maxc;
  B->total_histories = hist;
  B->min_w = particle_min_weight;
  B->slabs.assign(h_slabs, h_slabs + n_slabs);
  B->cell_off.resize(n_slabs);
  int64_t off = 0;
  for (int s = 0; s < n_slabs; ++s) {
    const mcg_slab &sl = h_slabs[s];
    B->cell_off[s] = (int32_t)off;
    const float dx = (1.0f - 0.0f) / (float)sl.n_cells; /* Layer(0, 1, 0, m): src/layer.cpp:47 */
    for (int j = 0; j < sl.n_cells; ++j)
      mcg_cell_params(h_sigs[off + j], h_rates[off + j], j, dx, cs[off + j], cf[off + j]);
    sd[s].cell_off = (int32_t)off;
    sd[s].m = sl.n_cells;
    sd[s].src.seed_mode = sl.seed_mode;
    sd[s].src.isotropic = sl.isotropic;
    sd[s].src.base_seed = sl.base_seed;
    sd[s].src.x0 = 0.0f;
    sd[s].src.mu0 = sl.mu0;
    sd[s].src.w0 = sl.w0;
    sd[s].src.cell0 = 0;
    off += sl.n_cells;
  }
  /* any failure from here on leaves no slabs set (launches return
   * MCG_ERR_STATE), with the launch shape kept */
  auto fail = [&](cudaError_t err, const char *what) {
    batch_free(B);
    B->block = keep_block;
    B->tally_mode = keep_tm;
    B->defer = keep_defer;
    B->item_histories = keep_item;
    return mcg_cuda_fail(err, what);
  };
  cudaError_t e;
  if ((e = mcg_dev_malloc((void **)&B->d_cells_strict, total * sizeof(float4))) != cudaSuccess ||
      (e = mcg_dev_malloc((void **)&B->d_cells_fast, total * sizeof(float4))) != cudaSuccess ||
      (e = mcg_dev_malloc((void **)&B->d_tally, total * sizeof(unsigned long long))) != cudaSuccess ||
      (e = mcg_dev_malloc(&B->d_slabs, n_slabs * sizeof(mcg_batch_slab_dev))) != cudaSuccess ||
      (e = mcg_dev_malloc((void **)&B->d_item_next, 64)) != cudaSuccess)
    return fail(e, "mcg_batch_set: cudaMalloc");
  if ((e = cudaMemcpy(B->d_cells_strict, cs.data(), total * sizeof(float4), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(B->d_cells_fast, cf.data(), total * sizeof(float4), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(B->d_slabs, sd.data(), n_slabs * sizeof(mcg_batch_slab_dev), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemset(B->d_tally, 0, total * sizeof(unsigned long long))) != cudaSuccess)
    return fail(e, "mcg_batch_set: upload");
  return mcg_tally_reset(ctx) == MCG_OK ? MCG_OK : MCG_ERR_CUDA;
}

/* Items of `item` histories, sorted by expected cost, optionally only the
 * first `fraction` of every slab's histories (autotuner samples). */
static int build_items(mcg_context *ctx, mcg_batch_state *B, int64_t item, double fraction)
{
  std::vector<mcg_batch_item> items;
  std::vector<double> cost;
  for (int s = 0; s < B->n_slabs; ++s) {
    int64_t n = B->slabs[s].n_histories;
    if (fraction < 1.0)
      n = std::max<int64_t>(std::min<int64_t>(n, 32), (int64_t)std::ceil(n * fraction));
    for (int64_t f = 0; f < n; f += item) {
      mcg_batch_item it;
      it.slab = s;
      it.pad = 0;
      it.first = f;
      it.count = std::min(item, n - f);
      items.push_back(it);
      cost.push_back((double)it.count * (double)B->slabs[s].n_cells);
    }
  }
  std::vector<size_t> order(items.size());
  for (size_t i = 0; i < order.size(); ++i)
    order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
  std::vector<mcg_batch_item> sorted(items.size());
  for (size_t i = 0; i < order.size(); ++i)
    sorted[i] = items[order[i]];
  if ((int)sorted.size() > B->items_cap) {
    if (B->d_items)
      cudaFree(B->d_items);
    B->d_items = nullptr;
    cudaError_t e = cudaMalloc(&B->d_items, sorted.size() * sizeof(mcg_batch_item));
    if (e != cudaSuccess)
      return mcg_cuda_fail(e, "mcg_batch: cudaMalloc(items)");
    B->items_cap = (int)sorted.size();
  }
  cudaError_t e = cudaMemcpy(B->d_items, sorted.data(), sorted.size() * sizeof(mcg_batch_item),
                             cudaMemcpyHostToDevice);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_batch: upload items");
  B->n_items = (int)sorted.size();
  B->graph_valid = false;
  return MCG_OK;
}

struct mcg_batch_launch {
  void (*kern)(mcg_batch_params);
  mcg_batch_params P;
  size_t smem;
  int grid;
};

/* Kernel choice, attributes and grid: done outside any stream capture. */
static int batch_configure(mcg_context *ctx, mcg_batch_state *B, mcg_batch_launch &L)
{
  const bool strict = ctx->mode == MCG_MODE_STRICT;
  mcg_batch_params &P = L.P;
  memset(&P, 0, sizeof(P));
  P.cells = strict ? B->d_cells_strict : B->d_cells_fast;
  P.slabs = static_cast<const mcg_batch_slab_dev *>(B->d_slabs);
  P.items = static_cast<const mcg_batch_item *>(B->d_items);
  P.n_items = B->n_items;
  P.max_cells = B->max_cells;
  P.item_next = B->d_item_next;
  P.tally = B->d_tally;
  P.counters = ctx->d_counters;
  P.libm = ctx->libm;
  P.libm_tab = ctx->libm_tab;
  P.min_w = B->min_w;
  P.q_log2 = ctx->log2_scale;
  P.refill_steps = ctx->refill;
  P.max_steps = ctx->max_steps;
  const int tm = B->tally_mode;
  L.smem = sizeof(mcg_libm_tab) + 16 * 8 + 4 * 8 +
           (tm == MCG_TALLY_GLOBAL ? 0 : (size_t)B->max_cells * 8);
  /* deferral is built for the shared-memory 32-bit tally (the autotuner's
   * candidates); other tally modes run without it */
  P.defer_lanes = B->defer;
  if (strict && B->defer && tm == MCG_TALLY_SMEM32)
    L.kern = mcg_batch_kernel<true, MCG_TALLY_SMEM32, true>;
  else if (!strict && B->defer && tm == MCG_TALLY_SMEM32)
    L.kern = mcg_batch_kernel<false, MCG_TALLY_SMEM32, true>;
  else if (strict)
    L.kern = tm == MCG_TALLY_SMEM64 ? mcg_batch_kernel<true, MCG_TALLY_SMEM64, false>
           : tm == MCG_TALLY_SMEM32 ? mcg_batch_kernel<true, MCG_TALLY_SMEM32, false>
                                    : mcg_batch_kernel<true, MCG_TALLY_GLOBAL, false>;
  else
    L.kern = tm == MCG_TALLY_SMEM64 ? mcg_batch_kernel<false, MCG_TALLY_SMEM64, false>
           : tm == MCG_TALLY_SMEM32 ? mcg_batch_kernel<false, MCG_TALLY_SMEM32, false>
                                    : mcg_batch_kernel<false, MCG_TALLY_GLOBAL, false>;
  cudaError_t e = cudaFuncSetAttribute(L.kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)L.smem);
  int bps = 0;
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, L.kern, B->block, L.smem);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_batch: launch set-up");
  L.grid = ctx->sm_count * std::max(bps, 1);
  return MCG_OK;
}

static int batch_enqueue(mcg_context *ctx, mcg_batch_state *B, const mcg_batch_launch &L)
{
  cudaError_t e;
  if ((e = cudaMemsetAsync(B->d_item_next, 0, 8, ctx->stream)) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_batch: memset");
  L.kern<<<L.grid, B->block, L.smem, ctx->stream>>>(L.P);
  if ((e = cudaGetLastError()) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_batch_kernel launch");
  ctx->last_grid = L.grid;
  ctx->last_block = B->block;
  ctx->launches++;
  return MCG_OK;
}

/* First history of each slab for the event engine, with the same sampled
 * history counts as build_items at this fraction; returns the total. */
static int build_hist0(mcg_batch_state *B, double fraction, unsigned long long *total)
{
  std::vector<unsigned long long> h0(B->n_slabs);
  unsigned long long t = 0;
  for (int s = 0; s < B->n_slabs; ++s) {
    int64_t n = B->slabs[s].n_histories;
    if (fraction < 1.0)
      n = std::max<int64_t>(std::min<int64_t>(n, 32), (int64_t)std::ceil(n * fraction));
    h0[s] = t;
    t += (unsigned long long)n;
  }
  *total = t;
  if (B->hist0_fraction == fraction && B->d_hist0)
    return MCG_OK;
  cudaError_t e = cudaSuccess;
  if (!B->d_hist0)
    e = cudaMalloc(&B->d_hist0, (size_t)B->n_slabs * sizeof(unsigned long long));
  if (e == cudaSuccess)
    e = cudaMemcpy(B->d_hist0, h0.data(), h0.size() * sizeof(unsigned long long),
                   cudaMemcpyHostToDevice);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_batch: slab history offsets");
  B->hist0_fraction = fraction;
  return MCG_OK;
}

/* One batched run with the event engine (histories at this fraction). */
static int batch_run_event(mcg_context *ctx, mcg_batch_state *B, double fraction, int steps)
{
  unsigned long long total = 0;
  int rc = build_hist0(B, fraction, &total);
  if (rc != MCG_OK)
    return rc;
  const bool strict = ctx->mode == MCG_MODE_STRICT;
  return mcg_event_run_slabs(ctx, strict ? B->d_cells_strict : B->d_cells_fast, B->d_tally,
                             B->d_slabs, B->d_hist0, B->n_slabs, total, B->min_w, steps);
}

static int batch_prepare(mcg_context *ctx, mcg_batch_state **out)
{
  if (!ctx || !ctx->ext || ctx->ext->batch.n_slabs == 0)
    return mcg_fail(MCG_ERR_STATE, "mcg_batch: no slabs set (mcg_batch_set)");
  int rc = MCG_OK;
  if (ctx->mode == MCG_MODE_STRICT && !ctx->libm_loaded)
    rc = mcg_load_libm(ctx);
  cudaSetDevice(ctx->device);
  *out = &ctx->ext->batch;
  return rc;
}

extern "C" int mcg_batch_run(mcg_context *ctx)
{
  mcg_batch_state *B;
  int rc = batch_prepare(ctx, &B);
  if (rc != MCG_OK)
    return rc;
  if (B->algorithm == MCG_ALGO_EVENT) {
    if ((rc = batch_run_event(ctx, B, 1.0, B->event_steps)) != MCG_OK)
      return rc;
    return mcg_sync(ctx);
  }
  if (B->items_built_for != (int)B->item_histories) {
    if ((rc = build_items(ctx, B, B->item_histories, 1.0)) != MCG_OK)
      return rc;
    B->items_built_for = (int)B->item_histories;
  }
  cudaError_t e;
  if (!B->graph_valid) {
    if (B->graph) {
      cudaGraphExecDestroy(B->graph);
      B->graph = nullptr;
    }
    mcg_batch_launch L;
    if ((rc = batch_configure(ctx, B, L)) != MCG_OK)
      return rc;
    cudaGraph_t g;
    if ((e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
      return mcg_cuda_fail(e, "mcg_batch_run: begin capture");
    rc = batch_enqueue(ctx, B, L);
    e = cudaStreamEndCapture(ctx->stream, &g);
    if (rc != MCG_OK)
      return rc;
    if (e != cudaSuccess)
      return mcg_cuda_fail(e, "mcg_batch_run: end capture");
    e = cudaGraphInstantiate(&B->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess)
      return mcg_cuda_fail(e, "mcg_batch_run: instantiate");
    B->graph_valid = true;
  }
  cudaEventRecord(ctx->ev0, ctx->stream);
  e = cudaGraphLaunch(B->graph, ctx->stream);
  cudaEventRecord(ctx->ev1, ctx->stream);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_batch_run: graph launch");
  return mcg_sync(ctx);
}

extern "C" int mcg_batch_run_per_slab(mcg_context *ctx)
{
  mcg_batch_state *B;
  int rc = batch_prepare(ctx, &B);
  if (rc != MCG_OK)
    return rc;
  const bool strict = ctx->mode == MCG_MODE_STRICT;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, ctx->stream);
  for (int s = 0; s < B->n_slabs && rc == MCG_OK; ++s) {
    const mcg_slab &sl = B->slabs[s];
    if (sl.n_histories == 0)
      continue;
    mcg_track_params P;
    memset(&P, 0, sizeof(P));
    P.cells = (strict ? B->d_cells_strict : B->d_cells_fast) + B->cell_off[s];
    P.n_cells = sl.n_cells;
    P.cell_lo = 0;
    P.min_w = B->min_w;
    P.q_log2 = ctx->log2_scale;
    P.n = sl.n_histories;
    P.src.seed_mode = sl.seed_mode;
    P.src.isotropic = sl.isotropic;
    P.src.base_seed = sl.base_seed;
    P.src.mu0 = sl.mu0;
    P.src.w0 = sl.w0;
    P.next = ctx->d_next;
    P.tally = B->d_tally + B->cell_off[s];
    P.counters = ctx->d_counters;
    P.libm = ctx->libm;
    P.libm_tab = ctx->libm_tab;
    P.refill_steps = ctx->refill;
    P.chunk = 64;
    P.max_steps = ctx->max_steps;
    const int block = ((size_t)sl.n_cells * 64 <= 24 * 1024) ? 256 : 1024;
    const int warps = block / 32;
    const int copies = ((size_t)sl.n_cells * 8 * warps <= 24 * 1024) ? warps : 1;
    P.tally_copies = copies;
    const size_t smem = sizeof(mcg_libm_tab) + 16 * 8 + (size_t)sl.n_cells * 8 * copies;
    auto kern = strict ? mcg_track_kernel<true, MCG_TALLY_SMEM32, false>
                       : mcg_track_kernel<false, MCG_TALLY_SMEM32, false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    int bps = 1;
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, block, smem);
    long long want = (sl.n_histories + block - 1) / block;
    const int grid = (int)std::min<long long>((long long)ctx->sm_count * std::max(bps, 1), want);
    if (e == cudaSuccess)
      e = cudaMemsetAsync(ctx->d_next, 0, 8, ctx->stream);
    if (e == cudaSuccess) {
      kern<<<grid, block, smem, ctx->stream>>>(P);
      e = cudaGetLastError();
    }
    if (e != cudaSuccess)
      rc = mcg_cuda_fail(e, "mcg_batch_run_per_slab");
    ctx->launches++;
  }
  cudaEventRecord(b, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc != MCG_OK)
    return rc;
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_batch_run_per_slab: execution");
  rc = mcg_sync(ctx);
  ctx->last_ms = ms;
  return rc;
}

extern "C" int mcg_batch_tally_reset(mcg_context *ctx)
{
  mcg_batch_state *B;
  int rc = batch_prepare(ctx, &B);
  if (rc != MCG_OK)
    return rc;
  cudaError_t e = cudaMemsetAsync(B->d_tally, 0, B->total_cells * sizeof(unsigned long long),
                                  ctx->stream);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_batch_tally_reset");
  return mcg_tally_reset(ctx);
}

extern "C" int mcg_batch_tally_read(mcg_context *ctx, int64_t *h_q, double *h_f64)
{
  mcg_batch_state *B;
  int rc = batch_prepare(ctx, &B);
  if (rc != MCG_OK)
    return rc;
  std::vector<int64_t> q(B->total_cells);
  cudaError_t e = cudaMemcpyAsync(q.data(), B->d_tally, q.size() * sizeof(int64_t),
                                  cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_batch_tally_read");
  const double inv = std::ldexp(1.0, -ctx->log2_scale);
  for (size_t i = 0; i < q.size(); ++i) {
    if (h_q)
      h_q[i] = q[i];
    if (h_f64)
      h_f64[i] = (double)q[i] * inv;
  }
  return MCG_OK;
}

extern "C" int mcg_batch_set_launch(mcg_context *ctx, int32_t block, int64_t item_histories,
                                    int32_t tally_mode)
{
  if (!ctx || (block && block != 256 && block != 512 && block != 1024) || item_histories < 0 ||
      tally_mode < -1 || tally_mode > 2)
    return mcg_fail(MCG_ERR_ARG, "mcg_batch_set_launch: bad arguments");
  mcg_batch_state *B = batch_of(ctx);
  if (block)
    B->block = block;
  if (item_histories)
    B->item_histories = item_histories;
  if (tally_mode >= 0)
    B->tally_mode = tally_mode;
  B->graph_valid = false;
  return MCG_OK;
}

extern "C" int mcg_batch_set_deferral(mcg_context *ctx, int32_t defer)
{
  if (!ctx || defer < 0 || defer > 32)
    return mcg_fail(MCG_ERR_ARG, "mcg_batch_set_deferral: bad arguments");
  mcg_batch_state *B = batch_of(ctx);
  B->defer = defer;
  B->graph_valid = false;
  return MCG_OK;
}

extern "C" int mcg_batch_set_algorithm(mcg_context *ctx, int32_t algorithm, int32_t steps_per_pass)
{
  if (!ctx || (algorithm != MCG_ALGO_HISTORY && algorithm != MCG_ALGO_EVENT) || steps_per_pass < 0)
    return mcg_fail(MCG_ERR_ARG, "mcg_batch_set_algorithm: bad arguments");
  mcg_batch_state *B = batch_of(ctx);
  B->algorithm = algorithm;
  B->event_steps = steps_per_pass ? steps_per_pass : 8;
  return MCG_OK;
}

extern "C" int mcg_batch_autotune(mcg_context *ctx, double sample_fraction, mcg_batch_tuning *out)
{
  mcg_batch_state *B;
  int rc = batch_prepare(ctx, &B);
  if (rc != MCG_OK)
    return rc;
  if (!(sample_fraction > 0.0 && sample_fraction <= 1.0))
    return mcg_fail(MCG_ERR_ARG, "mcg_batch_autotune: sample fraction must be in (0, 1]");
  const int blocks[] = {256, 512, 1024};
  const int64_t items[] = {4096, 16384, 65536};
  /* tally mode and deferral of the full step (waiting lanes) */
  const int shapes[][2] = {{MCG_TALLY_SMEM32, 0}, {MCG_TALLY_SMEM32, 4}, {MCG_TALLY_SMEM32, 8},
                           {MCG_TALLY_SMEM64, 0}};
  /* every candidate runs the same sample, of at least four times the event
   * engine's drain size (below it the event-based form is a single drain
   * launch, and a persistent launch is dominated by its tail), or the whole
   * run; candidates compete on time per history */
  unsigned long long n_full = 0, n_hist = 0;
  if ((rc = build_hist0(B, 1.0, &n_full)) != MCG_OK)
    return rc;
  sample_fraction = std::min(
      1.0, std::max(sample_fraction, 4.0 * (double)mcg_event_drain_below(ctx) / (double)n_full));
  if ((rc = build_hist0(B, sample_fraction, &n_hist)) != MCG_OK)
    return rc;
  const double f_event = sample_fraction;
  const unsigned long long n_event = n_hist;
  double best = 1e30; /* ms per history */
  int nc = 0;
  mcg_batch_tuning pick = {B->block, B->tally_mode, B->item_histories, 0.f, 0, MCG_ALGO_HISTORY,
                           0, B->defer};
  bool warmed = false;
  for (int64_t it : items) {
    /* the sample keeps the full run's number of items per slab, so the
     * item-level tail the candidate would see is represented */
    const int64_t sample_item = std::max<int64_t>(32, (int64_t)std::llround(it * sample_fraction));
    if ((rc = build_items(ctx, B, sample_item, sample_fraction)) != MCG_OK)
      return rc;
    for (int bl : blocks)
      for (const auto &sh : shapes) {
        const int tm = sh[0];
        B->block = bl;
        B->tally_mode = tm;
        B->defer = sh[1];
        mcg_batch_launch L;
        if ((rc = batch_configure(ctx, B, L)) != MCG_OK)
          return rc;
        for (int rep = warmed ? 1 : 0; rep < 2; ++rep) { /* the very first run warms up */
          cudaEventRecord(ctx->ev0, ctx->stream);
          if ((rc = batch_enqueue(ctx, B, L)) != MCG_OK)
            return rc;
          cudaEventRecord(ctx->ev1, ctx->stream);
          if ((rc = mcg_sync(ctx)) != MCG_OK)
            return rc;
        }
        warmed = true;
        ++nc;
        if (ctx->last_ms / (double)n_hist < best) {
          best = ctx->last_ms / (double)n_hist;
          pick = {bl, tm, it, ctx->last_ms, 0, MCG_ALGO_HISTORY, 0, sh[1]};
        }
      }
  }
  /* the event-based form */
  for (int k : {4, 16}) {
    for (int rep = 0; rep < 2; ++rep) /* the first run sizes the bank */
      if ((rc = batch_run_event(ctx, B, f_event, k)) != MCG_OK || (rc = mcg_sync(ctx)) != MCG_OK)
        return rc;
    ++nc;
    if (ctx->last_ms / (double)n_event < best) {
      best = ctx->last_ms / (double)n_event;
      pick = {B->block, B->tally_mode, B->item_histories, ctx->last_ms, 0, MCG_ALGO_EVENT, k, 0};
    }
  }
  B->algorithm = pick.algorithm;
  if (pick.algorithm == MCG_ALGO_EVENT)
    B->event_steps = pick.steps_per_pass;
  B->block = pick.block;
  B->tally_mode = pick.tally_mode;
  B->item_histories = pick.item_histories;
  B->defer = pick.defer;
  B->items_built_for = -1;
  B->graph_valid = false;
  pick.candidates = nc;
  if (out)
    *out = pick;
  return mcg_batch_tally_reset(ctx);
}
