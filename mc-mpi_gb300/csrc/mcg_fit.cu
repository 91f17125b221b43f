/*
 * mcg_fit.cu - batched inverse fit of per-cell absorption cross sections.
 *
 * Many independent slabs (each a Layer(0, 1, 0, m)) with known scattering
 * cross sections and measured absorption tallies t_c (weight absorbed per
 * history); the fit minimises L = sum over all cells of (a_c - t_c)^2, a_c the
 * simulated tally, over every cell's sig_a by Adam.  One Adam step is:
 *   1. one launch of the batched forward + adjoint kernel: each lane runs a
 *      history of its work item's slab forward (tally + G = sum w_c dep)
 *      and replays it from its seed accumulating dG/dsig_a (the pathwise
 *      derivative of mcg_adjoint.cu); the loss weights are
 *      w_c = 2 (a_c - t_c) from the previous step's tally (lagged by one
 *      step, so a single pass per step suffices);
 *   2. a kernel forming the new weights and the loss from this step's tally;
 *   3. the Adam update of every sig_a, written straight into the step table.
 * The three kernels are captured once in a CUDA graph and replayed for every
 * step; each step simulates fresh histories (source indices step * n + i).
 */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mcg_internal.h"
#include "mcg_track.cuh"

struct mcg_fit_slab_dev {
  int32_t cell_off, m;
  int64_t n_hist;
  mcg_source src;
};

struct mcg_fit_item {
  int32_t slab, pad;
  int64_t first, count;
};

struct mcg_fit_params {
  float4 *cells;  /* fast step table; .x = sig_a, updated by the Adam kernel */
  float2 *aux;    /* {w_c, unused} */
  const mcg_fit_slab_dev *slabs;
  const mcg_fit_item *items;
  int32_t n_items, max_cells;
  unsigned long long *item_next;
  unsigned long long *tally;
  double *grad;
  const long long *step;
  float min_w;
  int32_t q_log2, refill_steps, with_grad;
  uint32_t max_steps;
};

__device__ __forceinline__ void fit_ff_add(float &hi, float &lo, float v)
{
  const float s = __fadd_rn(hi, v);
  const float bv = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bv)), __fsub_rn(v, bv));
  hi = s;
  lo = __fadd_rn(lo, e);
}

__global__ void __launch_bounds__(512, 2) mcg_fit_kernel(mcg_fit_params P)
{
  extern __shared__ __align__(16) unsigned char smem[];
  long long *s_ctl = reinterpret_cast<long long *>(smem);
  unsigned long long *s_tally = reinterpret_cast<unsigned long long *>(s_ctl + 4);
  float *s_g = reinterpret_cast<float *>(s_tally + P.max_cells);
  const int tid = threadIdx.x, lane = tid & 31;
  const long long step = *P.step;
  int cur = -1, m = 0;
  const float4 *cells = nullptr;
  const float2 *aux = nullptr;
  unsigned long long *gtally = nullptr;
  double *ggrad = nullptr;
  mcg_libm_dev no_libm = {};
  for (;;) {
    __syncthreads();
    if (tid == 0)
      s_ctl[0] = (long long)atomicAdd(P.item_next, 1ull);
    __syncthreads();
    const long long item = s_ctl[0];
    if (item >= P.n_items)
      break;
    const mcg_fit_item it = P.items[item];
    if (it.slab != cur) {
      if (cur >= 0)
        for (int i = tid; i < m; i += blockDim.x) {
          if (s_tally[i])
            atomicAdd(&gtally[i], s_tally[i]);
          if (s_g[i] != 0.0f)
            atomicAdd(&ggrad[i], (double)s_g[i]);
        }
      __syncthreads();
      cur = it.slab;
      const mcg_fit_slab_dev sd = P.slabs[cur];
      m = sd.m;
      cells = P.cells + sd.cell_off;
      aux = P.aux + sd.cell_off;
      gtally = P.tally + sd.cell_off;
      ggrad = P.grad + sd.cell_off;
      for (int i = tid; i < m; i += blockDim.x) {
        s_tally[i] = 0ull;
        s_g[i] = 0.0f;
      }
    }
    if (tid == 0)
      s_ctl[1] = 0;
    __syncthreads();
    const mcg_fit_slab_dev sd = P.slabs[cur];
    const int64_t src_base = step * sd.n_hist + it.first;

    uint64_t seed = 0;
    float x = 0.f, mu = 0.f, wmc = 0.f, inv_mu = 0.f;
    int idx = 0, phase = 0;
    long long my_h = -1;
    uint32_t nst = 0, nsc = 0;
    float G_hi = 0.f, G_lo = 0.f, P_hi = 0.f, P_lo = 0.f;
    bool active = false;
    long long pool_next = 0, pool_end = 0;
    bool drained = false;
    for (;;) {
      unsigned need = __ballot_sync(0xffffffffu, !active);
      if (need) {
        int cnt = __popc(need), rank = __popc(need & lanemask_lt());
        long long avail = pool_end - pool_next, my = -1;
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
            if (rank >= avail && r2 < end - base)
              my = base + r2;
            pool_next = min(base + (cnt - avail), end);
            pool_end = end;
          }
        } else {
          pool_next += min((long long)cnt, avail);
        }
        if (!active && my >= 0) {
          my_h = my;
          mcg_source_particle(sd.src, src_base + my_h, seed, x, mu, wmc, idx);
          inv_mu = mcg_flight_rcp(mu);
          nst = nsc = 0;
          phase = 0;
          G_hi = G_lo = P_hi = P_lo = 0.f;
          active = true;
        }
      }
      if (!__any_sync(0xffffffffu, active))
        break;
      for (int k = 0; k < P.refill_steps; ++k) {
        if (!active)
          break;
        if (!((wmc >= P.min_w) && (idx < m) && (idx >= 0)) || nst >= P.max_steps) {
          if (phase == 0 && P.with_grad) {
            mcg_source_particle(sd.src, src_base + my_h, seed, x, mu, wmc, idx);
            inv_mu = mcg_flight_rcp(mu);
            nst = nsc = 0;
            phase = 1;
            continue;
          }
          active = false;
          break;
        }
        const int c = idx;
        const float wc = __ldg(&aux[c].x);
        float l, dep;
        bool coll;
        mcg_step<false, MCG_TALLY_SMEM32>(seed, x, mu, wmc, inv_mu, idx, nsc, cells[c],
                                          phase == 0 ? &s_tally[c] : nullptr, P.q_log2, nullptr,
                                          no_libm, &l, &coll, &dep);
        const float g = __fmul_rn(wc, dep);
        if (phase == 0) {
          fit_ff_add(G_hi, G_lo, g);
        } else {
          fit_ff_add(P_hi, P_lo, g);
          const float v_after = __fadd_rn(__fsub_rn(G_hi, P_hi), __fsub_rn(G_lo, P_lo));
          atomicAdd(&s_g[c], l * (wc * wmc - v_after));
        }
        ++nst;
      }
    }
  }
  if (cur >= 0)
    for (int i = tid; i < m; i += blockDim.x) {
      if (s_tally[i])
        atomicAdd(&gtally[i], s_tally[i]);
      if (s_g[i] != 0.0f)
        atomicAdd(&ggrad[i], (double)s_g[i]);
    }
}

/* w_c = 2 (a_c - t_c) from this step's tally, the step's loss, and the
 * accumulators cleared for the next step. */
__global__ void mcg_fit_weights_kernel(int n_cells, const int32_t *cell_slab,
                                       const mcg_fit_slab_dev *slabs, const double *target,
                                       unsigned long long *tally, float2 *aux, double *loss_hist,
                                       const long long *step, int q_log2, int max_steps)
{
  const double inv_scale = ldexp(1.0, -q_log2);
  double part = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n_cells; c += gridDim.x * blockDim.x) {
    const double a = (double)(long long)tally[c] * inv_scale / (double)slabs[cell_slab[c]].n_hist;
    const double d = a - target[c];
    aux[c].x = (float)(2.0 * d);
    part += d * d;
    tally[c] = 0ull;
  }
  for (int o = 16; o > 0; o >>= 1)
    part += __shfl_down_sync(0xffffffffu, part, o);
  const long long s = *step;
  if ((threadIdx.x & 31) == 0 && s < max_steps)
    atomicAdd(&loss_hist[s], part);
}

/* Adam on every sig_a; the new value goes straight into the step table. */
__global__ void mcg_fit_adam_kernel(int n_cells, const int32_t *cell_slab,
                                    const mcg_fit_slab_dev *slabs, double *grad, float *sig_a,
                                    float4 *cells, float *m1, float *m2, long long *step, float lr,
                                    float b1, float b2, float eps, float sig_min)
{
  const long long t = *step + 1;
  const float c1 = 1.0f - powf(b1, (float)t), c2 = 1.0f - powf(b2, (float)t);
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n_cells; c += gridDim.x * blockDim.x) {
    const float g = (float)(grad[c] / (double)slabs[cell_slab[c]].n_hist);
    grad[c] = 0.0;
    const float a = b1 * m1[c] + (1.0f - b1) * g;
    const float v = b2 * m2[c] + (1.0f - b2) * g * g;
    m1[c] = a;
    m2[c] = v;
    const float s = fmaxf(sig_a[c] - lr * (a / c1) / (sqrtf(v / c2) + eps), sig_min);
    sig_a[c] = s;
    cells[c].x = s;
  }
  __syncthreads();
  if (blockIdx.x == 0 && threadIdx.x == 0)
    *step = t;
}

/* ------------------------------------------------------------ host side */
struct mcg_fit_state {
  int n_slabs = 0, n_cells = 0, max_cells = 0, n_items = 0, max_steps = 0;
  std::vector<int32_t> cell_off;
  void *dev = nullptr; /* one allocation for everything below */
  float4 *cells = nullptr;
  float2 *aux = nullptr;
  mcg_fit_slab_dev *slabs = nullptr;
  mcg_fit_item *items = nullptr;
  int32_t *cell_slab = nullptr;
  double *target = nullptr, *grad = nullptr, *loss_hist = nullptr;
  float *sig_a = nullptr, *m1 = nullptr, *m2 = nullptr;
  unsigned long long *tally = nullptr, *item_next = nullptr;
  long long *step = nullptr;
  float min_w = 0.f;
};

static mcg_fit_state *fit_of(mcg_context *ctx, bool create)
{
  if (!ctx->ext) {
    if (!create)
      return nullptr;
    ctx->ext = new mcg_ext();
  }
  if (!ctx->ext->fit && create)
    ctx->ext->fit = new mcg_fit_state();
  return ctx->ext->fit;
}

extern "C" int mcg_fit_release(mcg_context *ctx)
{
  if (!ctx || !ctx->ext || !ctx->ext->fit)
    return MCG_OK;
  if (ctx->ext->fit->dev)
    cudaFree(ctx->ext->fit->dev);
  delete ctx->ext->fit;
  ctx->ext->fit = nullptr;
  return MCG_OK;
}

extern "C" int mcg_fit_set(mcg_context *ctx, int32_t n_slabs, const mcg_slab *h_slabs,
                           const float *h_sig_a0, const float *h_sig_s, const double *h_target,
                           float particle_min_weight, int32_t max_steps)
{
  if (!ctx || n_slabs <= 0 || !h_slabs || !h_sig_a0 || !h_sig_s || !h_target || max_steps <= 0)
    return mcg_fail(MCG_ERR_ARG, "mcg_fit_set: bad arguments");
  cudaSetDevice(ctx->device);
  mcg_fit_release(ctx);
  mcg_fit_state *F = fit_of(ctx, true);
  int total = 0, maxc = 0;
  for (int s = 0; s < n_slabs; ++s) {
    if (h_slabs[s].n_cells <= 0 || h_slabs[s].n_histories <= 0)
      return mcg_fail(MCG_ERR_ARG, "mcg_fit_set: bad slab %d", s);
    total += h_slabs[s].n_cells;
    maxc = std::max(maxc, h_slabs[s].n_cells);
  }
  if (16 * 4 + (size_t)maxc * 12 > (size_t)ctx->smem_optin)
    return mcg_fail(MCG_ERR_ARG, "mcg_fit_set: slab of %d cells too large", maxc);
  /* items of up to 8192 histories, largest first */
  std::vector<mcg_fit_item> items;
  for (int s = 0; s < n_slabs; ++s)
    for (int64_t f = 0; f < h_slabs[s].n_histories; f += 8192)
      items.push_back({s, 0, f, std::min<int64_t>(8192, h_slabs[s].n_histories - f)});
  std::stable_sort(items.begin(), items.end(), [&](const mcg_fit_item &a, const mcg_fit_item &b) {
    return a.count * h_slabs[a.slab].n_cells > b.count * h_slabs[b.slab].n_cells;
  });
  /* carve one allocation */
  size_t off = 0;
  auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~(size_t)255; return o; };
  const size_t o_cells = take(total * sizeof(float4)), o_aux = take(total * sizeof(float2));
  const size_t o_slabs = take(n_slabs * sizeof(mcg_fit_slab_dev));
  const size_t o_items = take(items.size() * sizeof(mcg_fit_item));
  const size_t o_cs = take(total * 4), o_t = take(total * 8), o_g = take(total * 8);
  const size_t o_lh = take(max_steps * 8), o_sa = take(total * 4), o_m1 = take(total * 4);
  const size_t o_m2 = take(total * 4), o_ta = take(total * 8), o_in = take(8), o_st = take(8);
  cudaError_t e = cudaMalloc(&F->dev, off);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_fit_set: cudaMalloc");
  char *b = static_cast<char *>(F->dev);
  F->cells = reinterpret_cast<float4 *>(b + o_cells);
  F->aux = reinterpret_cast<float2 *>(b + o_aux);
  F->slabs = reinterpret_cast<mcg_fit_slab_dev *>(b + o_slabs);
  F->items = reinterpret_cast<mcg_fit_item *>(b + o_items);
  F->cell_slab = reinterpret_cast<int32_t *>(b + o_cs);
  F->target = reinterpret_cast<double *>(b + o_t);
  F->grad = reinterpret_cast<double *>(b + o_g);
  F->loss_hist = reinterpret_cast<double *>(b + o_lh);
  F->sig_a = reinterpret_cast<float *>(b + o_sa);
  F->m1 = reinterpret_cast<float *>(b + o_m1);
  F->m2 = reinterpret_cast<float *>(b + o_m2);
  F->tally = reinterpret_cast<unsigned long long *>(b + o_ta);
  F->item_next = reinterpret_cast<unsigned long long *>(b + o_in);
  F->step = reinterpret_cast<long long *>(b + o_st);
  cudaMemset(F->dev, 0, off);
  std::vector<float4> cf(total);
  std::vector<float2> ax(total, make_float2(0.f, 0.f));
  std::vector<mcg_fit_slab_dev> sd(n_slabs);
  std::vector<int32_t> cs(total);
  int k = 0;
  for (int s = 0; s < n_slabs; ++s) {
    const mcg_slab &sl = h_slabs[s];
    const float dx = 1.0f / (float)sl.n_cells;
    sd[s].cell_off = k;
    sd[s].m = sl.n_cells;
    sd[s].n_hist = sl.n_histories;
    sd[s].src = {sl.seed_mode, sl.isotropic, sl.base_seed, 0.0f, sl.mu0, sl.w0, 0};
    for (int j = 0; j < sl.n_cells; ++j, ++k) {
      const float sig_s = h_sig_s[k];
      cf[k] = make_float4(h_sig_a0[k], sig_s > 1e-4f ? sig_s : 0.0f,
                          (float)j * dx, (float)(j + 1) * dx);
      cs[k] = s;
    }
  }
  if ((e = cudaMemcpy(F->cells, cf.data(), total * sizeof(float4), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(F->aux, ax.data(), total * sizeof(float2), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(F->slabs, sd.data(), n_slabs * sizeof(mcg_fit_slab_dev), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(F->items, items.data(), items.size() * sizeof(mcg_fit_item), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(F->cell_slab, cs.data(), total * 4, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(F->target, h_target, total * 8, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(F->sig_a, h_sig_a0, total * 4, cudaMemcpyHostToDevice)) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_fit_set: upload");
  F->n_slabs = n_slabs;
  F->n_cells = total;
  F->max_cells = maxc;
  F->n_items = (int)items.size();
  F->max_steps = max_steps;
  F->min_w = particle_min_weight;
  return MCG_OK;
}

static int fit_launch_track(mcg_context *ctx, mcg_fit_state *F, int with_grad)
{
  mcg_fit_params P;
  memset(&P, 0, sizeof(P));
  P.cells = F->cells;
  P.aux = F->aux;
  P.slabs = F->slabs;
  P.items = F->items;
  P.n_items = F->n_items;
  P.max_cells = F->max_cells;
  P.item_next = F->item_next;
  P.tally = F->tally;
  P.grad = F->grad;
  P.step = F->step;
  P.min_w = F->min_w;
  P.q_log2 = ctx->log2_scale;
  P.refill_steps = ctx->refill;
  P.with_grad = with_grad;
  P.max_steps = ctx->max_steps;
  const size_t smem = 4 * 8 + (size_t)F->max_cells * 12;
  cudaError_t e = cudaFuncSetAttribute(mcg_fit_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  int bps = 1;
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, mcg_fit_kernel, 512, smem);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_fit: launch set-up");
  if ((e = cudaMemsetAsync(F->item_next, 0, 8, ctx->stream)) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_fit: memset");
  mcg_fit_kernel<<<ctx->sm_count * std::max(bps, 1), 512, smem, ctx->stream>>>(P);
  if ((e = cudaGetLastError()) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_fit_kernel launch");
  ctx->launches++;
  return MCG_OK;
}

/* n_steps Adam steps (lr, beta1, beta2, eps; sig_a kept >= sig_min). */
extern "C" int mcg_fit_run(mcg_context *ctx, int32_t n_steps, float lr, float beta1, float beta2,
                           float eps, float sig_min)
{
  mcg_fit_state *F = ctx ? fit_of(ctx, false) : nullptr;
  if (!F || n_steps < 0)
    return mcg_fail(MCG_ERR_STATE, "mcg_fit_run: mcg_fit_set first");
  cudaSetDevice(ctx->device);
  long long step0 = 0;
  cudaMemcpy(&step0, F->step, 8, cudaMemcpyDeviceToHost);
  if (step0 + n_steps > F->max_steps)
    return mcg_fail(MCG_ERR_ARG, "mcg_fit_run: at most %d steps in total", F->max_steps);
  const int nb = std::min((F->n_cells + 255) / 256, ctx->sm_count * 4);
  int rc = MCG_OK;
  cudaError_t e;
  if (step0 == 0) {
    /* weights for the first step: a forward pass at the starting point */
    if ((rc = fit_launch_track(ctx, F, 0)) != MCG_OK)
      return rc;
    mcg_fit_weights_kernel<<<nb, 256, 0, ctx->stream>>>(F->n_cells, F->cell_slab, F->slabs, F->target,
                                                        F->tally, F->aux, F->loss_hist, F->step,
                                                        ctx->log2_scale, 0);
    cudaMemsetAsync(F->grad, 0, F->n_cells * 8, ctx->stream);
  }
  /* one step = fused forward+adjoint, weights + loss, Adam: a CUDA graph */
  cudaGraph_t g;
  cudaGraphExec_t ge = nullptr;
  if ((e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_fit_run: capture");
  rc = fit_launch_track(ctx, F, 1);
  mcg_fit_weights_kernel<<<nb, 256, 0, ctx->stream>>>(F->n_cells, F->cell_slab, F->slabs, F->target,
                                                      F->tally, F->aux, F->loss_hist, F->step,
                                                      ctx->log2_scale, F->max_steps);
  mcg_fit_adam_kernel<<<1, 1024, 0, ctx->stream>>>(F->n_cells, F->cell_slab, F->slabs, F->grad,
                                                   F->sig_a, F->cells, F->m1, F->m2, F->step, lr,
                                                   beta1, beta2, eps, sig_min);
  e = cudaStreamEndCapture(ctx->stream, &g);
  if (rc != MCG_OK)
    return rc;
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_fit_run: end capture");
  e = cudaGraphInstantiate(&ge, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_fit_run: instantiate");
  cudaEventRecord(ctx->ev0, ctx->stream);
  for (int s = 0; s < n_steps && e == cudaSuccess; ++s)
    e = cudaGraphLaunch(ge, ctx->stream);
  cudaEventRecord(ctx->ev1, ctx->stream);
  cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
  cudaGraphExecDestroy(ge);
  if (e != cudaSuccess || e2 != cudaSuccess)
    return mcg_cuda_fail(e != cudaSuccess ? e : e2, "mcg_fit_run");
  cudaEventElapsedTime(&ctx->last_ms, ctx->ev0, ctx->ev1);
  ctx->launches += 3LL * n_steps;
  return MCG_OK;
}

/* Current sig_a (all cells, slab order), the per-step loss history and the
 * number of steps done. */
extern "C" int mcg_fit_read(mcg_context *ctx, float *h_sig_a, double *h_loss_hist, int32_t *h_steps)
{
  mcg_fit_state *F = ctx ? fit_of(ctx, false) : nullptr;
  if (!F)
    return mcg_fail(MCG_ERR_STATE, "mcg_fit_read: mcg_fit_set first");
  cudaSetDevice(ctx->device);
  long long st = 0;
  cudaError_t e = cudaMemcpy(&st, F->step, 8, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && h_sig_a)
    e = cudaMemcpy(h_sig_a, F->sig_a, F->n_cells * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && h_loss_hist)
    e = cudaMemcpy(h_loss_hist, F->loss_hist, F->max_steps * 8, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_fit_read");
  if (h_steps)
    *h_steps = (int32_t)st;
  return MCG_OK;
}

/* One batched forward + adjoint launch of the fit kernel at the current
 * sig_a with the given loss weights (testing aid): histories step * n + i of
 * every slab, as the next Adam step would run, with w_c = h_weights[c]
 * instead of 2 (a_c - t_c).  Returns per cell the weight absorbed per history
 * (h_tally) and dF/dsig_a per history (h_grad), F = sum_c w_c a_c, so the
 * fit's gradient can be compared with mcg_adjoint's on the same histories.
 * The fit's own loss weights and accumulators are left as they were. */
extern "C" int mcg_fit_gradient(mcg_context *ctx, const double *h_weights, double *h_tally,
                                double *h_grad)
{
  mcg_fit_state *F = ctx ? fit_of(ctx, false) : nullptr;
  if (!F)
    return mcg_fail(MCG_ERR_STATE, "mcg_fit_gradient: mcg_fit_set first");
  if (!h_weights || !h_tally || !h_grad)
    return mcg_fail(MCG_ERR_ARG, "mcg_fit_gradient: bad arguments");
  cudaSetDevice(ctx->device);
  const int n = F->n_cells;
  std::vector<float2> saved(n), ax(n);
  std::vector<double> keep_grad(n);
  std::vector<unsigned long long> keep_tally(n), q(n);
  std::vector<mcg_fit_slab_dev> sd(F->n_slabs);
  std::vector<int32_t> cs(n);
  for (int c = 0; c < n; ++c)
    ax[c] = make_float2((float)h_weights[c], 0.0f);
  cudaError_t e;
  if ((e = cudaMemcpy(saved.data(), F->aux, n * sizeof(float2), cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(keep_grad.data(), F->grad, n * 8, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(keep_tally.data(), F->tally, n * 8, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(sd.data(), F->slabs, F->n_slabs * sizeof(mcg_fit_slab_dev), cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(cs.data(), F->cell_slab, n * 4, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(F->aux, ax.data(), n * sizeof(float2), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemset(F->grad, 0, n * 8)) != cudaSuccess ||
      (e = cudaMemset(F->tally, 0, n * 8)) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_fit_gradient: set-up");
  int rc = fit_launch_track(ctx, F, 1);
  if (rc != MCG_OK)
    return rc;
  if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess ||
      (e = cudaMemcpy(q.data(), F->tally, n * 8, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(h_grad, F->grad, n * 8, cudaMemcpyDeviceToHost)) != cudaSuccess ||
      (e = cudaMemcpy(F->aux, saved.data(), n * sizeof(float2), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(F->grad, keep_grad.data(), n * 8, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(F->tally, keep_tally.data(), n * 8, cudaMemcpyHostToDevice)) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_fit_gradient");
  const double inv_scale = std::ldexp(1.0, -ctx->log2_scale);
  for (int c = 0; c < n; ++c) {
    const double nh = (double)sd[cs[c]].n_hist;
    h_tally[c] = (double)(long long)q[c] * inv_scale / nh;
    h_grad[c] /= nh;
  }
  return MCG_OK;
}
