/*
 * mcg_adjoint.cu - forward tally plus adjoint gradients of a tally loss.
 *
 * Loss: F = sum_c w_c a_c, a_c = expected weight absorbed in chain cell c
 * per history.  Parameters: sig_a[c] = sigs*rates and sig_s[c] =
 * sigs*(1 - rates) of every chain cell (the two cross sections of
 * Layer::particle_step, src/layer.cpp:129-131).
 *
 * For one history with steps k (cell c_k, flight length l_k, weight W_k after
 * the step, deposit g_k = w_{c_k} (W_{k-1} - W_k)), G = sum_k g_k and
 * P_k = g_1 + ... + g_k:
 *  - sig_a enters only the weight attenuation exp(-sig_a l), never the flight
 *    sampling, so its derivative is pathwise:
 *        dG/dsig_a[c] = sum_{k: c_k = c} l_k (w_c W_k - (G - P_k));
 *    this is a deliberate deviation from a score-function (likelihood-ratio)
 *    estimator for sig_a: with implicit capture no sampled event depends on
 *    sig_a, so its score is zero and the pathwise derivative is the whole
 *    gradient (same expectation, far lower variance);
 *  - sig_s sets the flight distribution (exponential with rate sig_s): the
 *    log-density score of step k is 1/sig_s - l_k for a collision and -l_k
 *    for a crossing (no collision before the face), and it weights the loss
 *    deposited from step k on (earlier deposits do not depend on it):
 *        dG/dsig_s[c] = sum_{k: c_k = c} score_k (G - P_{k-1}).
 * Each lane runs a history forward (accumulating G and the tally), then
 * replays it from the same source index and seed (the path is never stored)
 * accumulating the two gradients.  G and P are float-float sums, so G - P
 * keeps its accuracy at the end of long histories.  The tally and the loss
 * are 64-bit fixed point (exact, order-independent); the gradients, which are
 * statistical estimates, are accumulated with fp32 shared-memory atomics
 * (one instruction per deposit) and flushed to fp64 once per block.
 */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

/* A warp whose lanes need both exp paths takes the general one for all: it
 * returns the small-argument path's bits wherever that applies.  Measured on
 * the adjoint kernels: about 0.5-1 % faster; on the single-chain tracker, whose
 * crossings almost all take the small path, 3 % slower, so it keeps the
 * per-lane choice. */
#define MCG_EXP_UNIFORM
#include "mcg_internal.h"
#include "mcg_track.cuh"

struct mcg_adj_params {
  const float4 *cells;
  const float2 *aux; /* {w_c, 1/sig_s or 0} */
  int32_t n_cells, cell_lo;
  float min_w;
  int32_t q_log2, g_log2;
  mcg_source src;
  int64_t first, n;
  unsigned long long *next;
  unsigned long long *tally, *loss, *counters;
  double *grad_a, *grad_s;
  mcg_libm_dev libm;
  const mcg_libm_tab *libm_tab;
  int32_t refill_steps, chunk, with_grad;
  uint32_t max_steps;
};

/* float-float accumulation s += v (TwoSum) */
__device__ __forceinline__ void ff_add(float &hi, float &lo, float v)
{
  const float s = __fadd_rn(hi, v);
  const float bv = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bv)), __fsub_rn(v, bv));
  hi = s;
  lo = __fadd_rn(lo, e);
}

template <bool STRICT>
__global__ void __launch_bounds__(1024) mcg_adjoint_kernel(mcg_adj_params P)
{
  extern __shared__ __align__(16) unsigned char smem[];
  mcg_libm_tab *T = reinterpret_cast<mcg_libm_tab *>(smem);
  unsigned long long *s_cnt = reinterpret_cast<unsigned long long *>(smem + sizeof(mcg_libm_tab));
  unsigned long long *s_tally = s_cnt + 16;
  float *s_ga = reinterpret_cast<float *>(s_tally + P.n_cells);
  float *s_gs = s_ga + P.n_cells;
  const int tid = threadIdx.x, lane = tid & 31;
  const int ncell = P.n_cells, lo = P.cell_lo;
  if (STRICT) {
    const float *src = reinterpret_cast<const float *>(P.libm_tab);
    float *dst = reinterpret_cast<float *>(T);
    for (int i = tid; i < (int)(sizeof(mcg_libm_tab) / 4); i += blockDim.x)
      dst[i] = src[i];
  }
  if (tid < 16)
    s_cnt[tid] = 0ull;
  for (int i = tid; i < 2 * ncell; i += blockDim.x)
    s_tally[i] = 0ull; /* the tally and both float gradient arrays */
  __syncthreads();
  const float min_w = P.min_w;
  const int qs = P.q_log2, gs = P.g_log2;

  uint64_t seed = 0;
  float x = 0.f, mu = 0.f, wmc = 0.f, inv_mu = 0.f;
  int idx = 0, phase = 0;
  int64_t hid = -1;
  uint32_t nst = 0, nsc = 0;
  float G_hi = 0.f, G_lo = 0.f, P_hi = 0.f, P_lo = 0.f;
  bool active = false;
  unsigned long long tot_steps = 0, tot_scat = 0;
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
        unsigned long long base = 0;
        if (lane == 0)
          base = atomicAdd(P.next, (unsigned long long)P.chunk);
        base = __shfl_sync(0xffffffffu, base, 0);
        if ((long long)base >= P.n) {
          drained = true;
          pool_next = pool_end = 0;
        } else {
          long long end = min((long long)base + P.chunk, (long long)P.n);
          long long r2 = rank - avail;
          if (rank >= avail && r2 < end - (long long)base)
            my = (long long)base + r2;
          pool_next = min((long long)base + (cnt - avail), end);
          pool_end = end;
        }
      } else {
        pool_next += min((long long)cnt, avail);
      }
      if (!active && my >= 0) {
        hid = my;
        mcg_source_particle(P.src, P.first + hid, seed, x, mu, wmc, idx);
        idx -= lo;
        inv_mu = mcg_flight_rcp(mu);
        nst = nsc = 0;
        phase = 0;
        G_hi = G_lo = P_hi = P_lo = 0.f;
        active = true;
      }
    }
    if (!__any_sync(0xffffffffu, active))
      break;

    if (active) {
      /* up to refill_steps steps, never past the step limit; idx is local
       * to the chain */
      const int kmax = (int)min((uint32_t)P.refill_steps, P.max_steps - nst);
      int k = 0;
      bool going = true;
      for (; k < kmax; ++k) {
        if (!((wmc >= min_w) & ((unsigned)idx < (unsigned)ncell))) {
          going = false;
          break;
        }
        const int c = idx;
        const float2 ax = __ldg(P.aux + c);
        float l, dep;
        bool coll;
        mcg_step<STRICT, MCG_TALLY_SMEM32>(seed, x, mu, wmc, inv_mu, idx, nsc, __ldg(P.cells + c),
                                           phase == 0 ? &s_tally[c] : nullptr, qs, T, P.libm, &l,
                                           &coll, &dep);
        const float g = __fmul_rn(ax.x, dep);
        if (phase == 0) {
          ff_add(G_hi, G_lo, g);
        } else {
          /* suffix before this step, then after it */
          const float v_before = __fadd_rn(__fsub_rn(G_hi, P_hi), __fsub_rn(G_lo, P_lo));
          ff_add(P_hi, P_lo, g);
          const float v_after = __fadd_rn(__fsub_rn(G_hi, P_hi), __fsub_rn(G_lo, P_lo));
          const float ga = l * (ax.x * wmc - v_after);
          const float score = (coll ? ax.y : 0.0f) - l;
          const float gsc = score * v_before;
          atomicAdd(&s_ga[c], ga);
          atomicAdd(&s_gs[c], gsc);
        }
      }
      nst += (uint32_t)k;
      if (!going || nst >= P.max_steps) {
        if ((wmc >= min_w) && ((unsigned)idx < (unsigned)ncell))
          atomicOr(&s_cnt[MCG_CNT_ERR], 1ull); /* the step limit */
        if (phase == 0) {
          tot_steps += nst;
          tot_scat += nsc;
        }
        if (phase == 0 && P.with_grad) {
          /* replay the same history from its start */
          mcg_source_particle(P.src, P.first + hid, seed, x, mu, wmc, idx);
          idx -= lo;
          inv_mu = mcg_flight_rcp(mu);
          nst = nsc = 0;
          phase = 1;
        } else {
          atomicAdd(&s_cnt[MCG_CNT_HIST], 1ull);
          mcg_tally_add<MCG_TALLY_SMEM32>(&s_cnt[MCG_CNT_WLEFT],
                                           mcg_to_fixed(G_hi, gs) + mcg_to_fixed(G_lo, gs));
          active = false;
        }
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    tot_steps += __shfl_down_sync(0xffffffffu, tot_steps, o);
    tot_scat += __shfl_down_sync(0xffffffffu, tot_scat, o);
  }
  if (lane == 0) {
    atomicAdd(&s_cnt[MCG_CNT_STEPS], tot_steps);
    atomicAdd(&s_cnt[MCG_CNT_SCAT], tot_scat);
  }
  __syncthreads();
  for (int i = tid; i < ncell; i += blockDim.x) {
    if (s_tally[i])
      atomicAdd(&P.tally[i], s_tally[i]);
    if (s_ga[i] != 0.0f)
      atomicAdd(&P.grad_a[i], (double)s_ga[i]);
    if (s_gs[i] != 0.0f)
      atomicAdd(&P.grad_s[i], (double)s_gs[i]);
  }
  if (tid == 0) {
    atomicAdd(P.loss, s_cnt[MCG_CNT_WLEFT]);
    atomicAdd(&P.counters[MCG_CNT_HIST], s_cnt[MCG_CNT_HIST]);
    atomicAdd(&P.counters[MCG_CNT_STEPS], s_cnt[MCG_CNT_STEPS]);
    atomicAdd(&P.counters[MCG_CNT_SCAT], s_cnt[MCG_CNT_SCAT]);
    if (s_cnt[MCG_CNT_ERR])
      atomicOr(&P.counters[MCG_CNT_ERR], s_cnt[MCG_CNT_ERR]);
  }
}

/* ------------------------------------------------------------ host side */
static mcg_adj_state *adj_of(mcg_context *ctx)
{
  if (!ctx->ext)
    ctx->ext = new mcg_ext();
  return &ctx->ext->adj;
}

void mcg_adjoint_release(mcg_adj_state *A)
{
  if (A->d_aux)
    cudaFree(A->d_aux);
  if (A->d_grad)
    cudaFree(A->d_grad);
  *A = mcg_adj_state();
}

extern "C" int mcg_adjoint_set_weights(mcg_context *ctx, const float *h_w)
{
  if (!ctx || !h_w || !ctx->d_tally)
    return mcg_fail(MCG_ERR_ARG, "mcg_adjoint_set_weights: bad arguments or no layers");
  cudaSetDevice(ctx->device);
  mcg_adj_state *A = adj_of(ctx);
  const int n = ctx->n_cells;
  if (A->n != n) {
    if (A->d_aux)
      cudaFree(A->d_aux);
    if (A->d_grad)
      cudaFree(A->d_grad);
    A->d_aux = nullptr;
    A->d_grad = nullptr;
    cudaError_t e;
    if ((e = cudaMalloc(&A->d_aux, n * sizeof(float2))) != cudaSuccess ||
        (e = cudaMalloc(&A->d_grad, (2 * (size_t)n + 1) * sizeof(unsigned long long))) != cudaSuccess)
      return mcg_cuda_fail(e, "mcg_adjoint_set_weights: cudaMalloc");
    A->n = n;
  }
  std::vector<float2> aux(n);
  for (int c = 0; c < n; ++c) {
    const float sig_i = ctx->cells_strict[c].y; /* the flight cross section of the step */
    aux[c] = make_float2(h_w[c], sig_i > 1e-4f ? 1.0f / sig_i : 0.0f);
  }
  cudaError_t e = cudaMemcpy(A->d_aux, aux.data(), n * sizeof(float2), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemset(A->d_grad, 0, (2 * (size_t)n + 1) * sizeof(unsigned long long));
  A->histories = 0;
  return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(e, "mcg_adjoint_set_weights");
}

extern "C" int mcg_adjoint_reset(mcg_context *ctx)
{
  if (!ctx)
    return mcg_fail(MCG_ERR_ARG, "mcg_adjoint_reset: null context");
  mcg_adj_state *A = adj_of(ctx);
  if (!A->d_grad)
    return mcg_fail(MCG_ERR_STATE, "mcg_adjoint_reset: no loss weights set");
  cudaSetDevice(ctx->device);
  cudaError_t e = cudaMemset(A->d_grad, 0, (2 * (size_t)A->n + 1) * sizeof(unsigned long long));
  A->histories = 0;
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_adjoint_reset");
  return mcg_tally_reset(ctx);
}

extern "C" int mcg_adjoint_run(mcg_context *ctx, const mcg_source *src, int64_t first, int64_t n,
                               int32_t with_gradient)
{
  if (!ctx || !src || n < 0 || first < 0)
    return mcg_fail(MCG_ERR_ARG, "mcg_adjoint_run: bad arguments");
  mcg_adj_state *A = adj_of(ctx);
  if (!A->d_aux || A->n != ctx->n_cells)
    return mcg_fail(MCG_ERR_STATE, "mcg_adjoint_run: set the loss weights first");
  cudaSetDevice(ctx->device);
  const bool strict = ctx->mode == MCG_MODE_STRICT;
  if (strict && !ctx->libm_loaded) {
    int rc = mcg_load_libm(ctx);
    if (rc != MCG_OK)
      return rc;
  }
  if (n == 0)
    return MCG_OK;
  mcg_adj_params P;
  memset(&P, 0, sizeof(P));
  P.cells = strict ? ctx->d_cells_strict : ctx->d_cells_fast;
  P.aux = A->d_aux;
  P.n_cells = ctx->n_cells;
  P.cell_lo = ctx->cell_lo;
  P.min_w = ctx->min_w;
  P.q_log2 = ctx->log2_scale;
  P.g_log2 = A->g_log2;
  P.src = *src;
  P.first = first;
  P.n = n;
  P.next = ctx->d_next;
  P.tally = ctx->d_tally;
  P.grad_a = reinterpret_cast<double *>(A->d_grad);
  P.grad_s = reinterpret_cast<double *>(A->d_grad) + A->n;
  P.loss = A->d_grad + 2 * A->n;
  P.counters = ctx->d_counters;
  P.libm = ctx->libm;
  P.libm_tab = ctx->libm_tab;
  P.refill_steps = ctx->refill;
  P.chunk = 64;
  P.with_grad = with_gradient ? 1 : 0;
  P.max_steps = ctx->max_steps;
  const int block = ctx->block ? ctx->block : 512;
  const size_t smem = sizeof(mcg_libm_tab) + 16 * 8 + 2 * (size_t)ctx->n_cells * 8;
  if (smem > (size_t)ctx->smem_optin)
    return mcg_fail(MCG_ERR_ARG, "mcg_adjoint_run: chain of %d cells too long (max %d)",
                    ctx->n_cells, (int)((ctx->smem_optin - 2048 - 128) / 16));
  auto kern = strict ? mcg_adjoint_kernel<true> : mcg_adjoint_kernel<false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int bps = 1;
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, block, smem);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_adjoint_run: launch set-up");
  long long want = (n + block - 1) / block;
  const int grid = (int)std::min<long long>((long long)ctx->sm_count * std::max(bps, 1), want);
  if ((e = cudaMemsetAsync(ctx->d_next, 0, 8, ctx->stream)) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_adjoint_run: memset");
  cudaEventRecord(ctx->ev0, ctx->stream);
  kern<<<grid, block, smem, ctx->stream>>>(P);
  e = cudaGetLastError();
  cudaEventRecord(ctx->ev1, ctx->stream);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_adjoint_kernel launch");
  ctx->launches++;
  A->histories += n;
  return mcg_sync(ctx);
}

extern "C" int mcg_adjoint_read(mcg_context *ctx, double *h_loss, double *h_grad_a, double *h_grad_s)
{
  if (!ctx)
    return mcg_fail(MCG_ERR_ARG, "mcg_adjoint_read: null context");
  mcg_adj_state *A = adj_of(ctx);
  if (!A->d_grad || A->histories == 0)
    return mcg_fail(MCG_ERR_STATE, "mcg_adjoint_read: nothing run");
  cudaSetDevice(ctx->device);
  std::vector<int64_t> q(2 * (size_t)A->n + 1);
  cudaError_t e = cudaMemcpy(q.data(), A->d_grad, q.size() * sizeof(int64_t), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_adjoint_read");
  const double inv = 1.0 / (double)A->histories;
  if (h_loss)
    *h_loss = (double)q[2 * A->n] * std::ldexp(1.0, -A->g_log2) * inv;
  for (int c = 0; c < A->n; ++c) {
    double ga, gs;
    memcpy(&ga, &q[c], 8);
    memcpy(&gs, &q[A->n + c], 8);
    if (h_grad_a)
      h_grad_a[c] = ga * inv;
    if (h_grad_s)
      h_grad_s[c] = gs * inv;
  }
  return MCG_OK;
}
