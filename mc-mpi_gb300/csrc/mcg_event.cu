/*
 * mcg_event.cu - event-based variant of the tracker.
 *
 * Live particles sit in structure-of-arrays buffers (seed u64; x, mu, wmc
 * f32; cell, history, step and scatter counts i32), double-buffered.  One
 * pass advances every live particle by up to K events (K = 1: one
 * particle_step per pass, the classic event-based form; larger K trades
 * memory traffic for divergence).  A thread handles four consecutive
 * particles and reads each field with one 128-bit load; particles still
 * alive after the pass are compacted into the other buffer (warp ballot +
 * popc gives every survivor its slot, one atomic per warp reserves the
 * warp's range), finished ones write their result and final state by
 * history index.  Deposits go straight to the global 64-bit fixed-point tally
 * (a pass touches cells all over the chain, so a per-block copy would cost
 * more to clear and flush than it saves).  The step is mcg_step
 * (Layer::particle_step, src/layer.cpp:123-190), so results are identical to
 * the history-based tracker's, particle by particle.
 *
 * Memory per particle and event (K = 1): 36 B read + 36 B written.
 */
#include <algorithm>
#include <cstring>

#include "mcg_internal.h"
#include "mcg_track.cuh"

struct mcg_event_params {
  const float4 *cells;
  int32_t n_cells, cell_lo;
  float min_w;
  int32_t q_log2;
  mcg_soa in, out;
  const unsigned *n_in;
  unsigned *n_out;
  unsigned long long *tally, *counters;
  mcg_particle *particles; /* AoS outputs by history (NULL: source mode) */
  int32_t *results;
  int64_t *steps, *scatters;
  int32_t steps_per_pass;
  uint32_t max_steps;
  mcg_libm_dev libm;
  const mcg_libm_tab *libm_tab;
};

/* Fill the first SoA buffer from AoS particles or from the source. */
__global__ void mcg_event_init_kernel(mcg_track_params src_params, mcg_soa out, unsigned *n_out)
{
  const int64_t n = src_params.n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t seed;
    float x, mu, wmc;
    int idx;
    mcg_load_particle(src_params, i, seed, x, mu, wmc, idx);
    out.seed[i] = seed;
    out.x[i] = x;
    out.mu[i] = mu;
    out.wmc[i] = wmc;
    out.idx[i] = idx;
    out.hid[i] = (int32_t)i;
    out.nst[i] = 0;
    out.nsc[i] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0)
    *n_out = (unsigned)n;
}

template <bool STRICT>
__global__ void __launch_bounds__(256) mcg_event_pass_kernel(mcg_event_params P)
{
  __shared__ mcg_libm_tab T;
  __shared__ unsigned long long s_cnt[16];
  const int tid = threadIdx.x, lane = tid & 31;
  if (STRICT)
    for (int i = tid; i < (int)(sizeof(mcg_libm_tab) / 4); i += blockDim.x)
      reinterpret_cast<float *>(&T)[i] = reinterpret_cast<const float *>(P.libm_tab)[i];
  if (tid < 16)
    s_cnt[tid] = 0ull;
  __syncthreads();
  const unsigned n = *P.n_in;
  const int lo = P.cell_lo, hi = P.cell_lo + P.n_cells;
  const float min_w = P.min_w;
  const int qs = P.q_log2;
  unsigned long long tot_steps = 0, tot_scat = 0;
  const unsigned n4 = (n + 3) / 4;
  /* a whole warp iterates together so the ballots below see every lane */
  for (unsigned base = blockIdx.x * blockDim.x; base < n4; base += gridDim.x * blockDim.x) {
    const unsigned q = base + tid; /* quad index */
    const unsigned i0 = 4 * q;
    uint64_t seed[4];
    float x[4], mu[4], wmc[4];
    int idx[4], hid[4], nst[4], nsc[4];
    bool live[4];
    if (i0 + 3 < n) {
      const ulonglong2 s01 = reinterpret_cast<const ulonglong2 *>(P.in.seed)[2 * q];
      const ulonglong2 s23 = reinterpret_cast<const ulonglong2 *>(P.in.seed)[2 * q + 1];
      const float4 vx = reinterpret_cast<const float4 *>(P.in.x)[q];
      const float4 vm = reinterpret_cast<const float4 *>(P.in.mu)[q];
      const float4 vw = reinterpret_cast<const float4 *>(P.in.wmc)[q];
      const int4 vi = reinterpret_cast<const int4 *>(P.in.idx)[q];
      const int4 vh = reinterpret_cast<const int4 *>(P.in.hid)[q];
      const int4 vs = reinterpret_cast<const int4 *>(P.in.nst)[q];
      const int4 vc = reinterpret_cast<const int4 *>(P.in.nsc)[q];
      seed[0] = s01.x, seed[1] = s01.y, seed[2] = s23.x, seed[3] = s23.y;
      x[0] = vx.x, x[1] = vx.y, x[2] = vx.z, x[3] = vx.w;
      mu[0] = vm.x, mu[1] = vm.y, mu[2] = vm.z, mu[3] = vm.w;
      wmc[0] = vw.x, wmc[1] = vw.y, wmc[2] = vw.z, wmc[3] = vw.w;
      idx[0] = vi.x, idx[1] = vi.y, idx[2] = vi.z, idx[3] = vi.w;
      hid[0] = vh.x, hid[1] = vh.y, hid[2] = vh.z, hid[3] = vh.w;
      nst[0] = vs.x, nst[1] = vs.y, nst[2] = vs.z, nst[3] = vs.w;
      nsc[0] = vc.x, nsc[1] = vc.y, nsc[2] = vc.z, nsc[3] = vc.w;
#pragma unroll
      for (int j = 0; j < 4; ++j)
        live[j] = true;
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const unsigned i = i0 + j;
        live[j] = i < n;
        if (live[j]) {
          seed[j] = P.in.seed[i];
          x[j] = P.in.x[i];
          mu[j] = P.in.mu[i];
          wmc[j] = P.in.wmc[i];
          idx[j] = P.in.idx[i];
          hid[j] = P.in.hid[i];
          nst[j] = P.in.nst[i];
          nsc[j] = P.in.nsc[i];
        }
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (!live[j])
        continue;
      float inv_mu = mcg_flight_rcp(mu[j]);
      uint32_t sc = (uint32_t)nsc[j];
      const int st0 = nst[j];
      for (int k = 0; k < P.steps_per_pass; ++k) {
        if (!((wmc[j] >= min_w) && (idx[j] < hi) && (idx[j] >= lo)) ||
            (uint32_t)nst[j] >= P.max_steps) {
          live[j] = false;
          break;
        }
        mcg_step<STRICT, MCG_TALLY_GLOBAL>(seed[j], x[j], mu[j], wmc[j], inv_mu, idx[j], sc,
                                           __ldg(P.cells + (idx[j] - lo)), &P.tally[idx[j] - lo],
                                           qs, &T, P.libm);
        ++nst[j];
      }
      tot_steps += (unsigned long long)(nst[j] - st0);
      tot_scat += sc - (uint32_t)nsc[j];
      nsc[j] = (int)sc;
      if (live[j] && !((wmc[j] >= min_w) && (idx[j] < hi) && (idx[j] >= lo)))
        live[j] = false; /* ended on the pass's last event */
      if (!live[j]) {
        const bool limit = (uint32_t)nst[j] >= P.max_steps && (wmc[j] >= min_w) &&
                           (idx[j] < hi) && (idx[j] >= lo);
        int r = limit ? 2 : idx[j] == lo - 1 ? -1 : idx[j] == hi ? 1 : wmc[j] < min_w ? 0 : -1;
        const int h = hid[j];
        if (P.particles) {
          mcg_particle o;
          o.seed = seed[j];
          o.x = x[j];
          o.mu = mu[j];
          o.wmc = wmc[j];
          o.index = idx[j];
          P.particles[h] = o;
        }
        if (P.results)
          P.results[h] = r;
        if (P.steps)
          P.steps[h] = nst[j];
        if (P.scatters)
          P.scatters[h] = nsc[j];
        atomicAdd(&s_cnt[MCG_CNT_HIST], 1ull);
        const unsigned long long wq = (unsigned long long)mcg_to_fixed(wmc[j], qs);
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
    }
    /* compaction: survivors of the whole warp, slot j after slot j-1 */
    unsigned ball[4], total = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      ball[j] = __ballot_sync(0xffffffffu, live[j]);
      total += __popc(ball[j]);
    }
    unsigned wbase = 0;
    if (lane == 0 && total)
      wbase = atomicAdd(P.n_out, total);
    wbase = __shfl_sync(0xffffffffu, wbase, 0);
    unsigned before = 0;
    const unsigned lt = lanemask_lt();
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (live[j]) {
        const unsigned o = wbase + before + __popc(ball[j] & lt);
        P.out.seed[o] = seed[j];
        P.out.x[o] = x[j];
        P.out.mu[o] = mu[j];
        P.out.wmc[o] = wmc[j];
        P.out.idx[o] = idx[j];
        P.out.hid[o] = hid[j];
        P.out.nst[o] = nst[j];
        P.out.nsc[o] = nsc[j];
      }
      before += __popc(ball[j]);
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
  if (tid < MCG_CNT_N && s_cnt[tid]) {
    if (tid == MCG_CNT_ERR)
      atomicOr(&P.counters[tid], s_cnt[tid]);
    else
      atomicAdd(&P.counters[tid], s_cnt[tid]);
  }
}

/* ------------------------------------------------------------ host side */
static int soa_alloc(mcg_soa &s, size_t cap, std::vector<void *> &owned)
{
  void *base = nullptr;
  /* one allocation, each field 256-byte aligned */
  const size_t pad = (cap + 63) & ~(size_t)63;
  cudaError_t e = cudaMalloc(&base, pad * (8 + 7 * 4) + 8 * 256);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "event buffers");
  owned.push_back(base);
  char *p = static_cast<char *>(base);
  s.seed = reinterpret_cast<unsigned long long *>(p);
  p += pad * 8;
  float **f[3] = {&s.x, &s.mu, &s.wmc};
  for (float **q : f) {
    *q = reinterpret_cast<float *>(p);
    p += pad * 4;
  }
  int32_t **ii[5] = {&s.idx, &s.hid, &s.nst, &s.nsc, nullptr};
  for (int k = 0; k < 4; ++k) {
    *ii[k] = reinterpret_cast<int32_t *>(p);
    p += pad * 4;
  }
  return MCG_OK;
}

int mcg_event_run(mcg_context *ctx, mcg_track_params &TP)
{
  const bool strict = ctx->mode == MCG_MODE_STRICT;
  if (TP.n > 0x7fffffffLL)
    return mcg_fail(MCG_ERR_ARG, "event mode: at most 2^31-1 particles per call");
  if ((size_t)TP.n > ctx->event_cap) {
    for (void *p : ctx->event_owned)
      cudaFree(p);
    ctx->event_owned.clear();
    ctx->event_cap = 0;
    int rc;
    if ((rc = soa_alloc(ctx->event_buf[0], TP.n, ctx->event_owned)) != MCG_OK ||
        (rc = soa_alloc(ctx->event_buf[1], TP.n, ctx->event_owned)) != MCG_OK)
      return rc;
    void *cnt = nullptr;
    cudaError_t e = cudaMalloc(&cnt, 256);
    if (e != cudaSuccess)
      return mcg_cuda_fail(e, "event counters");
    ctx->event_owned.push_back(cnt);
    ctx->event_count = static_cast<unsigned *>(cnt);
    ctx->event_cap = (size_t)TP.n;
  }
  mcg_event_params P;
  memset(&P, 0, sizeof(P));
  P.cells = TP.cells;
  P.n_cells = TP.n_cells;
  P.cell_lo = TP.cell_lo;
  P.min_w = TP.min_w;
  P.q_log2 = TP.q_log2;
  P.tally = TP.tally;
  P.counters = TP.counters;
  P.particles = TP.particles;
  P.results = TP.results;
  P.steps = TP.steps;
  P.scatters = TP.scatters;
  P.steps_per_pass = ctx->event_steps;
  P.max_steps = TP.max_steps;
  P.libm = TP.libm;
  P.libm_tab = TP.libm_tab;
  const int grid_init = (int)std::min<int64_t>((TP.n + 255) / 256, (int64_t)ctx->sm_count * 16);
  cudaEventRecord(ctx->ev0, ctx->stream);
  mcg_event_init_kernel<<<grid_init, 256, 0, ctx->stream>>>(TP, ctx->event_buf[0], ctx->event_count);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "event init");
  auto kern = strict ? mcg_event_pass_kernel<true> : mcg_event_pass_kernel<false>;
  int bps = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, 256, 0);
  const int grid = ctx->sm_count * std::max(bps, 1);
  /* passes in groups of 16 between checks of the live count; a pass whose
   * input count is zero returns at once */
  int pass = 0;
  const long long max_passes = (long long)ctx->max_steps / std::max(1, ctx->event_steps) + 2;
  for (;;) {
    for (int g = 0; g < 16; ++g, ++pass) {
      const int a = pass & 1, b = a ^ 1;
      P.in = ctx->event_buf[a];
      P.out = ctx->event_buf[b];
      P.n_in = ctx->event_count + a;
      P.n_out = ctx->event_count + b;
      if ((e = cudaMemsetAsync(ctx->event_count + b, 0, sizeof(unsigned), ctx->stream)) != cudaSuccess)
        return mcg_cuda_fail(e, "event memset");
      kern<<<grid, 256, 0, ctx->stream>>>(P);
      if ((e = cudaGetLastError()) != cudaSuccess)
        return mcg_cuda_fail(e, "event pass");
      ctx->launches++;
    }
    unsigned live = 0;
    if ((e = cudaMemcpyAsync(&live, ctx->event_count + (pass & 1), sizeof(unsigned),
                             cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess)
      return mcg_cuda_fail(e, "event pass loop");
    if (live == 0)
      break;
    if (pass > max_passes)
      return mcg_fail(MCG_ERR_LIMIT, "event mode: particles still alive after %d passes", pass);
  }
  cudaEventRecord(ctx->ev1, ctx->stream);
  ctx->last_grid = grid;
  ctx->last_block = 256;
  ctx->event_passes = pass;
  return MCG_OK;
}

extern "C" int mcg_set_algorithm(mcg_context *ctx, int32_t algorithm, int32_t steps_per_pass)
{
  if (!ctx || (algorithm != MCG_ALGO_HISTORY && algorithm != MCG_ALGO_EVENT) || steps_per_pass < 0)
    return mcg_fail(MCG_ERR_ARG, "mcg_set_algorithm: bad arguments");
  ctx->algorithm = algorithm;
  ctx->event_steps = steps_per_pass ? steps_per_pass : 1;
  return MCG_OK;
}
