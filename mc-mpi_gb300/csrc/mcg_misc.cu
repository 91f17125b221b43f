/*
 * mcg_misc.cu - small device entry points: the reference's rnd_real kernel
 * (src/curandom.cu:7-14), an evaluator of the strict libm, used to check
 * the device arithmetic against the host C library exhaustively, and the
 * check of the tracker's division by a cached reciprocal.
 */
#include "mcg_internal.h"


__global__ void mcg_rnd_real_kernel(uint64_t *seeds, float *reals, int64_t n)
{
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t s = seeds[i];
    reals[i] = mcg_rnd_real(s);
    seeds[i] = s;
  }
}

__global__ void mcg_libm_eval_kernel(int fn, const float *in, float *out, int64_t n,
                                     const mcg_libm_tab *tab, mcg_libm_dev L)
{
  __shared__ mcg_libm_tab T;
  for (int i = threadIdx.x; i < (int)(sizeof(mcg_libm_tab) / 4); i += blockDim.x)
    reinterpret_cast<float *>(&T)[i] = reinterpret_cast<const float *>(tab)[i];
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    float v = in[i], r;
    if (fn == 0)
      r = (v >= 0.0f && v <= 1.0f) ? mcg_logf_strict(v, &T, L) : __int_as_float(0x7fc00000);
    else if (fn == 2)
      r = mcg_ex2_approx(v);
    else if (fn == 4)
      r = __log2f(v);
    else if (fn == 5) {
      /* the fast step's collision probability 1 - e^-tau of optical depth
       * tau >= 0, as mcg_fast_flight computes it */
      r = fabsf(v) < 0x1p-7f ? mcg_one_minus_exp_small(-v) : mcg_one_minus_exp_fast(-v);
    }
    else if (fn == 6)
      /* the fast flight sample's log2 from the state's top 32 bits t,
       * passed as the argument's bit pattern */
      r = mcg_flight_log2((uint64_t)__float_as_uint(v) << 31);
    else if (fn == 3) {
      /* expf with the general path forced for every argument */
      float d = 0.5f;
      r = __int_as_float(0x7fc00000);
      if (v >= MCG_EXP_ONE_BOUND && v < 89.0f) {
        float y = mcg_exp_ff_general(v, mcg_rint_k(__fmul_rn(v, MCG_EXP_INV)), &d, &T);
        r = mcg_exp_fixup(v, y, d, L);
      }
    } else
      r = (v >= MCG_EXP_ONE_BOUND && v < 89.0f) ? mcg_expf_strict(v, &T, L)
                                                : __int_as_float(0x7fc00000);
    out[i] = r;
  }
}

extern "C" int mcg_rnd_real_device(mcg_context *ctx, uint64_t *d_seeds, float *d_reals, int64_t n)
{
  if (!ctx || n < 0 || (n > 0 && (!d_seeds || !d_reals)))
    return mcg_fail(MCG_ERR_ARG, "mcg_rnd_real_device: bad arguments");
  if (n == 0)
    return MCG_OK;
  cudaSetDevice(ctx->device);
  int grid = (int)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->sm_count * 8);
  mcg_rnd_real_kernel<<<grid, 256, 0, ctx->stream>>>(d_seeds, d_reals, n);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(ctx->stream);
  return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(e, "mcg_rnd_real_device");
}

extern "C" int mcg_libm_eval_device(mcg_context *ctx, int fn, const float *d_in, float *d_out,
                                    int64_t n)
{
  if (!ctx || fn < 0 || fn > 6 || n < 0 || (n > 0 && (!d_in || !d_out)))
    return mcg_fail(MCG_ERR_ARG, "mcg_libm_eval_device: bad arguments");
  if (!ctx->libm_loaded)
    return mcg_fail(MCG_ERR_STATE, "mcg_libm_eval_device: needs a strict context");
  if (n == 0)
    return MCG_OK;
  cudaSetDevice(ctx->device);
  int grid = (int)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->sm_count * 8);
  mcg_libm_eval_kernel<<<grid, 256, 0, ctx->stream>>>(fn, d_in, d_out, n, ctx->libm_tab, ctx->libm);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(ctx->stream);
  return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(e, "mcg_libm_eval_device");
}

/* Checks mcg_div_by_rcp against the IEEE quotient.  mode 0: every pair of
 * significands a, b in [1, 2) (b from b_first, b_count of them); mode 1: n
 * pseudo-random pairs of either sign, |a| in [2^-100, 4), |b| in
 * [2^-14, 1).  out[0] += pairs checked, out[1] += mismatches,
 * out[2] = bits of one mismatching pair (a << 32 | b) if any. */
__global__ void mcg_verify_div_kernel(int mode, uint32_t b_first, uint32_t b_count, uint64_t n,
                                      unsigned long long *out)
{
  unsigned long long checked = 0, bad = 0;
  if (mode == 0) {
    for (uint32_t jb = b_first + blockIdx.x; jb < b_first + b_count; jb += gridDim.x) {
      const float b = __uint_as_float(0x3f800000u | jb), y = __frcp_rn(b);
      for (uint32_t ia = threadIdx.x; ia < (1u << 23); ia += blockDim.x) {
        const float a = __uint_as_float(0x3f800000u | ia);
        const float q = mcg_div_by_rcp(a, b, y), ref = __fdiv_rn(a, b);
        ++checked;
        if (__float_as_uint(q) != __float_as_uint(ref)) {
          ++bad;
          atomicCAS(out + 2, 0ull, ((unsigned long long)__float_as_uint(a) << 32) | __float_as_uint(b));
        }
      }
    }
  } else {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
      uint64_t h = (i + 1) * 0x9E3779B97F4A7C15ull;
      h ^= h >> 31;
      h *= 0xBF58476D1CE4E5B9ull;
      h ^= h >> 29;
      const uint32_t u = (uint32_t)h, v = (uint32_t)(h >> 32);
      const uint32_t ea = 27u + (u >> 8) % 102u, eb = 113u + (v >> 8) % 14u;
      const float a = __uint_as_float((u & 0x80000000u) | (ea << 23) | ((u * 2654435761u) & 0x7fffffu));
      const float b = __uint_as_float((v & 0x80000000u) | (eb << 23) | ((v * 2246822519u) & 0x7fffffu));
      const float q = mcg_div_by_rcp(a, b, __frcp_rn(b)), ref = __fdiv_rn(a, b);
      ++checked;
      if (__float_as_uint(q) != __float_as_uint(ref)) {
        ++bad;
        atomicCAS(out + 2, 0ull, ((unsigned long long)__float_as_uint(a) << 32) | __float_as_uint(b));
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    checked += __shfl_down_sync(0xffffffffu, checked, o);
    bad += __shfl_down_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out, checked);
    if (bad)
      atomicAdd(out + 1, bad);
  }
}

extern "C" int mcg_verify_division(mcg_context *ctx, int mode, uint64_t n, uint64_t *checked,
                                   uint64_t *mismatches, uint64_t *example)
{
  if (!ctx || (mode != 0 && mode != 1) || !checked || !mismatches || !example)
    return mcg_fail(MCG_ERR_ARG, "mcg_verify_division: bad arguments");
  cudaSetDevice(ctx->device);
  unsigned long long *d = nullptr;
  cudaError_t e = cudaMalloc(&d, 3 * sizeof(unsigned long long));
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "cudaMalloc(verify)");
  e = cudaMemsetAsync(d, 0, 3 * sizeof(unsigned long long), ctx->stream);
  const int grid = ctx->sm_count * 8;
  /* mode 0 in 64 launches of 2^17 divisors (about half a second each) */
  for (int part = 0; e == cudaSuccess && part < (mode == 0 ? 64 : 1); ++part) {
    mcg_verify_div_kernel<<<grid, 256, 0, ctx->stream>>>(mode, (uint32_t)part << 17, 1u << 17, n, d);
    e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaStreamSynchronize(ctx->stream);
  }
  unsigned long long h[3] = {0, 0, 0};
  if (e == cudaSuccess)
    e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_verify_division");
  *checked = h[0];
  *mismatches = h[1];
  *example = h[2];
  return MCG_OK;
}

/* Throughput of the int <-> float conversions the trackers use (testing
 * aid for the roofline): every thread runs four independent dependency
 * chains of `iters` conversions of one kind, each followed by one 32-bit
 * logic operation that feeds the next conversion.  kind 0: u64 -> f32,
 * 1: f32 -> s64, 2: u32 -> f32, 3: f32 -> u32 (round to nearest). */
__global__ void mcg_conv_rate_kernel(int kind, int iters, unsigned long long *sink)
{
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t u[4];
  float f[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    u[j] = (0x9E3779B97F4A7C15ull * (t * 4u + j + 1)) >> 2;
    f[j] = __uint_as_float(0x3f800000u | ((uint32_t)u[j] & 0x7fffffu)) * 1.0e6f;
  }
  if (kind == 0) {
    for (int i = 0; i < iters; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j)
        u[j] ^= __float_as_uint(__ull2float_rn(u[j]));
  } else if (kind == 1) {
    for (int i = 0; i < iters; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j)
        f[j] = __uint_as_float(__float_as_uint(f[j]) ^ ((uint32_t)__float2ll_rn(f[j]) & 0x3ffu));
  } else if (kind == 2) {
    for (int i = 0; i < iters; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j)
        u[j] ^= __float_as_uint(__uint2float_rn((uint32_t)u[j]));
  } else {
    for (int i = 0; i < iters; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j)
        f[j] = __uint_as_float(__float_as_uint(f[j]) ^ (__float2uint_rn(f[j]) & 0x3ffu));
  }
  unsigned long long x = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j)
    x ^= u[j] ^ __float_as_uint(f[j]);
  if (x == 0x1234567ull) /* never in practice; keeps the chains live */
    sink[0] = x;
}

extern "C" int mcg_measure_conversion_rates(mcg_context *ctx, double *h_rates)
{
  if (!ctx || !h_rates)
    return mcg_fail(MCG_ERR_ARG, "mcg_measure_conversion_rates: bad arguments");
  cudaSetDevice(ctx->device);
  unsigned long long *d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(unsigned long long));
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "cudaMalloc(conversion rates)");
  const int grid = ctx->sm_count * 8, block = 256, iters = 2048;
  for (int kind = 0; kind < 4 && e == cudaSuccess; ++kind) {
    float ms = 0.f;
    for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) { /* warm-up, then timed */
      cudaEventRecord(ctx->ev0, ctx->stream);
      mcg_conv_rate_kernel<<<grid, block, 0, ctx->stream>>>(kind, iters, d);
      e = cudaGetLastError();
      cudaEventRecord(ctx->ev1, ctx->stream);
      if (e == cudaSuccess)
        e = cudaStreamSynchronize(ctx->stream);
      if (e == cudaSuccess)
        e = cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    }
    h_rates[kind] = (double)grid * block * iters * 4 / (ms * 1e-3);
  }
  cudaFree(d);
  return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(e, "mcg_measure_conversion_rates");
}
