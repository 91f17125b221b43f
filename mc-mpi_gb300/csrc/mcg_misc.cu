/*
 * mcg_misc.cu - small device entry points: the reference's rnd_real kernel
 * (src/curandom.cu:7-14) and an evaluator of the strict libm, used to check
 * the device arithmetic against the host C library exhaustively.
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
    else
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
  if (!ctx || fn < 0 || fn > 2 || n < 0 || (n > 0 && (!d_in || !d_out)))
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
