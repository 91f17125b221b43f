/*
 * mcg_noalloc.cu - the fast history tracker for callers that may not
 * allocate device memory.
 *
 * Some host codes reserve the GPU's memory for their own pool when they start
 * (an MPI transport code that sizes all of its buffers at initialisation, or
 * an application whose allocator owns the device) and then forbid libraries
 * from calling cudaMalloc/cudaFree, which may also synchronise the device in
 * the middle of their time step.  mcg_simulate_fast_noalloc serves them: the
 * caller passes the inputs and outputs, and everything else the tracker needs
 * between them (the per-cell step table, the fixed-point tally the blocks
 * flush into, the work counter and the event counters) lives in one
 * file-scope device array of fixed size, compiled into the library.
 *
 * The array is shared by every call on a device and keeps the previous
 * call's contents; each call clears the parts that must start at zero.  The
 * call is synchronous and holds a process-wide lock from the scratch set-up
 * to its return, so calls from several host threads of this process run one
 * after another; another process on the same GPU has its own copy of the
 * array.
 */
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <vector>

#include "mcg_internal.h"
#include "mcg_track.cuh"

/* Layout of the scratch array (bytes): step table, tally, counters, work
 * counter.  The tally region is sized as 8 bytes per cell. */
#define MCG_NOALLOC_CELLS_OFF 0
#define MCG_NOALLOC_TALLY_OFF (MCG_NOALLOC_CELLS_OFF + 16 * MCG_NOALLOC_MAX_CELLS)
#define MCG_NOALLOC_CNT_OFF (MCG_NOALLOC_TALLY_OFF + 8 * MCG_NOALLOC_MAX_CELLS)
#define MCG_NOALLOC_NEXT_OFF (MCG_NOALLOC_CNT_OFF + 8 * 16)
#define MCG_NOALLOC_BYTES (MCG_NOALLOC_NEXT_OFF + 256)

static __device__ __align__(256) unsigned char g_noalloc_scratch[MCG_NOALLOC_BYTES];

/* Serialises whole calls (the scratch array is shared). */
static std::mutex g_noalloc_call_mu;

/* Device address of g_noalloc_scratch in the current device's context.  In
 * host code the symbol names a host-side stand-in, not device memory, so the
 * address is looked up with the device current, on every call: a caller that
 * resets the device (cudaDeviceReset) or otherwise recreates its context gets
 * the new context's copy of the array, never a stale address. */
static int noalloc_scratch(unsigned char **out)
{
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "cudaGetSymbolAddress(no-allocation scratch)");
  *out = static_cast<unsigned char *>(p);
  return MCG_OK;
}

extern "C" int mcg_simulate_fast_noalloc(int n_layers, const int32_t *h_index_start,
                                         const int32_t *h_m, const float *h_dx,
                                         const float *h_sigs, const float *h_rates,
                                         float particle_min_weight, int32_t log2_scale,
                                         mcg_particle *d_particles, int64_t n,
                                         int32_t *d_results, int64_t *d_tally_q)
{
  if (n_layers <= 0 || !h_index_start || !h_m || !h_dx || !h_sigs || !h_rates || n < 0 ||
      (n > 0 && !d_particles) || !d_tally_q || log2_scale < 0 || log2_scale > 62)
    return mcg_fail(MCG_ERR_ARG, "mcg_simulate_fast_noalloc: bad arguments");
  /* the running total is checked against the limit at every layer, so it
   * never grows past MCG_NOALLOC_MAX_CELLS + INT32_MAX (held in 64 bits) */
  int64_t total64 = 0;
  for (int l = 0; l < n_layers; ++l) {
    if (h_m[l] <= 0 || (l > 0 && (int64_t)h_index_start[l] !=
                                     (int64_t)h_index_start[l - 1] + h_m[l - 1]))
      return mcg_fail(MCG_ERR_ARG, "mcg_simulate_fast_noalloc: layer %d is empty or not contiguous", l);
    total64 += h_m[l];
    if (total64 > MCG_NOALLOC_MAX_CELLS)
      return mcg_fail(MCG_ERR_ARG,
                      "mcg_simulate_fast_noalloc: chain of more than %d cells exceeds the fixed "
                      "scratch (at most %d cells)", MCG_NOALLOC_MAX_CELLS, MCG_NOALLOC_MAX_CELLS);
  }
  const int total = (int)total64;
  if (n > 0 && (reinterpret_cast<uintptr_t>(d_particles) & 7u))
    return mcg_fail(MCG_ERR_ARG, "mcg_simulate_fast_noalloc: d_particles must be 8-byte aligned");
  std::lock_guard<std::mutex> call_lock(g_noalloc_call_mu);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "cudaGetDevice");
  unsigned char *base = nullptr;
  int rc = noalloc_scratch(&base);
  if (rc != MCG_OK)
    return rc;
  float4 *cells = reinterpret_cast<float4 *>(base + MCG_NOALLOC_CELLS_OFF);
  unsigned long long *tally = reinterpret_cast<unsigned long long *>(base + MCG_NOALLOC_TALLY_OFF);
  unsigned long long *cnt = reinterpret_cast<unsigned long long *>(base + MCG_NOALLOC_CNT_OFF);
  unsigned long long *next = reinterpret_cast<unsigned long long *>(base + MCG_NOALLOC_NEXT_OFF);

  /* step table on the host (as mcg_set_layers), then into the scratch */
  std::vector<float4> cs(total), cf(total);
  int k = 0;
  for (int l = 0; l < n_layers; ++l)
    for (int j = 0; j < h_m[l]; ++j, ++k)
      mcg_cell_params(h_sigs[k], h_rates[k], h_index_start[l] + j, h_dx[l], cs[k], cf[k]);
  cudaStream_t st = 0;
  if ((e = cudaMemcpyAsync(cells, cf.data(), total * sizeof(float4), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(tally, 0, total * sizeof(unsigned long long), st)) != cudaSuccess ||
      (e = cudaMemsetAsync(cnt, 0, 16 * sizeof(unsigned long long), st)) != cudaSuccess ||
      (e = cudaMemsetAsync(next, 0, sizeof(unsigned long long), st)) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_simulate_fast_noalloc: scratch set-up");

  if (n > 0) {
    mcg_track_params P;
    memset(&P, 0, sizeof(P));
    P.cells = cells;
    P.n_cells = total;
    P.cell_lo = h_index_start[0];
    P.min_w = particle_min_weight;
    P.q_log2 = log2_scale;
    P.particles = d_particles;
    P.results = d_results;
    P.n = n;
    P.next = next;
    P.tally = tally;
    P.counters = cnt;
    P.refill_steps = 8;
    P.chunk = 64;
    P.max_steps = 1u << 28;
    const int block = ((size_t)total * 8 * 8 <= 24 * 1024) ? 256 : 1024;
    const int warps = block / 32;
    const int copies = ((size_t)total * 8 * warps <= 24 * 1024) ? warps : 1;
    P.tally_copies = copies;
    const size_t base_smem = sizeof(mcg_libm_tab) + 16 * sizeof(unsigned long long);
    int sms = 0, optin = 0, bps = 0;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
        (e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess)
      return mcg_cuda_fail(e, "mcg_simulate_fast_noalloc: device attributes");
    /* as the context path: a chain whose tally does not fit in the block's
     * shared memory adds its deposits to the scratch tally directly */
    const bool smem_tally = base_smem + (size_t)total * 8 * copies <= (size_t)optin;
    const size_t smem = base_smem + (smem_tally ? (size_t)total * 8 * copies : 0);
    auto kern = smem_tally ? mcg_track_kernel<false, MCG_TALLY_SMEM32, false>
                           : mcg_track_kernel<false, MCG_TALLY_GLOBAL, false>;
    /* the attribute is raised to the device's limit (the same value every
     * caller of this library sets), so a concurrent launch of the same kernel
     * from another host thread can never lower it below this launch's need */
    if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin)) != cudaSuccess ||
        (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, block, smem)) != cudaSuccess)
      return mcg_cuda_fail(e, "mcg_simulate_fast_noalloc: launch set-up");
    long long want = (n + block - 1) / block;
    int grid = (int)std::min<long long>((long long)sms * std::max(bps, 1), std::max(want, 1LL));
    kern<<<grid, block, smem, st>>>(P);
    if ((e = cudaGetLastError()) != cudaSuccess)
      return mcg_cuda_fail(e, "mcg_simulate_fast_noalloc: launch");
  }
  unsigned long long err = 0;
  if ((e = cudaMemcpyAsync(d_tally_q, tally, total * sizeof(int64_t), cudaMemcpyDeviceToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(&err, cnt + MCG_CNT_ERR, sizeof(err), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_simulate_fast_noalloc");
  if (err)
    return mcg_fail(MCG_ERR_LIMIT, "mcg_simulate_fast_noalloc: a history exceeded the step limit");
  return MCG_OK;
}
