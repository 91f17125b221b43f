/*
 * mcg_api.cu - host side of libmcgb300: contexts, layer set-up, the strict
 * libm exception tables, kernel launches and the C ABI of include/mcgb300.h.
 */
#include <cuda_runtime.h>

#include <atomic>
#include <new>
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "exact_libm.h"
#include "libm_file.h"
#include "mcg_internal.h"
#include "mcg_track.cuh"

static thread_local std::string g_last_error;

int mcg_fail(int code, const char *fmt, ...)
{
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int mcg_cuda_fail(cudaError_t e, const char *what)
{
  return mcg_fail(MCG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

extern "C" const char *mcg_last_error(void) { return g_last_error.c_str(); }
extern "C" const char *mcg_version(void) { return "mcgb300 1.0 (sm_103a)"; }

/* ------------------------------------------------------------ libm tables */
static std::string library_dir()
{
  Dl_info info;
  if (dladdr((void *)&mcg_version, &info) && info.dli_fname) {
    std::string p(info.dli_fname);
    size_t s = p.find_last_of('/');
    return s == std::string::npos ? std::string(".") : p.substr(0, s);
  }
  return ".";
}

static int build_hash(const std::vector<uint32_t> &pairs, std::vector<uint2> &tab, uint32_t &mask,
                      int &probes)
{
  size_t n = pairs.size() / 2, cap = 64;
  while (cap < 2 * n + 1)
    cap <<= 1;
  tab.assign(cap, make_uint2(MCG_HASH_EMPTY, 0u));
  mask = (uint32_t)(cap - 1);
  probes = 1;
  for (size_t i = 0; i < n; ++i) {
    uint32_t key = pairs[2 * i], slot = (key * 0x9E3779B1u) & mask;
    int p = 1;
    while (tab[slot].x != MCG_HASH_EMPTY) {
      if (tab[slot].x == key)
        return mcg_fail(MCG_ERR_TABLES, "duplicate key in libm exception table");
      slot = (slot + 1) & mask;
      ++p;
    }
    tab[slot] = make_uint2(key, pairs[2 * i + 1]);
    probes = std::max(probes, p);
  }
  probes += 1; /* one more probe reaches the empty slot that ends a miss */
  return MCG_OK;
}

int mcg_load_libm(mcg_context *ctx)
{
  if (ctx->libm_loaded)
    return MCG_OK;
  const char *env = getenv("MCG_LIBM_TABLE");
  std::string path = env ? std::string(env) : library_dir() + "/libm_exceptions.bin";
  FILE *f = fopen(path.c_str(), "rb");
  if (!f)
    return mcg_fail(MCG_ERR_TABLES,
                    "strict mode needs the host-libm exception table %s (built by build())",
                    path.c_str());
  mcg_libm_file hdr;
  std::vector<uint32_t> lp, ep;
  bool ok = fread(&hdr, sizeof(hdr), 1, f) == 1 && memcmp(hdr.magic, MCG_LIBM_MAGIC, 8) == 0;
  if (ok) {
    lp.resize(2 * (size_t)hdr.n_log);
    ep.resize(2 * (size_t)hdr.n_exp);
    ok = (lp.empty() || fread(lp.data(), 4, lp.size(), f) == lp.size()) &&
         (ep.empty() || fread(ep.data(), 4, ep.size(), f) == ep.size());
  }
  fclose(f);
  if (!ok)
    return mcg_fail(MCG_ERR_TABLES, "malformed libm exception table %s", path.c_str());
  const mcg_libm_tab tab = MCG_LIBM_TAB_INIT;
  if (hdr.fingerprint != mcg_libm_fingerprint(&tab))
    return mcg_fail(MCG_ERR_TABLES,
                    "libm exception table %s was made against another C library (%s) or "
                    "another version of the evaluators; rebuild",
                    path.c_str(), hdr.libc_version);
  if (!(hdr.logf_relerr <= MCG_LOGF_RELERR_MAX))
    return mcg_fail(MCG_ERR_TABLES,
                    "host logf relative error %.3e exceeds the %.3e the strict tracker's "
                    "certain-crossing test assumes",
                    (double)hdr.logf_relerr, (double)MCG_LOGF_RELERR_MAX);
  std::vector<uint2> hl, he;
  int rc;
  if ((rc = build_hash(lp, hl, ctx->libm.mask_log, ctx->libm.probes_log)) != MCG_OK)
    return rc;
  if ((rc = build_hash(ep, he, ctx->libm.mask_exp, ctx->libm.probes_exp)) != MCG_OK)
    return rc;
  float tl = -1.f, te = -1.f;
  for (int b = 0; b < MCG_TAU_BUCKETS; ++b) {
    tl = std::max(tl, hdr.tau_log[b]);
    te = std::max(te, hdr.tau_exp[b]);
  }
  ctx->libm.tau_log_max = tl;
  ctx->libm.tau_exp_max = te;
  cudaError_t e;
  float *dtl = nullptr, *dte = nullptr;
  uint2 *dhl = nullptr, *dhe = nullptr;
  mcg_libm_tab *dtab = nullptr;
  /* each allocation joins the context's list as soon as it exists, so a
   * failure part-way leaves nothing behind at mcg_destroy */
  auto alloc = [ctx](void **p, size_t bytes) {
    cudaError_t r = cudaMalloc(p, bytes);
    if (r == cudaSuccess)
      ctx->owned.push_back(*p);
    return r;
  };
  if ((e = alloc((void **)&dtl, sizeof(hdr.tau_log))) != cudaSuccess ||
      (e = alloc((void **)&dte, sizeof(hdr.tau_exp))) != cudaSuccess ||
      (e = alloc((void **)&dhl, hl.size() * sizeof(uint2))) != cudaSuccess ||
      (e = alloc((void **)&dhe, he.size() * sizeof(uint2))) != cudaSuccess ||
      (e = alloc((void **)&dtab, sizeof(tab))) != cudaSuccess)
    return mcg_cuda_fail(e, "cudaMalloc(libm tables)");
  if ((e = cudaMemcpy(dtl, hdr.tau_log, sizeof(hdr.tau_log), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(dte, hdr.tau_exp, sizeof(hdr.tau_exp), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(dhl, hl.data(), hl.size() * sizeof(uint2), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(dhe, he.data(), he.size() * sizeof(uint2), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(dtab, &tab, sizeof(tab), cudaMemcpyHostToDevice)) != cudaSuccess)
    return mcg_cuda_fail(e, "cudaMemcpy(libm tables)");
  ctx->libm.tau_log = dtl;
  ctx->libm.tau_exp = dte;
  ctx->libm.hash_log = dhl;
  ctx->libm.hash_exp = dhe;
  ctx->libm_tab = dtab;
  ctx->libm_n_log = hdr.n_log;
  ctx->libm_n_exp = hdr.n_exp;
  ctx->libm_loaded = true;
  return MCG_OK;
}

/* ------------------------------------------------------------ context */
static int ensure_device(const mcg_context *ctx)
{
  cudaError_t e = cudaSetDevice(ctx->device);
  return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(e, "cudaSetDevice");
}

extern "C" int mcg_create(int device, int mode, mcg_context **out)
{
  if (!out || (mode != MCG_MODE_STRICT && mode != MCG_MODE_FAST))
    return mcg_fail(MCG_ERR_ARG, "mcg_create: bad arguments");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "cudaGetDeviceCount");
  if (device < 0 || device >= ndev)
    return mcg_fail(MCG_ERR_ARG, "mcg_create: device %d of %d", device, ndev);
  mcg_context *ctx = new mcg_context();
  ctx->device = device;
  ctx->mode = mode;
  int rc = ensure_device(ctx);
  if (rc == MCG_OK) {
    cudaDeviceProp prop;
    if ((e = cudaGetDeviceProperties(&prop, device)) != cudaSuccess)
      rc = mcg_cuda_fail(e, "cudaGetDeviceProperties");
    else {
      ctx->sm_count = prop.multiProcessorCount;
      ctx->smem_optin = (int)prop.sharedMemPerBlockOptin;
      ctx->cc_major = prop.major;
      ctx->cc_minor = prop.minor;
    }
  }
  if (rc == MCG_OK && ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess ||
                       (e = cudaEventCreate(&ctx->ev0)) != cudaSuccess ||
                       (e = cudaEventCreate(&ctx->ev1)) != cudaSuccess))
    rc = mcg_cuda_fail(e, "stream/event create");
  if (rc == MCG_OK) {
    if ((e = cudaMalloc(&ctx->d_counters, 16 * sizeof(unsigned long long))) == cudaSuccess)
      ctx->owned.push_back(ctx->d_counters);
    if (e == cudaSuccess &&
        (e = cudaMalloc(&ctx->d_next, 8 * sizeof(unsigned long long))) == cudaSuccess)
      ctx->owned.push_back(ctx->d_next);
    if (e != cudaSuccess)
      rc = mcg_cuda_fail(e, "cudaMalloc(counters)");
    else
      cudaMemset(ctx->d_counters, 0, 16 * sizeof(unsigned long long));
  }
  if (rc == MCG_OK && mode == MCG_MODE_STRICT)
    rc = mcg_load_libm(ctx);
  if (rc != MCG_OK) {
    std::string msg = g_last_error;
    mcg_destroy(ctx);
    g_last_error = msg;
    return rc;
  }
  *out = ctx;
  return MCG_OK;
}

/* Releases the chain's device buffers and leaves the context with no
 * geometry: launches and tally reads then return MCG_ERR_STATE. */
static void free_geometry(mcg_context *ctx)
{
  for (void *p : {(void *)ctx->d_cells_strict, (void *)ctx->d_cells_fast, (void *)ctx->d_tally})
    if (p)
      cudaFree(p);
  ctx->d_cells_strict = ctx->d_cells_fast = nullptr;
  ctx->d_tally = nullptr;
  ctx->n_layers = ctx->n_cells = ctx->cell_lo = 0;
  ctx->layer_start.clear();
  ctx->layer_m.clear();
  ctx->layer_dx.clear();
  ctx->sigs.clear();
  ctx->rates.clear();
  ctx->cells_strict.clear();
  ctx->cells_fast.clear();
  ctx->thin = false;
}

/* Allocations still to succeed before one is made to fail (-1: none). */
static std::atomic<int> g_fail_alloc_in{-1};

cudaError_t mcg_dev_malloc(void **p, size_t bytes)
{
  int k = g_fail_alloc_in.load();
  while (k >= 0) {
    if (g_fail_alloc_in.compare_exchange_weak(k, k - 1)) {
      if (k == 0) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
      }
      break;
    }
  }
  return cudaMalloc(p, bytes);
}

extern "C" int mcg_testing_fail_allocation(int32_t after)
{
  g_fail_alloc_in.store(after < 0 ? -1 : after);
  return MCG_OK;
}

static void free_scratch(mcg_context *ctx)
{
  for (void *p : {(void *)ctx->d_part, (void *)ctx->d_res, (void *)ctx->d_steps, (void *)ctx->d_scat})
    if (p)
      cudaFree(p);
  ctx->d_part = nullptr;
  ctx->d_res = nullptr;
  ctx->d_steps = ctx->d_scat = nullptr;
  ctx->scratch_cap = 0;
}

extern "C" int mcg_destroy(mcg_context *ctx)
{
  if (!ctx)
    return MCG_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream)
    cudaStreamSynchronize(ctx->stream);
  free_geometry(ctx);
  free_scratch(ctx);
  mcg_fit_release(ctx);
  mcg_ext_destroy(ctx);
  for (void *p : ctx->owned)
    cudaFree(p);
  for (void *p : ctx->event_owned)
    cudaFree(p);
  if (ctx->ev0)
    cudaEventDestroy(ctx->ev0);
  if (ctx->ev1)
    cudaEventDestroy(ctx->ev1);
  if (ctx->stream)
    cudaStreamDestroy(ctx->stream);
  delete ctx;
  return MCG_OK;
}

extern "C" int mcg_set_mode(mcg_context *ctx, int mode)
{
  if (!ctx || (mode != MCG_MODE_STRICT && mode != MCG_MODE_FAST))
    return mcg_fail(MCG_ERR_ARG, "mcg_set_mode: bad arguments");
  int rc = ensure_device(ctx);
  if (rc == MCG_OK && mode == MCG_MODE_STRICT)
    rc = mcg_load_libm(ctx);
  if (rc == MCG_OK)
    ctx->mode = mode;
  return rc;
}

/* Per-cell step parameters exactly as Layer::particle_step forms them
 * (src/layer.cpp:129-131, 146, 150). */
void mcg_cell_params(float sig, float rate, int gi, float dx, float4 &strict, float4 &fast)
{
  const float interaction_rate = (float)(1.0 - (double)rate);
  const float sig_a = sig * rate;
  const float sig_i = sig * interaction_rate;
  const float elo = (float)gi * dx, ehi = (float)(gi + 1) * dx;
  strict = make_float4(sig_a, sig_i, elo, ehi);
  fast = make_float4(sig_a, sig_i > 1e-4f ? sig_i : 0.0f,
                     elo, ehi);
}

/* A chain is optically thin when every cell's absorption optical width
 * sig_a (edge_hi - edge_lo) is at most 5e-4: a crossing then has
 * |sig_a d_edge| >= MCG_EXP_SMALL_T (0.0054) only for |mu| < 0.093, which
 * takes under 1 % of the crossings (their share of directions is about
 * mu^2), so the strict tracker's certain-crossing path may evaluate the
 * small-argument exp form alone and send the others to the full step. */
static void update_thin(mcg_context *ctx)
{
  float widest = 0.0f;
  for (const float4 &c : ctx->cells_strict)
    widest = std::max(widest, std::fabs(c.x) * (c.w - c.z));
  ctx->thin = !ctx->cells_strict.empty() && widest <= 5e-4f;
}

extern "C" int mcg_set_layers(mcg_context *ctx, int n_layers, const int32_t *h_index_start,
                              const int32_t *h_m, const float *h_dx, const float *h_sigs,
                              const float *h_rates, float particle_min_weight)
{
  if (!ctx || n_layers <= 0 || !h_index_start || !h_m || !h_dx || !h_sigs || !h_rates)
    return mcg_fail(MCG_ERR_ARG, "mcg_set_layers: bad arguments");
  int64_t total64 = 0;
  for (int l = 0; l < n_layers; ++l) {
    if (h_m[l] <= 0)
      return mcg_fail(MCG_ERR_ARG, "mcg_set_layers: layer %d has %d cells", l, h_m[l]);
    if (l > 0 && (int64_t)h_index_start[l] != (int64_t)h_index_start[l - 1] + h_m[l - 1])
      return mcg_fail(MCG_ERR_ARG, "mcg_set_layers: layer %d is not contiguous", l);
    total64 += h_m[l];
    if (total64 > INT32_MAX)
      return mcg_fail(MCG_ERR_ARG, "mcg_set_layers: more than 2^31 - 1 cells");
  }
  const int total = (int)total64;
  int rc = ensure_device(ctx);
  if (rc != MCG_OK)
    return rc;
  std::vector<float4> cs, cf;
  try {
    cs.resize(total);
    cf.resize(total);
  } catch (const std::bad_alloc &) {
    return mcg_fail(MCG_ERR_ARG, "mcg_set_layers: no host memory for %d cells", total);
  }
  int k = 0;
  for (int l = 0; l < n_layers; ++l)
    for (int j = 0; j < h_m[l]; ++j, ++k)
      mcg_cell_params(h_sigs[k], h_rates[k], h_index_start[l] + j, h_dx[l], cs[k], cf[k]);
  cudaStreamSynchronize(ctx->stream);
  /* the old geometry goes first; any failure below leaves no geometry */
  free_geometry(ctx);
  cudaError_t e;
  if ((e = mcg_dev_malloc((void **)&ctx->d_cells_strict, total * sizeof(float4))) != cudaSuccess ||
      (e = mcg_dev_malloc((void **)&ctx->d_cells_fast, total * sizeof(float4))) != cudaSuccess ||
      (e = mcg_dev_malloc((void **)&ctx->d_tally, total * sizeof(unsigned long long))) != cudaSuccess) {
    free_geometry(ctx);
    return mcg_cuda_fail(e, "cudaMalloc(layers)");
  }
  if ((e = cudaMemcpy(ctx->d_cells_strict, cs.data(), total * sizeof(float4), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(ctx->d_cells_fast, cf.data(), total * sizeof(float4), cudaMemcpyHostToDevice)) != cudaSuccess) {
    free_geometry(ctx);
    return mcg_cuda_fail(e, "cudaMemcpy(layers)");
  }
  ctx->n_layers = n_layers;
  ctx->layer_start.assign(h_index_start, h_index_start + n_layers);
  ctx->layer_m.assign(h_m, h_m + n_layers);
  ctx->layer_dx.assign(h_dx, h_dx + n_layers);
  ctx->sigs.assign(h_sigs, h_sigs + total);
  ctx->rates.assign(h_rates, h_rates + total);
  ctx->cells_strict = cs;
  ctx->cells_fast = cf;
  update_thin(ctx);
  ctx->n_cells = total;
  ctx->cell_lo = h_index_start[0];
  ctx->min_w = particle_min_weight;
  return mcg_tally_reset(ctx);
}

/* Same as mcg_set_layers with the two cross sections of particle_step given
 * per cell directly: sig_a (absorption) and sig_s (flight sampling). */
extern "C" int mcg_set_layers_xs(mcg_context *ctx, int n_layers, const int32_t *h_index_start,
                                 const int32_t *h_m, const float *h_dx, const float *h_sig_a,
                                 const float *h_sig_s, float particle_min_weight)
{
  if (!ctx || n_layers <= 0 || !h_index_start || !h_m || !h_dx || !h_sig_a || !h_sig_s)
    return mcg_fail(MCG_ERR_ARG, "mcg_set_layers_xs: bad arguments");
  int64_t total64 = 0;
  for (int l = 0; l < n_layers; ++l) {
    if (h_m[l] <= 0 || (l > 0 && (int64_t)h_index_start[l] != (int64_t)h_index_start[l - 1] + h_m[l - 1]))
      return mcg_fail(MCG_ERR_ARG, "mcg_set_layers_xs: layer %d is empty or not contiguous", l);
    total64 += h_m[l];
    if (total64 > INT32_MAX)
      return mcg_fail(MCG_ERR_ARG, "mcg_set_layers_xs: more than 2^31 - 1 cells");
  }
  const int total = (int)total64;
  std::vector<float> sigs(total), rates(total);
  for (int c = 0; c < total; ++c) {
    sigs[c] = h_sig_a[c] + h_sig_s[c];
    rates[c] = sigs[c] > 0.0f ? h_sig_a[c] / sigs[c] : 0.0f;
  }
  int rc = mcg_set_layers(ctx, n_layers, h_index_start, h_m, h_dx, sigs.data(), rates.data(),
                          particle_min_weight);
  if (rc != MCG_OK)
    return rc;
  /* replace the derived cross sections by the given ones */
  int k = 0;
  for (int l = 0; l < n_layers; ++l)
    for (int j = 0; j < h_m[l]; ++j, ++k) {
      float4 &cs = ctx->cells_strict[k], &cf = ctx->cells_fast[k];
      cs.x = cf.x = h_sig_a[k];
      cs.y = h_sig_s[k];
      cf.y = h_sig_s[k] > 1e-4f ? h_sig_s[k] : 0.0f;
    }
  update_thin(ctx);
  cudaError_t e;
  if ((e = cudaMemcpy(ctx->d_cells_strict, ctx->cells_strict.data(), total * sizeof(float4),
                      cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(ctx->d_cells_fast, ctx->cells_fast.data(), total * sizeof(float4),
                      cudaMemcpyHostToDevice)) != cudaSuccess) {
    free_geometry(ctx);
    return mcg_cuda_fail(e, "mcg_set_layers_xs: upload");
  }
  return MCG_OK;
}

extern "C" int mcg_set_slab(mcg_context *ctx, float x_min, float x_max, int32_t nb_cells,
                            int32_t n_layers, const float *h_sigs, const float *h_rates,
                            float particle_min_weight)
{
  if (!ctx || nb_cells <= 0 || n_layers <= 0 || n_layers > nb_cells || !(x_max > x_min))
    return mcg_fail(MCG_ERR_ARG, "mcg_set_slab: bad arguments");
  std::vector<int32_t> st(n_layers), m(n_layers);
  std::vector<float> dx(n_layers), sigs(nb_cells), rates(nb_cells);
  /* decompose_domain (src/layer.cpp:17-42) and Layer::Layer (:44-69) */
  const int cpl = nb_cells / n_layers, extra = nb_cells % n_layers;
  const float gdx = (x_max - x_min) / ((float)nb_cells);
  for (int r = 0; r < n_layers; ++r) {
    m[r] = cpl + (r < extra);
    st[r] = r * cpl + std::min(r, extra);
    const float lx0 = x_min + (float)st[r] * gdx, lx1 = x_min + (float)(st[r] + m[r]) * gdx;
    dx[r] = (lx1 - lx0) / (float)m[r];
    for (int i = 0; i < m[r]; ++i) {
      const float x_mid = (float)((double)(lx0 + (float)i * dx[r]) + 0.5 * (double)dx[r]);
      sigs[st[r] + i] = h_sigs ? h_sigs[st[r] + i] : expf(-x_mid);
      rates[st[r] + i] = h_rates ? h_rates[st[r] + i] : 0.5f;
    }
  }
  return mcg_set_layers(ctx, n_layers, st.data(), m.data(), dx.data(), sigs.data(), rates.data(),
                        particle_min_weight);
}

extern "C" int mcg_set_tally_scale(mcg_context *ctx, int32_t log2_scale)
{
  if (!ctx || log2_scale < 0 || log2_scale > 62)
    return mcg_fail(MCG_ERR_ARG, "mcg_set_tally_scale: scale 2^%d out of [0, 62]", log2_scale);
  ctx->log2_scale = log2_scale;
  return mcg_tally_reset(ctx);
}

extern "C" int mcg_tally_reset(mcg_context *ctx)
{
  if (!ctx)
    return mcg_fail(MCG_ERR_ARG, "mcg_tally_reset: null context");
  int rc = ensure_device(ctx);
  if (rc != MCG_OK)
    return rc;
  cudaError_t e = cudaMemsetAsync(ctx->d_counters, 0, 16 * sizeof(unsigned long long), ctx->stream);
  if (e == cudaSuccess && ctx->d_tally)
    e = cudaMemsetAsync(ctx->d_tally, 0, ctx->n_cells * sizeof(unsigned long long), ctx->stream);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(ctx->stream);
  return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(e, "mcg_tally_reset");
}

extern "C" int mcg_tally_read(mcg_context *ctx, int64_t *h_q, double *h_f64)
{
  if (!ctx || !ctx->d_tally)
    return mcg_fail(MCG_ERR_STATE, "mcg_tally_read: no layers set");
  int rc = ensure_device(ctx);
  if (rc != MCG_OK)
    return rc;
  std::vector<int64_t> q(ctx->n_cells);
  cudaError_t e = cudaMemcpyAsync(q.data(), ctx->d_tally, ctx->n_cells * sizeof(int64_t),
                                  cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_tally_read");
  const double inv = std::ldexp(1.0, -ctx->log2_scale);
  for (int i = 0; i < ctx->n_cells; ++i) {
    if (h_q)
      h_q[i] = q[i];
    if (h_f64)
      h_f64[i] = (double)q[i] * inv;
  }
  return MCG_OK;
}

extern "C" int mcg_counters_read(mcg_context *ctx, mcg_counters *out)
{
  if (!ctx || !out)
    return mcg_fail(MCG_ERR_ARG, "mcg_counters_read: bad arguments");
  int rc = ensure_device(ctx);
  if (rc != MCG_OK)
    return rc;
  unsigned long long c[16];
  cudaError_t e = cudaMemcpyAsync(c, ctx->d_counters, sizeof(c), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_counters_read");
  out->histories = (int64_t)c[MCG_CNT_HIST];
  out->steps = (int64_t)c[MCG_CNT_STEPS];
  out->scatters = (int64_t)c[MCG_CNT_SCAT];
  out->leaked_left = (int64_t)c[MCG_CNT_LEFT];
  out->leaked_right = (int64_t)c[MCG_CNT_RIGHT];
  out->killed = (int64_t)c[MCG_CNT_KILL];
  out->w_left_q = (int64_t)c[MCG_CNT_WLEFT];
  out->w_right_q = (int64_t)c[MCG_CNT_WRIGHT];
  out->w_killed_q = (int64_t)c[MCG_CNT_WKILL];
  out->error_flags = (int64_t)c[MCG_CNT_ERR];
  return MCG_OK;
}

extern "C" int mcg_last_kernel_ms(mcg_context *ctx, float *ms)
{
  if (!ctx || !ms)
    return mcg_fail(MCG_ERR_ARG, "mcg_last_kernel_ms: bad arguments");
  *ms = ctx->last_ms;
  return MCG_OK;
}

extern "C" int mcg_set_launch(mcg_context *ctx, int32_t block, int32_t blocks_per_sm,
                              int32_t refill_steps)
{
  if (!ctx || block < 0 || block > 1024 || (block % 32) || blocks_per_sm < 0 || refill_steps < 0)
    return mcg_fail(MCG_ERR_ARG, "mcg_set_launch: bad arguments");
  ctx->block = block; /* 0: chosen per launch from the chain length */
  ctx->blocks_per_sm = blocks_per_sm;
  ctx->refill = refill_steps ? refill_steps : 8;
  return MCG_OK;
}

extern "C" int mcg_set_tally_mode(mcg_context *ctx, int32_t mode)
{
  if (!ctx || mode < 0 || mode > 2)
    return mcg_fail(MCG_ERR_ARG, "mcg_set_tally_mode: mode must be 0, 1 or 2");
  ctx->tally_mode = mode;
  return MCG_OK;
}

extern "C" int mcg_set_step_limit(mcg_context *ctx, int64_t max_steps)
{
  if (!ctx || max_steps < 1 || max_steps > 0xffffffffll)
    return mcg_fail(MCG_ERR_ARG, "mcg_set_step_limit: limit must be in [1, 2^32-1]");
  ctx->max_steps = (uint32_t)max_steps;
  return MCG_OK;
}

/* ------------------------------------------------------------ launches */
int mcg_track_launch(mcg_context *ctx, mcg_particle *d_particles, int64_t n, int32_t *d_results,
                     int64_t *d_steps, int64_t *d_scatters, const mcg_source *src, int64_t first)
{
  if (!ctx->d_tally)
    return mcg_fail(MCG_ERR_STATE, "no layers set (mcg_set_layers / mcg_set_slab)");
  if (n <= 0)
    return MCG_OK;
  const bool strict = ctx->mode == MCG_MODE_STRICT;
  if (strict && !ctx->libm_loaded) {
    int rc = mcg_load_libm(ctx);
    if (rc != MCG_OK)
      return rc;
  }
  mcg_track_params P;
  memset(&P, 0, sizeof(P));
  P.cells = strict ? ctx->d_cells_strict : ctx->d_cells_fast;
  P.n_cells = ctx->n_cells;
  P.cell_lo = ctx->cell_lo;
  P.min_w = ctx->min_w;
  P.q_log2 = ctx->log2_scale;
  P.particles = d_particles;
  P.results = d_results;
  P.steps = d_steps;
  P.scatters = d_scatters;
  P.n = n;
  P.first = first;
  if (src)
    P.src = *src;
  P.next = ctx->d_next;
  P.tally = ctx->d_tally;
  P.counters = ctx->d_counters;
  P.libm = ctx->libm;
  P.libm_tab = ctx->libm_tab;
  P.refill_steps = ctx->refill;
  P.chunk = 64;
  P.max_steps = ctx->max_steps;
  if (ctx->algorithm == MCG_ALGO_EVENT) {
    ctx->launches++;
    return mcg_event_run(ctx, P);
  }
  /* default shape: short chains keep one tally copy per warp in 256-thread
   * blocks; long chains share one copy per 1024-thread block */
  int block = ctx->block;
  if (block == 0)
    block = ((size_t)ctx->n_cells * 8 * 8 <= 24 * 1024) ? 256 : 1024;
  const int warps = block / 32;
  const size_t base = sizeof(mcg_libm_tab) + 16 * sizeof(unsigned long long);
  int tmode = ctx->tally_mode;
  /* one tally copy per warp while it stays small, else one per block */
  int copies = ((size_t)ctx->n_cells * 8 * warps <= 24 * 1024) ? warps : 1;
  if (tmode != MCG_TALLY_GLOBAL && base + (size_t)ctx->n_cells * 8 > (size_t)ctx->smem_optin)
    tmode = MCG_TALLY_GLOBAL; /* chain too long for a shared-memory copy */
  size_t smem = base + (tmode == MCG_TALLY_GLOBAL ? 0 : (size_t)ctx->n_cells * 8 * copies);
  P.tally_copies = copies;
  void (*kern)(mcg_track_params);
  if (strict && mcg_strict_thin(ctx))
    kern = tmode == MCG_TALLY_SMEM64 ? mcg_track_kernel<true, MCG_TALLY_SMEM64, true>
         : tmode == MCG_TALLY_SMEM32 ? mcg_track_kernel<true, MCG_TALLY_SMEM32, true>
                                     : mcg_track_kernel<true, MCG_TALLY_GLOBAL, true>;
  else if (strict)
    kern = tmode == MCG_TALLY_SMEM64 ? mcg_track_kernel<true, MCG_TALLY_SMEM64, false>
         : tmode == MCG_TALLY_SMEM32 ? mcg_track_kernel<true, MCG_TALLY_SMEM32, false>
                                     : mcg_track_kernel<true, MCG_TALLY_GLOBAL, false>;
  else if (ctx->thin) /* the fast step ignores THIN but for the loop's unrolling */
    kern = tmode == MCG_TALLY_SMEM64 ? mcg_track_kernel<false, MCG_TALLY_SMEM64, true>
         : tmode == MCG_TALLY_SMEM32 ? mcg_track_kernel<false, MCG_TALLY_SMEM32, true>
                                     : mcg_track_kernel<false, MCG_TALLY_GLOBAL, true>;
  else
    kern = tmode == MCG_TALLY_SMEM64 ? mcg_track_kernel<false, MCG_TALLY_SMEM64, false>
         : tmode == MCG_TALLY_SMEM32 ? mcg_track_kernel<false, MCG_TALLY_SMEM32, false>
                                     : mcg_track_kernel<false, MCG_TALLY_GLOBAL, false>;
  /* the limit is raised to the device's opt-in maximum, the same value on
   * every call, so launches of the same kernel from other host threads (other
   * contexts, the no-allocation entry point) cannot lower it under this one */
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       ctx->smem_optin);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "cudaFuncSetAttribute");
  int bps = ctx->blocks_per_sm;
  if (bps <= 0) {
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, block, smem);
    if (e != cudaSuccess)
      return mcg_cuda_fail(e, "occupancy");
    bps = std::max(bps, 1);
  }
  long long want_blocks = (n + block - 1) / block;
  int grid = (int)std::min<long long>((long long)ctx->sm_count * bps, std::max(want_blocks, 1LL));
  if ((e = cudaMemsetAsync(ctx->d_next, 0, sizeof(unsigned long long), ctx->stream)) != cudaSuccess)
    return mcg_cuda_fail(e, "cudaMemsetAsync");
  cudaEventRecord(ctx->ev0, ctx->stream);
  kern<<<grid, block, smem, ctx->stream>>>(P);
  e = cudaGetLastError();
  cudaEventRecord(ctx->ev1, ctx->stream);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "mcg_track_kernel launch");
  ctx->last_grid = grid;
  ctx->last_block = block;
  ctx->launches++;
  return MCG_OK;
}

int mcg_sync(mcg_context *ctx)
{
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "kernel execution");
  cudaEventElapsedTime(&ctx->last_ms, ctx->ev0, ctx->ev1);
  unsigned long long err = 0;
  e = cudaMemcpy(&err, ctx->d_counters + MCG_CNT_ERR, sizeof(err), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "read error flags");
  if (err)
    return mcg_fail(MCG_ERR_LIMIT, "a history exceeded the step limit (error flags %llx)", err);
  return MCG_OK;
}

static int ensure_scratch(mcg_context *ctx, int64_t n)
{
  if ((size_t)n <= ctx->scratch_cap)
    return MCG_OK;
  free_scratch(ctx);
  cudaError_t e;
  if ((e = cudaMalloc(&ctx->d_part, n * sizeof(mcg_particle))) != cudaSuccess ||
      (e = cudaMalloc(&ctx->d_res, n * sizeof(int32_t))) != cudaSuccess ||
      (e = cudaMalloc(&ctx->d_steps, n * sizeof(int64_t))) != cudaSuccess ||
      (e = cudaMalloc(&ctx->d_scat, n * sizeof(int64_t))) != cudaSuccess) {
    free_scratch(ctx);
    return mcg_cuda_fail(e, "cudaMalloc(particle buffers)");
  }
  ctx->scratch_cap = (size_t)n;
  return MCG_OK;
}

/* Device address of a page-locked (pinned or registered) host buffer, or
 * nullptr for pageable memory.  Pinned memory is mapped into the device's
 * address space (unified addressing), so the tracker can read and write it
 * in place: over NVLink-C2C on Grace machines, over PCIe elsewhere. */
static void *pinned_device_ptr(const void *h)
{
  if (!h)
    return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
    cudaGetLastError(); /* clear the (non-sticky) error of an unknown pointer */
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

extern "C" int mcg_simulate(mcg_context *ctx, mcg_particle *h_particles, int64_t n,
                            int32_t *h_results, int64_t *h_steps, int64_t *h_scatters)
{
  if (!ctx || n < 0 || (n > 0 && !h_particles))
    return mcg_fail(MCG_ERR_ARG, "mcg_simulate: bad arguments");
  if (n == 0)
    return MCG_OK;
  int rc = ensure_device(ctx);
  if (rc != MCG_OK)
    return rc;
  /* every buffer page-locked: one history reads and writes its 24-byte
   * particle once over ~1e2-1e4 steps, so the tracker works on the host
   * buffers in place instead of copying them through device memory */
  void *zp = pinned_device_ptr(h_particles);
  void *zr = pinned_device_ptr(h_results), *zs = pinned_device_ptr(h_steps);
  void *zc = pinned_device_ptr(h_scatters);
  if (zp && (!h_results || zr) && (!h_steps || zs) && (!h_scatters || zc)) {
    rc = mcg_track_launch(ctx, static_cast<mcg_particle *>(zp), n, static_cast<int32_t *>(zr),
                          static_cast<int64_t *>(zs), static_cast<int64_t *>(zc), nullptr, 0);
    return rc == MCG_OK ? mcg_sync(ctx) : rc;
  }
  rc = ensure_scratch(ctx, n);
  if (rc != MCG_OK)
    return rc;
  cudaError_t e = cudaMemcpyAsync(ctx->d_part, h_particles, n * sizeof(mcg_particle),
                                  cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "cudaMemcpyAsync(particles)");
  rc = mcg_track_launch(ctx, ctx->d_part, n, ctx->d_res, h_steps ? ctx->d_steps : nullptr,
                        h_scatters ? ctx->d_scat : nullptr, nullptr, 0);
  if (rc != MCG_OK)
    return rc;
  e = cudaMemcpyAsync(h_particles, ctx->d_part, n * sizeof(mcg_particle), cudaMemcpyDeviceToHost,
                      ctx->stream);
  if (e == cudaSuccess && h_results)
    e = cudaMemcpyAsync(h_results, ctx->d_res, n * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess && h_steps)
    e = cudaMemcpyAsync(h_steps, ctx->d_steps, n * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess && h_scatters)
    e = cudaMemcpyAsync(h_scatters, ctx->d_scat, n * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream);
  if (e != cudaSuccess)
    return mcg_cuda_fail(e, "cudaMemcpyAsync(results)");
  return mcg_sync(ctx);
}

extern "C" int mcg_simulate_device(mcg_context *ctx, mcg_particle *d_particles, int64_t n,
                                   int32_t *d_results, int64_t *d_steps, int64_t *d_scatters)
{
  if (!ctx || n < 0 || (n > 0 && !d_particles))
    return mcg_fail(MCG_ERR_ARG, "mcg_simulate_device: bad arguments");
  int rc = ensure_device(ctx);
  if (rc == MCG_OK)
    rc = mcg_track_launch(ctx, d_particles, n, d_results, d_steps, d_scatters, nullptr, 0);
  return rc == MCG_OK ? mcg_sync(ctx) : rc;
}

extern "C" int mcg_simulate_source(mcg_context *ctx, const mcg_source *src, int64_t first, int64_t n)
{
  if (!ctx || !src || n < 0 || first < 0 || src->seed_mode < 0 || src->seed_mode > 1 ||
      src->isotropic < 0 || src->isotropic > 2)
    return mcg_fail(MCG_ERR_ARG, "mcg_simulate_source: bad arguments");
  int rc = ensure_device(ctx);
  if (rc == MCG_OK)
    rc = mcg_track_launch(ctx, nullptr, n, nullptr, nullptr, nullptr, src, first);
  return rc == MCG_OK ? mcg_sync(ctx) : rc;
}

/* ------------------------------------------------------------ particle source */
__global__ void mcg_make_particles_kernel(mcg_source S, int64_t first, int64_t n, mcg_particle *out)
{
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    mcg_particle p;
    mcg_source_particle(S, first + i, p.seed, p.x, p.mu, p.wmc, p.index);
    out[i] = p;
  }
}

extern "C" int mcg_create_particles(mcg_context *ctx, const mcg_source *src, int64_t first,
                                    int64_t n, mcg_particle *h_out)
{
  if (!ctx || !src || n < 0 || first < 0 || (n > 0 && !h_out))
    return mcg_fail(MCG_ERR_ARG, "mcg_create_particles: bad arguments");
  if (n == 0)
    return MCG_OK;
  int rc = ensure_device(ctx);
  if (rc == MCG_OK)
    rc = ensure_scratch(ctx, n);
  if (rc != MCG_OK)
    return rc;
  int grid = (int)std::min<int64_t>((n + 255) / 256, (int64_t)ctx->sm_count * 8);
  mcg_make_particles_kernel<<<grid, 256, 0, ctx->stream>>>(*src, first, n, ctx->d_part);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h_out, ctx->d_part, n * sizeof(mcg_particle), cudaMemcpyDeviceToHost,
                        ctx->stream);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(ctx->stream);
  return e == cudaSuccess ? MCG_OK : mcg_cuda_fail(e, "mcg_create_particles");
}

/* ------------------------------------------------------------ cusimulate */
static thread_local mcg_context *g_cu_ctx = nullptr;

extern "C" int mcg_cusimulate(int n, mcg_particle *particles, const float *sigs,
                              const float *absorption_rates, float *weights_absorbed,
                              int min_index, int max_index, float dx)
{
  if (n < 0 || (n > 0 && !particles) || !sigs || !absorption_rates || !weights_absorbed ||
      max_index <= min_index)
    return mcg_fail(MCG_ERR_ARG, "cusimulate: bad arguments");
  int rc = MCG_OK;
  if (!g_cu_ctx) {
    int dev = 0;
    cudaGetDevice(&dev);
    rc = mcg_create(dev, MCG_MODE_STRICT, &g_cu_ctx);
    if (rc != MCG_OK)
      return rc;
  }
  const int m = max_index - min_index;
  /* the reference kernel has no weight cut: run until the particle leaves */
  rc = mcg_set_layers(g_cu_ctx, 1, &min_index, &m, &dx, sigs, absorption_rates, -INFINITY);
  if (rc == MCG_OK)
    rc = mcg_simulate(g_cu_ctx, particles, n, nullptr, nullptr, nullptr);
  if (rc != MCG_OK)
    return rc;
  std::vector<double> t(m);
  rc = mcg_tally_read(g_cu_ctx, nullptr, t.data());
  if (rc == MCG_OK)
    for (int j = 0; j < m; ++j)
      weights_absorbed[j] += (float)t[j];
  return rc;
}

extern "C" void cusimulate(int n, mcg_particle *particles, float const *const sigs,
                           float const *const absorption_rates, float *const weights_absorbed,
                           int min_index, int max_index, float dx)
{
  int rc = mcg_cusimulate(n, particles, sigs, absorption_rates, weights_absorbed, min_index,
                          max_index, dx);
  if (rc != MCG_OK) {
    fprintf(stderr, "cusimulate: %s\n", mcg_last_error());
    exit(rc);
  }
}
