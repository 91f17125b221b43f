/*
 * libm_tablegen - build step of the strict tracker.
 *
 * The strict GPU tracker must return, for every logf/expf argument the
 * reference tracker can produce (src/layer.cpp:137 and :175), the very float
 * the host C library returns.  This program enumerates every such binary32
 * argument, evaluates the host library and the device evaluator of
 * exact_libm.h (compiled here for the host, bit-identical to the device), and
 * writes the arguments where the two differ, together with per-bucket
 * thresholds on the evaluator's midpoint distance, to a table file that the
 * library uploads to the GPU.
 *
 * Domains (the only arguments reachable from the tracker):
 *   logf: every float in (0, 1]   (h = RN(s) * 2^-63, s a 63-bit LCG state)
 *   expf: every float in [-17.5, 89).  Below -17.5 the tracker only uses
 *         1 - expf(t), which must round to 1.0f: verified here for every
 *         float below the bound (and -inf).  At or above 89, expf is +inf:
 *         verified here too.
 *
 * Usage: libm_tablegen <output file>
 *        libm_tablegen --fingerprint-matches <table>   (exit 0 if current)
 * Build: g++ -O2 -std=c++17 -ffp-contract=off -fopenmp (no -ffast-math).
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <gnu/libc-version.h>
#include <omp.h>

#include "exact_libm.h"
#include "libm_file.h"

static const mcg_libm_tab kTab = MCG_LIBM_TAB_INIT;

struct Exc {
  uint32_t key, val;
  float delta;
};

static float asf(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t asu(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

int main(int argc, char **argv)
{
  if (argc == 3 && strcmp(argv[1], "--fingerprint-matches") == 0) {
    mcg_libm_file h;
    FILE *fp = fopen(argv[2], "rb");
    bool ok = fp && fread(&h, sizeof(h), 1, fp) == 1 && memcmp(h.magic, MCG_LIBM_MAGIC, 8) == 0 &&
              h.fingerprint == mcg_libm_fingerprint(&kTab);
    if (fp)
      fclose(fp);
    return ok ? 0 : 1;
  }
  if (argc != 2) {
    fprintf(stderr, "usage: %s <output file>\n", argv[0]);
    return 2;
  }
  const int nt = omp_get_max_threads();
  std::vector<std::vector<Exc>> log_exc(nt), exp_exc(nt);
  long long bad_low = 0, bad_high = 0, bad_path = 0;

  /* ---- logf on (0, 1] ---- */
  const uint32_t log_hi = 0x3f800000u;
#pragma omp parallel for schedule(dynamic, 1 << 16)
  for (long long ui = 1; ui <= (long long)log_hi; ++ui) {
    float x = asf((uint32_t)ui);
    float d;
    float y = mcg_log_ff(x, &d, &kTab);
    float g = logf(x);
    if (asu(y) != asu(g))
      log_exc[omp_get_thread_num()].push_back({(uint32_t)ui, asu(g), d});
  }

  /* ---- expf: all floats; [-17.5, 89) tabulated, the rest verified ---- */
#pragma omp parallel for schedule(dynamic, 1 << 16) reduction(+ : bad_low, bad_high, bad_path)
  for (long long ui = 0; ui <= 0xffffffffll; ++ui) {
    float t = asf((uint32_t)ui);
    if (std::isnan(t))
      continue;
    float g = expf(t);
    if (t < MCG_EXP_ONE_BOUND) {
      volatile float one_m = 1.0f - g;
      if (one_m != 1.0f)
        bad_low++;
      continue;
    }
    if (!(t < 89.0f)) {
      if (!(std::isinf(g) && g > 0))
        bad_high++;
      continue;
    }
    float d;
    float y = mcg_exp_ff(t, &d, &kTab);
    if (asu(y) != asu(g))
      exp_exc[omp_get_thread_num()].push_back({(uint32_t)ui, asu(g), d});
    /* the general path must reproduce the small-argument path (value and
     * midpoint measure) wherever the latter applies */
    if (mcg_rint_k(MCG_MUL(t, MCG_EXP_INV)) == 0) {
      float d2;
      float y2 = mcg_exp_ff_general(t, 0, &d2, &kTab);
      if (asu(y2) != asu(y) || asu(d2) != asu(d))
        bad_path++;
    }
  }
  if (bad_path) {
    fprintf(stderr, "libm_tablegen: the general exp path differs from the small-argument "
                    "path on %lld arguments\n", bad_path);
    return 1;
  }
  if (bad_low || bad_high) {
    fprintf(stderr, "libm_tablegen: host expf violates the tracker's assumptions "
                    "(%lld below %g, %lld at/above 89)\n",
            bad_low, (double)MCG_EXP_ONE_BOUND, bad_high);
    return 1;
  }

  mcg_libm_file f;
  memset(&f, 0, sizeof(f));
  memcpy(f.magic, MCG_LIBM_MAGIC, 8);
  snprintf(f.libc_version, sizeof(f.libc_version), "glibc %s", gnu_get_libc_version());
  f.fingerprint = mcg_libm_fingerprint(&kTab);
  std::vector<uint32_t> pairs[2];
  for (int fn = 0; fn < 2; ++fn) {
    std::vector<Exc> all;
    for (auto &v : (fn == 0 ? log_exc : exp_exc))
      all.insert(all.end(), v.begin(), v.end());
    std::sort(all.begin(), all.end(), [](const Exc &a, const Exc &b) { return a.key < b.key; });
    float *tau = fn == 0 ? f.tau_log : f.tau_exp;
    for (int b = 0; b < MCG_TAU_BUCKETS; ++b)
      tau[b] = -1.0f;
    float dmax = 0.0f;
    for (const Exc &e : all) {
      uint32_t b = e.key >> 19;
      tau[b] = std::max(tau[b], e.delta);
      dmax = std::max(dmax, e.delta);
      pairs[fn].push_back(e.key);
      pairs[fn].push_back(e.val);
    }
    (fn == 0 ? f.n_log : f.n_exp) = (uint32_t)all.size();
    printf("%s: %zu exceptions, max midpoint distance %.4f ulp\n", fn == 0 ? "logf" : "expf",
           all.size(), (double)dmax);
  }
  /* the host logf's largest relative error on (0, 1), against the double
   * log (itself within 1e-16): the strict tracker's certain-crossing test
   * assumes at most 2^-22 */
  {
    double worst = 0.0;
#pragma omp parallel for reduction(max : worst) schedule(dynamic, 1 << 16)
    for (long long ui = 1; ui < (long long)log_hi; ++ui) {
      float x = asf((uint32_t)ui);
      double g = log((double)x);
      double rel = fabs((double)logf(x) - g) / fabs(g);
      if (rel > worst)
        worst = rel;
    }
    f.logf_relerr = (float)worst;
    printf("logf: max relative error on (0, 1) %.3e\n", worst);
  }
  /* fraction of uniformly distributed h in (0,1) whose logf passes the filter */
  {
    double pass = 0.0;
#pragma omp parallel for reduction(+ : pass) schedule(dynamic, 1 << 16)
    for (long long ui = 1; ui < (long long)log_hi; ++ui) {
      float x = asf((uint32_t)ui);
      float d;
      (void)mcg_log_ff(x, &d, &kTab);
      if (d <= f.tau_log[ui >> 19])
        pass += (double)(asf((uint32_t)ui + 1) - x);
    }
    printf("logf: probe rate for uniform arguments %.4f\n", pass);
  }

  FILE *fp = fopen(argv[1], "wb");
  if (!fp) {
    perror(argv[1]);
    return 1;
  }
  bool ok = fwrite(&f, sizeof(f), 1, fp) == 1;
  for (int fn = 0; fn < 2; ++fn)
    ok = ok && (pairs[fn].empty() ||
                fwrite(pairs[fn].data(), 4, pairs[fn].size(), fp) == pairs[fn].size());
  ok = (fclose(fp) == 0) && ok;
  if (!ok) {
    fprintf(stderr, "libm_tablegen: write failed\n");
    return 1;
  }
  printf("wrote %s (%s, fingerprint %016llx)\n", argv[1], f.libc_version,
         (unsigned long long)f.fingerprint);
  return 0;
}
