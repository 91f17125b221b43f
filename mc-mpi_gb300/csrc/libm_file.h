/*
 * libm_file.h - on-disk layout of the host-libm exception table written by
 * libm_tablegen and read by the library when a strict context is created.
 *
 *   mcg_libm_file header
 *   uint32_t log_pairs[2 * n_log]   (argument bits, host logf result bits)
 *   uint32_t exp_pairs[2 * n_exp]   (argument bits, host expf result bits)
 *
 * The fingerprint hashes the host library's logf/expf, and the float-float
 * evaluators of exact_libm.h (value and midpoint distance), on a fixed set
 * of arguments; the loader recomputes it, so a table made against another C
 * library (another machine) or by another version of the evaluators is
 * refused instead of silently used.  Host-only header; include exact_libm.h
 * first.
 */
#ifndef MCG_LIBM_FILE_H
#define MCG_LIBM_FILE_H

#include <math.h>
#include <stdint.h>
#include <string.h>

#define MCG_LIBM_MAGIC "MCGLIBM3"
#ifndef MCG_TAU_BUCKETS
#define MCG_TAU_BUCKETS 8192
#endif

typedef struct mcg_libm_file {
  char magic[8];
  char libc_version[56];
  uint64_t fingerprint;
  uint32_t n_log, n_exp;
  float logf_relerr; /* max |logf(x) - ln x| / |ln x| over floats x in (0, 1) */
  uint32_t reserved;
  float tau_log[MCG_TAU_BUCKETS];
  float tau_exp[MCG_TAU_BUCKETS];
} mcg_libm_file;

static inline uint64_t mcg_fnv_word(uint64_t h, float v)
{
  uint32_t u;
  memcpy(&u, &v, 4);
  for (int b = 0; b < 4; ++b) {
    h ^= (u >> (8 * b)) & 0xffu;
    h *= 1099511628211ull;
  }
  return h;
}

/* FNV-1a over the bits of logf/expf and of the evaluators at 8192
 * arguments spread over both domains by a 32-bit LCG (the exp arguments
 * cover both evaluator paths and both signs). */
static inline uint64_t mcg_libm_fingerprint(const mcg_libm_tab *T)
{
  uint64_t h = 1469598103934665603ull;
  uint32_t s = 12345u;
  for (int i = 0; i < 8192; ++i) {
    s = s * 1664525u + 1013904223u;
    uint32_t ux = (s >> 2) % 0x3f800000u + 1u; /* (0, 1] */
    float x, d, t = 0.0f;
    memcpy(&x, &ux, 4);
    if (i & 1)
      t = (i & 2) ? -x * 17.0f : (i & 4) ? x * 0.005f : -x * 0.005f;
    h = mcg_fnv_word(h, (i & 1) ? expf(t) : logf(x));
    h = mcg_fnv_word(h, (i & 1) ? mcg_exp_ff(t, &d, T) : mcg_log_ff(x, &d, T));
    h = mcg_fnv_word(h, d);
  }
  return h;
}

#endif
