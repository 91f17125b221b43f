/*
 * exact_libm.h - float-float evaluators of log and exp in binary32 that are
 * near-correctly-rounded and report how close the exact value lies to a
 * rounding midpoint.
 *
 * Why: the reference tracker (src/layer.cpp:137 `-log(h)`, src/layer.cpp:175
 * `expf(-sig_a * di)`) calls the host C library's logf/expf.  Those are not
 * correctly rounded: measured exhaustively they differ from the correctly
 * rounded result on about 2e5 inputs each, always by one unit in the last
 * place and always for inputs whose exact result lies near a midpoint.  The
 * strict GPU tracker must reproduce the host library bit for bit, so it:
 *   1. evaluates log here to ~2^-45 and exp to ~2^-37 relative accuracy
 *      (float-float), which equals the correctly rounded value except in
 *      rare hard cases;
 *   2. measures delta = distance of the float-float value from the nearest
 *      rounding midpoint, in units of the local float spacing (0 .. 0.5);
 *   3. if delta is at most the per-bucket threshold tau (computed by the
 *      exhaustive table generator from the host library), probes a hash table
 *      of the inputs where the host library's result differs from (1).
 *
 * The same source is compiled for the GPU by nvcc and for the host by gcc
 * (libm_tablegen.cpp), so the generator sees exactly the bits the GPU
 * computes.  Only IEEE-754 round-to-nearest +, -, *, fma and exact integer/bit
 * operations are used; on the device they are spelled with the __f*_rn
 * intrinsics so the compiler can neither contract nor reassociate them, and
 * host translation units that include this file are built with
 * -ffp-contract=off.
 *
 * Constants: libm_tables.inc, generated from the mathematics by
 * gen_libm_tables.py (see its docstring for the argument reductions).
 */
#ifndef MCG_EXACT_LIBM_H
#define MCG_EXACT_LIBM_H

#include <stdint.h>
#ifndef __CUDACC__
#include <math.h>
#include <string.h>
#endif

#if defined(__CUDACC__)
#define MCG_HD __host__ __device__ __forceinline__
#else
#define MCG_HD static inline
#endif

/* ---- exact arithmetic primitives (no contraction, round to nearest) ---- */
#if defined(__CUDA_ARCH__)
#define MCG_ADD(a, b) __fadd_rn((a), (b))
#define MCG_SUB(a, b) __fsub_rn((a), (b))
#define MCG_MUL(a, b) __fmul_rn((a), (b))
#define MCG_FMA(a, b, c) __fmaf_rn((a), (b), (c))
MCG_HD uint32_t mcg_f2u(float f) { return __float_as_uint(f); }
MCG_HD float mcg_u2f(uint32_t u) { return __uint_as_float(u); }
#else
#define MCG_ADD(a, b) ((a) + (b))
#define MCG_SUB(a, b) ((a) - (b))
#define MCG_MUL(a, b) ((a) * (b))
#define MCG_FMA(a, b, c) fmaf((a), (b), (c))
MCG_HD uint32_t mcg_f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
MCG_HD float mcg_u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
#endif

#include "libm_tables.inc"

/* Exact small-integer <-> float conversions through the 1.5 * 2^23 bias
 * (|k| < 2^22), on the FP32/INT pipes rather than the conversion unit.
 * mcg_rint_k returns RN-even(x) as an int, like rintf. */
#define MCG_MAGIC 12582912.0f /* 1.5 * 2^23, bits 0x4b400000 */
MCG_HD float mcg_int_to_float(int k) { return MCG_SUB(mcg_u2f(0x4b400000u + (uint32_t)k), MCG_MAGIC); }
MCG_HD int mcg_rint_k(float x) { return (int)(mcg_f2u(MCG_ADD(x, MCG_MAGIC)) - 0x4b400000u); }

/* Lookup tables of the evaluators.  Kernels stage one copy in shared memory
 * (lanes index it divergently) and pass its address. */
typedef struct mcg_libm_tab {
  float log_invc[MCG_LOG_NB];
  float log_lhi[MCG_LOG_NB];
  float log_llo[MCG_LOG_NB];
  float exp_thi[MCG_EXP_NT];
  float exp_tlo[MCG_EXP_NT];
} mcg_libm_tab;

/* Buckets for the per-bucket delta thresholds: sign, exponent and the top 4
 * mantissa bits of the INPUT. */
#define MCG_TAU_BUCKETS 8192
MCG_HD uint32_t mcg_tau_bucket(float x) { return mcg_f2u(x) >> 19; }

/* delta of a normalised float-float (yh, yl): distance of yh + yl from the
 * nearest rounding midpoint, in units of the float spacing on the side yl
 * points to.  yh must be a normal nonzero float with |yl| <= ulp(yh)/2. */
MCG_HD float mcg_midpoint_delta(float yh, float yl)
{
  uint32_t ub = mcg_f2u(yh);
  uint32_t eb = (ub >> 23) & 0xffu;
  /* 1/ulp(yh) = 2^(23 - (eb - 127)) = 2^(150 - eb) as a float. */
  int s = 150 - (int)eb;
  /* eb is in [1, 254]; 2^s is representable for s in [-126, 127].  The
   * callers' results have eb in [103, 254] (|log| >= 2^-24, exp >= 2^-26). */
  if (s > 127) s = 127;
  if (s < -126) s = -126;
  float inv_ulp = mcg_u2f((uint32_t)(s + 127) << 23);
  float v = MCG_MUL(fabsf(yl), inv_ulp);
  /* At a power of two the spacing below is half the spacing above. */
  if ((ub & 0x007fffffu) == 0u && ((mcg_f2u(yl) ^ ub) & 0x80000000u) && yl != 0.0f)
    v = MCG_MUL(v, 2.0f);
  return MCG_SUB(0.5f, v);
}

/* log(x) for finite x > 0.  Returns RN of the float-float value; *delta as
 * above.  x == 1 returns 0 with delta 0.5 (exact). */
MCG_HD float mcg_log_ff(float x, float *delta, const mcg_libm_tab *T)
{
  uint32_t u = mcg_f2u(x);
  int kadj = 0;
  if (u < 0x00800000u) { /* subnormal: scale by 2^23 (exact) */
    x = MCG_MUL(x, 8388608.0f);
    u = mcg_f2u(x);
    kadj = -23;
  }
  int e = (int)(u >> 23) - 127;
  uint32_t i = (u >> 16) & 127u;
  uint32_t sel = i >> 6; /* 1: mantissa >= 1.5, use m/2 and k+1 */
  float m = mcg_u2f((u & 0x007fffffu) | (0x3f800000u - (sel << 23)));
  int k = e + (int)sel + kadj;
  float invc = T->log_invc[i];
  float lhi = T->log_lhi[i];
  float llo = T->log_llo[i];
  float r = MCG_FMA(m, invc, -1.0f); /* exact: invc has 8 significant bits */
  float r2h = MCG_MUL(r, r);
  float r2l = MCG_FMA(r, r, -r2h);
  float P = MCG_FMA(r, MCG_FMA(r, MCG_FMA(r, MCG_LOG_P6, MCG_LOG_P5), MCG_LOG_P4), MCG_LOG_P3);
  float t3 = MCG_MUL(MCG_MUL(r2h, r), P);
  float hh = MCG_MUL(-0.5f, r2h);
  /* log1p(r) = s_hi + s_lo, Fast2Sum since |r| >= |r^2/2| */
  float s_hi = MCG_ADD(r, hh);
  float s_lo = MCG_ADD(MCG_SUB(r, s_hi), hh);
  s_lo = MCG_ADD(s_lo, MCG_FMA(-0.5f, r2l, t3));
  float kf = mcg_int_to_float(k);
  float kh = MCG_MUL(kf, MCG_LN2_HI);  /* exact */
  float km = MCG_MUL(kf, MCG_LN2_MID); /* exact */
  float kl = MCG_MUL(kf, MCG_LN2_LO);
  /* a = kh + lhi: Fast2Sum (|kh| >= 0.69 > |lhi|, or kh == 0) */
  float a = MCG_ADD(kh, lhi);
  float ae = MCG_ADD(MCG_SUB(kh, a), lhi);
  /* b = a + s_hi: TwoSum */
  float b = MCG_ADD(a, s_hi);
  float bv = MCG_SUB(b, a);
  float be = MCG_ADD(MCG_SUB(a, MCG_SUB(b, bv)), MCG_SUB(s_hi, bv));
  /* c = b + km: Fast2Sum (km == 0, or |b| > 0.25 > |km|) */
  float c = MCG_ADD(b, km);
  float ce = MCG_ADD(MCG_SUB(b, c), km);
  float lo = MCG_ADD(MCG_ADD(MCG_ADD(ae, be), MCG_ADD(ce, s_lo)), MCG_ADD(llo, kl));
  float yh = MCG_ADD(c, lo);
  float yl = MCG_ADD(MCG_SUB(c, yh), lo);
  *delta = (yh == 0.0f) ? 0.5f : mcg_midpoint_delta(yh, yl);
  return yh;
}

/* e^(rh + rl) for |rh| <= ln2/128, |rl| <= ulp(rh): (1 + rh) as an exact
 * float-float (Fast2Sum) plus rh^2 (1/2 + rh/6 + rh^2/24) + rl, within
 * 2^-38 relative; returns the rounded value, *yl the float-float remainder.
 * With rl = 0 (the small-argument path) the added rl changes nothing. */
MCG_HD float mcg_exp_small_form(float rh, float rl, float *yl)
{
  float p = MCG_FMA(rh, MCG_EXP_Q4, MCG_EXP_Q3);
  p = MCG_FMA(rh, p, 0.5f);
  const float r2 = MCG_MUL(MCG_MUL(rh, rh), p);
  const float s = MCG_ADD(1.0f, rh);
  const float se = MCG_SUB(rh, MCG_SUB(s, 1.0f));
  const float lo = MCG_ADD(MCG_ADD(se, r2), rl);
  const float yh = MCG_ADD(s, lo);
  *yl = MCG_ADD(MCG_SUB(s, yh), lo);
  return yh;
}

/* The small-argument form for rl = 0 without the addition of rl: the same
 * yh, and yl equal up to the sign of a zero (lo is at most a signed zero
 * apart, s + lo = s then, and (s - yh) + lo is +0 either way), so |yl| and
 * every test on it agree with mcg_exp_small_form(t, 0, yl). */
MCG_HD float mcg_exp_small_yl(float t, float *yl)
{
  float p = MCG_FMA(t, MCG_EXP_Q4, MCG_EXP_Q3);
  p = MCG_FMA(t, p, 0.5f);
  const float r2 = MCG_MUL(MCG_MUL(t, t), p);
  const float s = MCG_ADD(1.0f, t);
  const float se = MCG_SUB(t, MCG_SUB(s, 1.0f));
  const float lo = MCG_ADD(se, r2);
  const float yh = MCG_ADD(s, lo);
  *yl = MCG_ADD(MCG_SUB(s, yh), lo);
  return yh;
}

/* Midpoint distance of the small-argument path, in units of 2^-24, the float
 * spacing below 1 (every t < 0); above 1 the spacing is 2^-23 and this
 * measure is only a filter key, which the table generator, running this
 * same code, sets its thresholds by. */
MCG_HD float mcg_exp_small_delta(float yl)
{
  return MCG_SUB(0.5f, MCG_MUL(fabsf(yl), 16777216.0f));
}

/* exp(t), k = rint(t 64 / ln2) == 0: the small-argument path. */
MCG_HD float mcg_exp_ff_small(float t, float *delta)
{
  float yl;
  const float yh = mcg_exp_small_form(t, 0.0f, &yl);
  *delta = mcg_exp_small_delta(yl);
  return yh;
}

/* exp(t), any k: t = k ln2/64 + r (r as a float-float), e^r by the small
 * form, times 2^(j/64) (a float-float table entry, j = k mod 64), times
 * 2^((k - j)/64).  For k == 0 every step is exact or an exact identity (r
 * = t, rl = 0, table entry 1 + 0, scale 1) and the midpoint measure is the
 * small path's, so this path returns the small path's bits: the two are
 * interchangeable (kernels may choose the path per warp), which the GPU
 * tests check over every argument. */
MCG_HD float mcg_exp_ff_general(float t, int k, float *delta, const mcg_libm_tab *T)
{
  const float kf = mcg_int_to_float(k);
  const float p1 = MCG_MUL(kf, MCG_EXP_C1); /* exact */
  const float r1 = MCG_SUB(t, p1);           /* exact */
  const float p2 = MCG_MUL(kf, MCG_EXP_C2);
  const float p2e = MCG_FMA(kf, MCG_EXP_C2, -p2);
  /* r = r1 - p2 (TwoSum) - p2e - k*C3 */
  const float rh0 = MCG_SUB(r1, p2);
  const float bv = MCG_SUB(rh0, r1);
  const float re = MCG_SUB(MCG_SUB(r1, MCG_SUB(rh0, bv)), MCG_ADD(p2, bv));
  const float rl0 = MCG_SUB(MCG_SUB(re, p2e), MCG_MUL(kf, MCG_EXP_C3));
  const float rh = MCG_ADD(rh0, rl0);
  const float rl = MCG_ADD(MCG_SUB(rh0, rh), rl0);
  float el;
  const float eh = mcg_exp_small_form(rh, rl, &el); /* e^r = eh + el */
  const int j = k & 63;
  int q = (k - j) / 64; /* exact floor division: k - j is a multiple of 64 */
  const float thi = T->exp_thi[j];
  const float tlo = T->exp_tlo[j];
  /* (thi + tlo)(eh + el) = P + (Pe + thi el + tlo eh), renormalised */
  const float P = MCG_MUL(thi, eh);
  const float Pe = MCG_FMA(thi, eh, -P);
  const float lo = MCG_ADD(Pe, MCG_FMA(thi, el, MCG_MUL(tlo, eh)));
  float yh = MCG_ADD(P, lo);
  const float yl = MCG_ADD(MCG_SUB(P, yh), lo);
  *delta = k == 0 ? mcg_exp_small_delta(yl) : mcg_midpoint_delta(yh, yl);
  /* scale by 2^q, q in [-26, 128]; the product is exact unless it overflows */
  if (q > 127) { yh = MCG_MUL(yh, 2.0f); q -= 1; }
  return MCG_MUL(yh, mcg_u2f((uint32_t)(q + 127) << 23));
}

/* exp(t) for -17.5 <= t < 89 (other arguments give meaningless values,
 * and touch nothing outside T).  The path is chosen by the argument; in
 * translation units that define MCG_EXP_UNIFORM a warp whose lanes mix the
 * two takes the general path for all (identical bits, no divergence). */
MCG_HD float mcg_exp_ff_core(float t, float *delta, const mcg_libm_tab *T)
{
  const int k = mcg_rint_k(MCG_MUL(t, MCG_EXP_INV));
#if defined(__CUDA_ARCH__) && defined(MCG_EXP_UNIFORM)
  if (__all_sync(__activemask(), k == 0))
#else
  if (k == 0)
#endif
    return mcg_exp_ff_small(t, delta);
  return mcg_exp_ff_general(t, k, delta, T);
}

/* exp(t) for -17.5 <= t < 89.  Larger t returns +inf with delta 0.5. */
MCG_HD float mcg_exp_ff(float t, float *delta, const mcg_libm_tab *T)
{
  if (!(t < 89.0f)) { *delta = 0.5f; return mcg_u2f(0x7f800000u); }
  return mcg_exp_ff_core(t, delta, T);
}

/* |t| below this bound gives k = rint(RN(t * MCG_EXP_INV)) = 0
 * (0.0054 * 92.3325 = 0.4986 < 1/2), so mcg_exp_ff_small(t) returns the bits
 * of mcg_exp_ff_core(t) there. */
#define MCG_EXP_SMALL_T 0.0054f

/* Below this argument 1 - expf(t) rounds to exactly 1.0f whatever expf
 * returns (its result is below 2^-25); the table generator re-verifies this
 * against the host library for every float below the bound. */
#define MCG_EXP_ONE_BOUND (-17.5f)

#endif /* MCG_EXACT_LIBM_H */
