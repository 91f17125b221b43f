/*
 * mcg_device.cuh - device building blocks of the trackers: the reference's
 * LCG (src/random.cpp:12-16), the strict libm with its host-libm exception
 * tables, the fast approximations, and fixed-point tally conversion.
 */
#ifndef MCG_DEVICE_CUH
#define MCG_DEVICE_CUH

#include <cstdint>
#include <cfloat>
#include "exact_libm.h"

#define MCG_EPS 1e-4f              /* EPS_PRECISION, include/types/types.hpp:15 */
#define MCG_MAXREAL FLT_MAX        /* MAXREAL, include/types/types.hpp:14 */
#define MCG_RNG_G 6364136223846793005ull
#define MCG_RNG_C 1442695040888963407ull
#define MCG_RNGS_G 5177284530976225183ull
#define MCG_RNGS_C 2096348467109453893ull
#define MCG_MASK63 0x7fffffffffffffffull
#define MCG_HASH_EMPTY 0xffffffffu

/* Host-libm exception table as seen by kernels (device pointers). */
struct mcg_libm_dev {
  const float *tau_log;  /* [MCG_TAU_BUCKETS], -1 where no exception */
  const float *tau_exp;
  const uint2 *hash_log; /* open addressing, key = argument bits */
  const uint2 *hash_exp;
  uint32_t mask_log, mask_exp;
  int32_t probes_log, probes_exp; /* longest probe sequence + 1 */
  float tau_log_max, tau_exp_max;
};

/* RN((float)s) * 2^-63 for s < 2^63 with integer operations only (the
 * alternative to the hardware conversion, see mcg_rnd_real).  Round to
 * nearest, ties to even, as the reference's (float)seed (src/random.cpp:15). */
__device__ __forceinline__ float mcg_u63_unit(uint64_t s)
{
  if (s == 0)
    return 0.0f;
  const uint32_t hi = (uint32_t)(s >> 32), lo = (uint32_t)s;
  const int lz = hi ? __clz(hi) : 32 + __clz(lo);
  const uint64_t m = s << lz; /* bit 63 set */
  const uint32_t mh = (uint32_t)(m >> 32), ml = (uint32_t)m;
  const uint32_t mant = mh >> 8, low8 = mh & 0xffu;
  const uint32_t up = (low8 > 0x80u) | ((low8 == 0x80u) & ((ml != 0u) | (mant & 1u)));
  /* value = s * 2^-63 has biased exponent 127 - lz; mant carries the
   * implicit bit, and a rounding carry bumps the exponent */
  return __uint_as_float(((uint32_t)(126 - lz) << 23) + mant + up);
}

/* The reference's LCG step s <- (G s + C) mod 2^63 (src/random.cpp:14). */
__device__ __forceinline__ void mcg_lcg_next(uint64_t &s)
{
  s = (MCG_RNG_G * s + MCG_RNG_C) & MCG_MASK63;
}

/* rnd_real's value of a state s < 2^63: RN((float)s) * 2^-63
 * (src/random.cpp:15).  The hardware u64 -> f32 conversion issues on the
 * FP64 pipe (about 6e11 conversions/s per GB300), so the trackers call this
 * only where the float value itself is needed (scatters, near-ties, the
 * source's directions); the certain-crossing test compares the state's top
 * bits as an integer instead (mcg_cross_threshold).  MCG_INT_CONVERSIONS
 * selects the integer version (same bits). */
__device__ __forceinline__ float mcg_unit_of(uint64_t s)
{
#ifdef MCG_INT_CONVERSIONS
  return mcg_u63_unit(s);
#else
  return __fmul_rn(__ull2float_rn(s), 0x1p-63f);
#endif
}

/* rnd_real: s <- (G s + C) mod 2^63; h = RN((float)s) * 2^-63. */
__device__ __forceinline__ float mcg_rnd_real(uint64_t &s)
{
  mcg_lcg_next(s);
  return mcg_unit_of(s);
}

/* Fast arithmetic's uniform for directions: the same LCG step, then the
 * state's top 23 bits k as the midpoint (k + 1/2) 2^-23 of their interval
 * (two integer/float operations instead of an exact 64-bit rounding).  The
 * subtraction from [1, 2) of 1 - 2^-24 is exact (Sterbenz).  The midpoint
 * makes mu = 2h - 1 symmetric about 0 and h never 0.  (Flight samples use
 * mcg_flight_u, at 2^-32 resolution.) */
__device__ __forceinline__ float mcg_rnd_real_fast(uint64_t &s)
{
  mcg_lcg_next(s);
  return __fsub_rn(__uint_as_float(0x3f800000u | (uint32_t)(s >> 40)), 0x1.fffffep-1f);
}

/* RN(1 / mu) of a flight, 0 when |mu| <= EPS (the reference then uses
 * d_edge = MAXREAL, src/layer.cpp:159). */
__device__ __forceinline__ float mcg_flight_rcp(float mu)
{
  return (mu < -MCG_EPS || MCG_EPS < mu) ? __frcp_rn(mu) : 0.0f;
}

/* RN(a / b) from y = RN(1 / b): q = RN(a y), r = a - b q (exact by fma),
 * q + r y rounded once.  Equal to the IEEE quotient for every pair of
 * significands (checked exhaustively, all 2^46 pairs, by the GPU tests
 * through mcg_verify_division); each operation commutes with scaling a and
 * b by powers of two while no intermediate leaves the normal range, which
 * the caller guarantees by |a| >= 2^-100, 2^-100 <= |b| <= 2^100. */
__device__ __forceinline__ float mcg_div_by_rcp(float a, float b, float y)
{
  const float q = __fmul_rn(a, y);
  return __fmaf_rn(__fmaf_rn(-b, q, a), y, q);
}

/* Hardware 2^x (one MUFU operation; subnormal results flush to zero). */
__device__ __forceinline__ float mcg_ex2_approx(float x)
{
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

/* Certain-crossing test of the strict tracker.  The reference samples
 * h = RN((float)s) 2^-63, di = RN(-logf(h) / sig_i) and crosses when
 * !(di < de).  The tracker first tests, on the state s itself,
 *     floor(s / 2^32) < B,   B = trunc(RN(E * K)),
 *     E = ex2(RN(RN(sig_i de) * -log2(e))),  K = 2^31 (1 - m), m = 2^-14,
 * with one MUFU operation and one 32-bit conversion (no 64-bit one), and
 * only evaluates h and the exact logarithm when the test fails.
 *
 * Why the test implies the crossing (T = sig_i de exactly, u = 2^-24):
 *  - s < (floor(s / 2^32) + 1) 2^32 <= B 2^32 <= E (1 - m)(1 + u) 2^63, and
 *    RN is monotonic, so h <= E (1 - m)(1 + u)^2;
 *  - the two roundings and RN(log2 e) give an exponent T log2(e) (1 + eps)
 *    with |eps| <= 3.01 u, so 2^exponent lies within a factor
 *    exp(+-T |eps|) of e^-T;
 *  - ex2.approx is at most 2^-20 above 2^x (exhaustively checked over every
 *    argument the test can see by the GPU tests);
 *  - h >= 2^-63 when nonzero, so the test passing forces T < 44;
 *  - hence -ln h > T + m - 2^-20 - 2u - m^2 - 44 |eps|, and with the host
 *    logf within rho = 2^-22 relative of ln (verified exhaustively when the
 *    exception table is built):
 *    -logf(h) >= -ln(h) (1 - rho) > T + m - 2^-20 - 2u - m^2 - 44 (|eps| + rho) > T
 *    (m = 6.1e-5 against 2.0e-5 for the rest), so the exact quotient
 *    -logf(h) / sig_i is at least de and its rounding, RN being monotonic
 *    and de a float, is too;
 *  - h == 0 gives -logf(0) = inf, a crossing for the reference as well;
 *  - sig_i <= EPS: the reference crosses whatever h is (di = MAXREAL), so
 *    the test may pass there too; sig_i or de NaN or infinite gives E NaN or
 *    0 and B = 0 (the conversion takes NaN to 0), which fails.
 * A false result only costs the exact evaluation: the exact path decides
 * every case the test does not settle (about 2e-5 of crossings). */
#define MCG_LOG2E_F 1.44269502f
#define MCG_CROSS_FACTOR 0.99993896484375f /* 1 - 2^-14 */
#define MCG_CROSS_SCALE 2147352576.0f      /* 2^31 (1 - 2^-14) = 2^31 - 2^17, exact */
#define MCG_LOGF_RELERR_MAX 0x1p-22f       /* rho above, checked at table load */

/* B of the certain-crossing test for a flight of length de in a cell of
 * interaction cross section sig_i (the truncating conversion saturates: B is
 * 0 for NaN and 2^32 - 1 above the range, where s < 2^63 always passes). */
__device__ __forceinline__ uint32_t mcg_cross_threshold(float sig_i, float de)
{
  const float e = mcg_ex2_approx(__fmul_rn(__fmul_rn(sig_i, de), -MCG_LOG2E_F));
  return __float2uint_rz(__fmul_rn(e, MCG_CROSS_SCALE));
}

/* The state's top 31 bits, floor(s / 2^32), compared against B. */
__device__ __forceinline__ uint32_t mcg_state_hi(uint64_t s)
{
  return (uint32_t)(s >> 32);
}

__device__ __forceinline__ uint64_t mcg_rnd_seed(uint64_t &s)
{
  s = (MCG_RNGS_G * s + MCG_RNGS_C) & MCG_MASK63;
  return s;
}

/* State after n steps of the seed-chain (chain=1) or real (chain=0) LCG. */
__device__ __forceinline__ uint64_t mcg_lcg_skip(uint64_t seed, uint64_t n, int chain)
{
  uint64_t a = chain ? MCG_RNGS_G : MCG_RNG_G, c = chain ? MCG_RNGS_C : MCG_RNG_C;
  uint64_t A = 1, C = 0;
  while (n) {
    if (n & 1) {
      A = A * a;
      C = C * a + c;
    }
    c = c * a + c;
    a = a * a;
    n >>= 1;
  }
  return (A * seed + C) & MCG_MASK63;
}

__device__ __forceinline__ uint32_t mcg_hash_slot(uint32_t key, uint32_t mask)
{
  return (key * 0x9E3779B1u) & mask;
}

/* Bounded linear probe; returns true and the value if key is present. */
__device__ __forceinline__ bool mcg_hash_find(const uint2 *tab, uint32_t mask, int probes,
                                              uint32_t key, uint32_t &val)
{
  uint32_t slot = mcg_hash_slot(key, mask);
  for (int p = 0; p < probes; ++p) {
    uint2 e = __ldg(tab + slot);
    if (e.x == key) {
      val = e.y;
      return true;
    }
    if (e.x == MCG_HASH_EMPTY)
      return false;
    slot = (slot + 1) & mask;
  }
  return false;
}

/* logf(x) bit-identical to the host C library, for x in (0, 1]; x == 0 gives
 * -inf as the C library. */
__device__ __forceinline__ float mcg_logf_strict(float x, const mcg_libm_tab *T,
                                                 const mcg_libm_dev &L)
{
  if (x == 0.0f)
    return -INFINITY;
  float d;
  float y = mcg_log_ff(x, &d, T);
  if (d <= L.tau_log_max) {
    uint32_t key = __float_as_uint(x);
    if (d <= __ldg(L.tau_log + (key >> 19))) {
      uint32_t v;
      if (mcg_hash_find(L.hash_log, L.mask_log, L.probes_log, key, v))
        y = __uint_as_float(v);
    }
  }
  return y;
}

/* 1 - expf(t) with expf bit-identical to the host C library. */
__device__ __forceinline__ float mcg_one_minus_expf_strict(float t, const mcg_libm_tab *T,
                                                           const mcg_libm_dev &L)
{
  if (t < MCG_EXP_ONE_BOUND)
    return 1.0f;
  float d;
  float y = mcg_exp_ff(t, &d, T);
  if (d <= L.tau_exp_max) {
    uint32_t key = __float_as_uint(t);
    if (d <= __ldg(L.tau_exp + (key >> 19))) {
      uint32_t v;
      if (mcg_hash_find(L.hash_exp, L.mask_exp, L.probes_exp, key, v))
        y = __uint_as_float(v);
    }
  }
  return __fsub_rn(1.0f, y);
}

/* The exception lookup of expf: y, d from mcg_exp_ff (either path). */
__device__ __forceinline__ float mcg_exp_fixup(float t, float y, float d, const mcg_libm_dev &L)
{
  if (d <= L.tau_exp_max) {
    uint32_t key = __float_as_uint(t);
    if (d <= __ldg(L.tau_exp + (key >> 19))) {
      uint32_t v;
      if (mcg_hash_find(L.hash_exp, L.mask_exp, L.probes_exp, key, v))
        y = __uint_as_float(v);
    }
  }
  return y;
}

__device__ __forceinline__ float mcg_expf_strict(float t, const mcg_libm_tab *T,
                                                 const mcg_libm_dev &L)
{
  float d;
  float y = mcg_exp_ff(t, &d, T);
  if (d <= L.tau_exp_max) {
    uint32_t key = __float_as_uint(t);
    if (d <= __ldg(L.tau_exp + (key >> 19))) {
      uint32_t v;
      if (mcg_hash_find(L.hash_exp, L.mask_exp, L.probes_exp, key, v))
        y = __uint_as_float(v);
    }
  }
  return y;
}

/* The fast arithmetic's flight sample, drawn from the state s (already
 * advanced) at 2^-32 resolution: t = the state's top 32 bits,
 * h = (t + 1/2) 2^-32 and u = 1 - h = (~t + 1/2) 2^-32 (exact for u < 2^-9,
 * within 2^-24 relative above).  A thin cell's collision probability per
 * crossing is ~1e-4 (10,000-cell slab), decided by u within ~1e-4 of 0, so
 * u must be fine-grained there: on a 2^-23 grid it shifts each cell's
 * collision probability by up to half a grid step (3e-4 relative rms per
 * cell against the reference's 2^-24 grid), a 2^-32 grid by ~1e-6. */
__device__ __forceinline__ float mcg_flight_u(uint64_t s)
{
  return __fmaf_rn(__uint2float_rn(~(uint32_t)(s >> 31)), 0x1p-32f, 0x1p-33f);
}

/* log2(h) of that sample, for the distance of a collision: near 1
 * (u < 2^-8) the series -ln(1 - u) = u (1 + u/2 + u^2/3) (truncation below
 * 2^-26 relative); elsewhere the hardware log2 of h computed from t
 * directly (so h keeps its relative precision when it is small), documented
 * to an absolute error of 2^-22 on [0.5, 2], which near 1 would be a
 * relative error of a few 1e-4. */
__device__ __forceinline__ float mcg_flight_log2(uint64_t s)
{
  const uint32_t t = (uint32_t)(s >> 31);
  const float u = __fmaf_rn(__uint2float_rn(~t), 0x1p-32f, 0x1p-33f);
  float p = fmaf(u, MCG_LOG2E_F * (1.0f / 3.0f), MCG_LOG2E_F * 0.5f);
  p = fmaf(u, p, MCG_LOG2E_F);
  const float near1 = -u * p;
  return u < 0x1p-8f ? near1 : __log2f(__fmaf_rn(__uint2float_rn(t), 0x1p-32f, 0x1p-33f));
}

/* 1 - e^t for |t| < 2^-7: -t (1 + t/2 + t^2/6), truncation below
 * |t|^3/24 < 2^-25.5 relative, under the rounding of the float result. */
__device__ __forceinline__ float mcg_one_minus_exp_small(float t)
{
  float p = fmaf(t, 1.0f / 6.0f, 0.5f);
  p = fmaf(t, p, 1.0f);
  return -t * p;
}

/* Fast build: 1 - e^t for t <= 0 to a few ulp without cancellation. */
__device__ __forceinline__ float mcg_one_minus_exp_fast(float t)
{
  if (t > -0.25f) {
    /* -expm1(t) = -t (1 + t/2 + t^2/6 + ... + t^6/5040) */
    float p = fmaf(t, 1.0f / 5040.0f, 1.0f / 720.0f);
    p = fmaf(t, p, 1.0f / 120.0f);
    p = fmaf(t, p, 1.0f / 24.0f);
    p = fmaf(t, p, 1.0f / 6.0f);
    p = fmaf(t, p, 0.5f);
    p = fmaf(t, p, 1.0f);
    return -t * p;
  }
  return 1.0f - __expf(t);
}

/* Fixed-point deposit llrint(dw * 2^S), ties to even.  By default the
 * hardware conversion; with MCG_INT_CONVERSIONS the integer version below
 * (identical results).  Requires |dw| * 2^S < 2^63. */
__device__ __forceinline__ long long mcg_to_fixed(float dw, int S)
{
#ifndef MCG_INT_CONVERSIONS
  /* hardware conversion on the FP64 pipe (see mcg_rnd_real); dw * 2^S is
   * exact, and |dw| 2^S < 2^63 is the tally's range */
  return __float2ll_rn(__fmul_rn(dw, __int_as_float((127 + S) << 23)));
#endif
  const uint32_t u = __float_as_uint(dw);
  const int e = (int)((u >> 23) & 0xffu);
  const uint32_t mant = (u & 0x007fffffu) | 0x00800000u; /* dw = mant * 2^(e-150) */
  const int sh = e - 150 + S;
  uint64_t q;
  if (e == 0) {
    q = 0; /* zero or subnormal: |dw| 2^S < 2^-64 */
  } else if (sh > 38) {
    q = 0x3fffffffffffffffull; /* beyond the tally's range (or inf): saturate */
  } else if (sh >= 0) {
    q = (uint64_t)mant << sh;
  } else if (sh >= -24) {
    const int r = -sh;
    const uint32_t qi = mant >> r, rem = mant & ((1u << r) - 1u), half = 1u << (r - 1);
    q = qi + ((rem > half) | ((rem == half) & (qi & 1u)));
  } else {
    q = 0; /* below one half unit */
  }
  return (u >> 31) ? -(long long)q : (long long)q;
}

/* The scale 2^S as a float (0 <= S <= 62). */
__device__ __forceinline__ float mcg_fixed_scale(int S)
{
  return __int_as_float((127 + S) << 23);
}

__device__ __forceinline__ unsigned lanemask_lt()
{
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

#endif
