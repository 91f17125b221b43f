/*
 * mcg_track.cuh - the history-based tracker.
 *
 * One lane carries one particle history at a time through the whole chain of
 * layers (a sub-domain crossing is just the next cell's parameters, so the
 * hand-over between sub-domains costs nothing).  The grid is persistent:
 * every warp takes chunks of history indices from a global counter and
 * refills finished lanes from its chunk every `refill_steps` steps, so warps
 * stay full however uneven the history lengths are.  Deposits go to a
 * shared-memory 64-bit fixed-point histogram (one copy per block, or one per
 * warp when the chain is short) and are added to the global tally once per
 * block at the end; the sums are exact, hence order-independent.
 *
 * The step follows Layer::particle_step (src/layer.cpp:123-190) and the loop
 * Layer::simulate_particle (src/layer.cpp:192-218).
 */
#ifndef MCG_TRACK_CUH
#define MCG_TRACK_CUH

#include "mcg_device.cuh"
#include "mcgb300.h"

/* Per-cell step parameters.  strict: {sig_a, sig_i, edge_lo, edge_hi}
 * fast: {sig_a, sig_i (0 when sig_i <= EPS), edge_lo, edge_hi}
 * edge_lo = (float)i * dx_layer, edge_hi = (float)(i+1) * dx_layer with the
 * GLOBAL cell index i and the cell's own layer spacing (src/layer.cpp:146,150). */
struct mcg_track_params {
  const float4 *cells;
  int32_t n_cells, cell_lo;
  float min_w;
  int32_t q_log2;
  mcg_particle *particles; /* NULL: source mode */
  int32_t *results;
  int64_t *steps, *scatters;
  int64_t n, first;
  mcg_source src;
  unsigned long long *next;  /* work counter, starts at 0 */
  unsigned long long *tally; /* [n_cells] fixed point */
  unsigned long long *counters; /* mcg_counters fields */
  mcg_libm_dev libm;
  const mcg_libm_tab *libm_tab;
  int32_t refill_steps;
  int32_t tally_copies; /* 1 or warps per block */
  int32_t chunk;        /* histories per warp grab (multiple of 32) */
  uint32_t max_steps;
};

/* Tally accumulation: shared-memory 64-bit atomics, shared-memory 32-bit
 * halves with an explicit carry, or 64-bit atomics straight to the global
 * tally (no shared memory, higher occupancy). */
enum { MCG_TALLY_SMEM64 = 0, MCG_TALLY_SMEM32 = 1, MCG_TALLY_GLOBAL = 2 };

template <int TALLY>
__device__ __forceinline__ void mcg_tally_add(unsigned long long *t, long long q)
{
  if (TALLY == MCG_TALLY_SMEM32) {
    /* exact 64-bit sum from 32-bit atomics: a carry out of the low word is
     * detected by the adder that caused it and added to the high word */
    const uint64_t v = (uint64_t)q;
    const uint32_t lo = (uint32_t)v, hi = (uint32_t)(v >> 32);
    unsigned *w = reinterpret_cast<unsigned *>(t);
    const uint32_t old = atomicAdd(w, lo);
    const uint32_t add_hi = hi + (((uint32_t)(old + lo) < old) ? 1u : 0u);
    if (add_hi)
      atomicAdd(w + 1, add_hi);
  } else {
    atomicAdd(t, (unsigned long long)q);
  }
}

/* Adds the fixed-point deposit llrint(dw 2^S) (ties to even, the oracle's
 * quantisation) to a tally cell.  A deposit with 0 <= dw 2^S < 2^31 (all but
 * the largest, and the negative ones of particles started outside their
 * cell) converts with the 32-bit conversion and adds with one 32-bit atomic
 * and a carry into the high word; the others take the 64-bit conversion,
 * which issues on the FP64 pipe (about 6e11/s per GB300, the strict
 * tracker's binding resource while it ran on every step). */
template <int TALLY>
__device__ __forceinline__ void mcg_deposit_u31(unsigned long long *t, float v)
{
  /* v = dw 2^S with +0 <= v < 2^31: the 32-bit conversion is exact */
  const uint32_t q = __float2uint_rn(v);
  if (TALLY == MCG_TALLY_SMEM32) {
    unsigned *w = reinterpret_cast<unsigned *>(t);
    const uint32_t old = atomicAdd(w, q);
    if ((uint32_t)(old + q) < old)
      atomicAdd(w + 1, 1u);
  } else {
    atomicAdd(t, (unsigned long long)q);
  }
}

template <int TALLY>
__device__ __forceinline__ void mcg_deposit(unsigned long long *t, float dw, int S)
{
  const float v = __fmul_rn(dw, mcg_fixed_scale(S));
  if (__float_as_uint(v) < 0x4f000000u) /* +0 <= v < 2^31 */
    mcg_deposit_u31<TALLY>(t, v);
  else
    mcg_tally_add<TALLY>(t, mcg_to_fixed(dw, S));
}

enum { MCG_CNT_HIST = 0, MCG_CNT_STEPS, MCG_CNT_SCAT, MCG_CNT_LEFT, MCG_CNT_RIGHT, MCG_CNT_KILL,
       MCG_CNT_WLEFT, MCG_CNT_WRIGHT, MCG_CNT_WKILL, MCG_CNT_ERR, MCG_CNT_N };

/* Particle of a device-born source (see mcg_source in mcgb300.h) whose
 * seed-chain state s is known: particle k has s = the chain's (k+1)-th
 * state from base_seed (seed_mode 0) or base_seed + k (seed_mode 1). */
__device__ __forceinline__ void mcg_source_particle_at(const mcg_source &S, uint64_t s,
                                                       uint64_t &seed, float &x, float &mu,
                                                       float &wmc, int &idx)
{
  float m = S.mu0;
  if (S.isotropic == 1)
    m = __fsub_rn(__fmul_rn(2.0f, mcg_rnd_real(s)), 1.0f);
  else if (S.isotropic == 2)
    m = mcg_rnd_real(s);
  seed = s;
  x = S.x0;
  mu = m;
  wmc = S.w0;
  idx = S.cell0;
}

/* Particle k of a device-born source. */
__device__ __forceinline__ void mcg_source_particle(const mcg_source &S, int64_t k, uint64_t &seed,
                                                    float &x, float &mu, float &wmc, int &idx)
{
  const uint64_t s = S.seed_mode == 0 ? mcg_lcg_skip(S.base_seed, (uint64_t)k + 1, 1)
                                      : ((S.base_seed + (uint64_t)k) & MCG_MASK63);
  mcg_source_particle_at(S, s, seed, x, mu, wmc, idx);
}

__device__ __forceinline__ void mcg_load_particle(const mcg_track_params &P, int64_t i,
                                                  uint64_t &seed, float &x, float &mu, float &wmc,
                                                  int &idx)
{
  if (P.particles) {
    const unsigned long long *q = reinterpret_cast<const unsigned long long *>(P.particles + i);
    unsigned long long a = q[0], b = q[1], c = q[2];
    seed = a;
    x = __uint_as_float((uint32_t)b);
    mu = __uint_as_float((uint32_t)(b >> 32));
    wmc = __uint_as_float((uint32_t)c);
    idx = (int)(uint32_t)(c >> 32);
  } else {
    mcg_source_particle(P.src, P.first + i, seed, x, mu, wmc, idx);
  }
}

/* The fast arithmetic's weight update wmc <- RN(wmc - dep), with the exact
 * rounding residue (Fast2Sum: |dep| <= |wmc|) added to *wres when given: the
 * particle's weight is then the pair wmc + wres, so deposits plus final
 * weights conserve the born weight, while each deposit stays the rounded
 * product om wmc (no per-cell bias). */
__device__ __forceinline__ void mcg_fast_weight_update(float &wmc, float dep, float *wres)
{
  const float w = __fsub_rn(wmc, dep);
  if (wres)
    *wres = __fadd_rn(*wres, __fsub_rn(__fsub_rn(wmc, w), dep));
  wmc = w;
}

/* The fast step's flight: the crossing's absorption 1 - e^(-sig_a de) into
 * om_cross, and whether the flight ends in a collision before the face, the
 * event -ln(1 - u) / sig_i < de of the reference's test evaluated as
 * u < 1 - e^(-sig_i de) (no logarithm per step; the collision's distance is
 * computed only when it happens).  sig_i = 0 when it is at most EPS (never a
 * collision, as the reference's di = MAXREAL). */
__device__ __forceinline__ bool mcg_fast_flight(uint64_t seed, float sig_a, float sig_i, float de,
                                                float &om_cross)
{
  const float ta = -sig_a * de, ti = -sig_i * de;
  float p;
  if (fmaxf(fabsf(ta), fabsf(ti)) < 0x1p-7f) {
    om_cross = mcg_one_minus_exp_small(ta);
    p = mcg_one_minus_exp_small(ti);
  } else {
    om_cross = mcg_one_minus_exp_fast(ta);
    p = mcg_one_minus_exp_fast(ti);
  }
  return mcg_flight_u(seed) < p;
}

/* Distance of the fast step's collision: -ln(1 - u) / sig_i, at most de. */
__device__ __forceinline__ float mcg_fast_collision_distance(uint64_t seed, float sig_i, float de)
{
  return fminf(mcg_flight_log2(seed) * __fdividef(-0.6931472f, sig_i), de);
}

/* One Layer::particle_step (src/layer.cpp:123-190) on a lane's particle in
 * cell c = {sig_a, sig_i (fast: 0 when at most EPS), edge_lo, edge_hi}; deposits into
 * *tally_cell.  STRICT: the reference's float operations and host-libm
 * logf/expf; the crossing's absorption is computed before the logarithm and
 * a certified exponential bound settles most crossings without it (see
 * mcg_cross_threshold).  FAST: hardware log2/exp2.  THIN (strict; chains
 * whose crossings almost all have |sig_a de| < MCG_EXP_SMALL_T): the
 * certain-crossing path evaluates only the small-argument exp form and
 * leaves the rarer larger arguments to the full step. */
template <bool STRICT, int TALLY, bool THIN = false>
__device__ __forceinline__ void mcg_step(uint64_t &seed, float &x, float &mu, float &wmc,
                                         float &inv_mu, int &idx, uint32_t &nsc, const float4 c,
                                         unsigned long long *tally_cell, int qs,
                                         const mcg_libm_tab *T, const mcg_libm_dev &LM,
                                         float *l_out = nullptr,
                                         bool *coll_out = nullptr, float *dep_out = nullptr,
                                         float *wres = nullptr)
{
  const float sig_a = c.x;
  mcg_lcg_next(seed); /* the flight sample's state */
  const bool neg = mu < 0.0f;
  int inew = neg ? idx - 1 : idx + 1;
  const float edge = neg ? c.z : c.w;
  float om;
  if (STRICT) {
    /* The certain crossing, computed without branches: d_edge by the cached
     * reciprocal, the crossing's absorption by the exp evaluator, its
     * deposit, and the certified bound.  It is the reference's step exactly
     * when every condition in `easy` holds (division and exp arguments in the
     * range where those forms are exact, no exception-table candidate, a
     * deposit below 2^31 fixed-point units, a flight certainly past the
     * edge); almost every step of a fine mesh is such a crossing.  Any other
     * step takes the full step below with the same state. */
    const float a = __fsub_rn(edge, x), aa = fabsf(a);
    const float de_q = mcg_div_by_rcp(a, mu, inv_mu);
    const float t_q = __fmul_rn(-sig_a, de_q);
    /* no exception-table candidate: the midpoint distance 0.5 - |yl| 2^24
     * above the table's largest threshold tau; the thin form tests |yl|
     * against (0.5 - tau) 2^-24 (1 - 2^-21) instead, which implies it: the
     * bound's two roundings leave it below (0.5 - tau) 2^-24 (1 - 3.5e-7),
     * so 0.5 - |yl| 2^24 exceeds tau by more than 3.5e-8 for tau < 0.4,
     * more than the 2^-25 rounding of that subtraction (the host takes this
     * form only for tables with tau < 0.25, mcg_strict_thin); two
     * operations less per step */
    float d_q = 0.f, yl_q = 0.f;
    const float y_q = THIN ? mcg_exp_small_yl(t_q, &yl_q) : mcg_exp_ff_core(t_q, &d_q, T);
    const bool far_q =
        THIN ? (fabsf(yl_q) < __fmul_rn(__fsub_rn(0.5f, LM.tau_exp_max), 0x1.fffffp-25f))
             : (d_q > LM.tau_exp_max);
    const float dw_q = __fmul_rn(__fsub_rn(1.0f, y_q), wmc);
    const float v_q = __fmul_rn(dw_q, mcg_fixed_scale(qs));
    const bool t_ok = THIN ? (fabsf(t_q) < MCG_EXP_SMALL_T)
                           : ((t_q >= MCG_EXP_ONE_BOUND) & (t_q < 89.0f));
    const bool easy = (inv_mu != 0.0f) & (aa >= 0x1p-100f) & (aa <= 0x1p100f) & t_ok &
                      far_q & (__float_as_uint(v_q) < 0x4f000000u) &
                      (mcg_state_hi(seed) < mcg_cross_threshold(c.y, de_q));
    if (easy) {
      x = edge;
      wmc = __fsub_rn(wmc, dw_q);
      if (tally_cell)
        mcg_deposit_u31<TALLY>(tally_cell, v_q);
      if (l_out) {
        *l_out = de_q;
        *coll_out = false;
        *dep_out = dw_q;
      }
      idx = inew;
      return;
    }
    bool cross = true;
    float de, di = MCG_MAXREAL;
    {
      /* d_edge, and the crossing's absorption, do not depend on the flight
       * sample: start them before the logarithm */
      de = inv_mu == 0.0f ? MCG_MAXREAL
           : (aa >= 0x1p-100f && aa <= 0x1p100f) ? de_q
                                                  : __fdiv_rn(a, mu);
      const float om_cross = mcg_one_minus_expf_strict(__fmul_rn(-sig_a, de), T, LM);
      /* di = sig_i > EPS ? -log(h) / sig_i : MAXREAL; the exact value is
       * only needed when the flight may end inside the cell: the certified
       * test settles almost every crossing */
      if (c.y > MCG_EPS) {
        if (!(mcg_state_hi(seed) < mcg_cross_threshold(c.y, de))) {
          di = __fdiv_rn(-mcg_logf_strict(mcg_unit_of(seed), T, LM), c.y);
          cross = !(di < de);
        }
      } else {
        cross = !(di < de);
      }
      if (!cross) {
        inew = idx;
        x = __fadd_rn(x, __fmul_rn(di, mu));
        mu = __fsub_rn(__fmul_rn(2.0f, mcg_rnd_real(seed)), 1.0f);
        inv_mu = mcg_flight_rcp(mu);
        om = mcg_one_minus_expf_strict(__fmul_rn(-sig_a, di), T, LM);
        ++nsc;
      } else {
        x = edge;
        om = om_cross;
      }
    }
    const float dw = __fmul_rn(om, wmc);
    wmc = __fsub_rn(wmc, dw);
    if (tally_cell)
      mcg_deposit<TALLY>(tally_cell, dw, qs);
    if (l_out) {
      *l_out = cross ? de : di;
      *coll_out = !cross;
      *dep_out = dw;
    }
  } else {
    /* The common crossing without branches: a direction (|mu| > EPS), both
     * optical depths to the face below 2^-7 (the short series), no
     * collision and a deposit below 2^31 fixed-point units; it computes
     * exactly what the full step below computes for such a step. */
    const float de_q = (edge - x) * inv_mu;
    const float ta = -sig_a * de_q, ti = -c.y * de_q;
    const float dep_q = __fmul_rn(mcg_one_minus_exp_small(ta), wmc);
    const float v_q = __fmul_rn(dep_q, mcg_fixed_scale(qs));
    const bool easy = (inv_mu != 0.0f) & (fmaxf(fabsf(ta), fabsf(ti)) < 0x1p-7f) &
                      !(mcg_flight_u(seed) < mcg_one_minus_exp_small(ti)) &
                      (__float_as_uint(v_q) < 0x4f000000u);
    if (easy) {
      x = edge;
      mcg_fast_weight_update(wmc, dep_q, wres);
      if (tally_cell)
        mcg_deposit_u31<TALLY>(tally_cell, v_q);
      if (l_out) {
        *l_out = de_q;
        *coll_out = false;
        *dep_out = dep_q;
      }
      idx = inew;
      return;
    }
    const float de = inv_mu != 0.0f ? (edge - x) * inv_mu : MCG_MAXREAL;
    float om_cross;
    const bool coll = mcg_fast_flight(seed, sig_a, c.y, de, om_cross);
    const float di = coll ? mcg_fast_collision_distance(seed, c.y, de) : de;
    if (l_out) {
      *l_out = di;
      *coll_out = coll;
    }
    if (coll) {
      inew = idx;
      x = fmaf(di, mu, x);
      mu = fmaf(2.0f, mcg_rnd_real_fast(seed), -1.0f);
      inv_mu = mcg_flight_rcp(mu);
      om = mcg_one_minus_exp_fast(-sig_a * di);
      ++nsc;
    } else {
      x = edge;
      om = om_cross;
    }
    /* the deposit is the rounded product om wmc, as the reference's dw: a
     * deposit taken as the weight actually removed, wmc - RN(wmc - om wmc),
     * conserves the born weight exactly but carries the rounding of the
     * subtraction, up to half an ulp of wmc, which on a thin absorber
     * (om ~ 1e-5) is a 3e-3 relative error of the deposit, the same for
     * every uncollided particle of a cell: a systematic per-cell bias */
    const float dep = __fmul_rn(om, wmc);
    mcg_fast_weight_update(wmc, dep, wres);
    if (tally_cell)
      mcg_deposit<TALLY>(tally_cell, dep, qs);
    if (dep_out)
      *dep_out = dep;
  }
  idx = inew;
}

/* One Layer::particle_step (src/layer.cpp:123-190) on a lane's particle in
 * cell c = {sig_a, sig_i (fast: 0 when at most EPS), edge_lo, edge_hi}, in two parts, for
 * the event-based tracker: mcg_step_cross advances the state to the flight
 * sample's and completes the step when it is a certain crossing (STRICT: the
 * branch-free path of mcg_step; FAST: the flight ends past the edge),
 * returning true; otherwise it changes nothing but the seed and returns
 * false, and mcg_step_rest completes the step from the advanced state, which
 * determines the flight sample.  Together they perform exactly
 * mcg_step's operations (mcg_step, the one-piece form above, serves the
 * history-based kernels, where the split costs about 6 %).  STRICT: the reference's float operations and host-libm
 * logf/expf; the crossing's absorption is computed before the logarithm and
 * a certified exponential bound settles most crossings without it (see
 * MCG_CROSS_FACTOR).  FAST: hardware log2/exp2.  Deposits go into
 * *tally_cell; l_out/coll_out/dep_out (adjoint) receive the flight length,
 * whether it ended in a collision and the deposit. */
template <bool STRICT, int TALLY>
__device__ __forceinline__ bool mcg_step_cross(uint64_t &seed, float &x, float &mu, float &wmc,
                                               float &inv_mu, int &idx, const float4 c,
                                               unsigned long long *tally_cell, int qs,
                                               const mcg_libm_tab *T, const mcg_libm_dev &LM,
                                               float *l_out = nullptr,
                                               bool *coll_out = nullptr, float *dep_out = nullptr,
                                               float *wres = nullptr)
{
  const float sig_a = c.x;
  mcg_lcg_next(seed); /* the flight sample's state */
  const bool neg = mu < 0.0f;
  const float edge = neg ? c.z : c.w;
  if (STRICT) {
    /* The certain crossing, computed without branches: d_edge by the cached
     * reciprocal, the crossing's absorption by the exp evaluator, and the
     * certified bound.  It is the reference's step exactly when every
     * condition in `easy` holds (division and exp arguments in the range
     * where those forms are exact, no exception-table candidate, a flight
     * certainly past the edge); almost every step of a fine mesh is such a
     * crossing. */
    const float a = __fsub_rn(edge, x), aa = fabsf(a);
    const float de_q = mcg_div_by_rcp(a, mu, inv_mu);
    const float t_q = __fmul_rn(-sig_a, de_q);
    float d_q;
    const float y_q = mcg_exp_ff_core(t_q, &d_q, T);
    const bool easy = (inv_mu != 0.0f) & (aa >= 0x1p-100f) & (aa <= 0x1p100f) &
                      (t_q >= MCG_EXP_ONE_BOUND) & (t_q < 89.0f) & (d_q > LM.tau_exp_max) &
                      (mcg_state_hi(seed) < mcg_cross_threshold(c.y, de_q));
    if (!easy)
      return false;
    x = edge;
    const float dw = __fmul_rn(__fsub_rn(1.0f, y_q), wmc);
    wmc = __fsub_rn(wmc, dw);
    if (tally_cell)
      mcg_deposit<TALLY>(tally_cell, dw, qs);
    if (l_out) {
      *l_out = de_q;
      *coll_out = false;
      *dep_out = dw;
    }
  } else {
    const float de = inv_mu != 0.0f ? (edge - x) * inv_mu : MCG_MAXREAL;
    float om;
    if (mcg_fast_flight(seed, sig_a, c.y, de, om))
      return false;
    if (l_out) {
      *l_out = de;
      *coll_out = false;
    }
    x = edge;
    /* the deposit is the rounded product om wmc, as the reference's dw: a
     * deposit taken as the weight actually removed, wmc - RN(wmc - om wmc),
     * conserves the born weight exactly but carries the rounding of the
     * subtraction, up to half an ulp of wmc, which on a thin absorber
     * (om ~ 1e-5) is a 3e-3 relative error of the deposit, the same for
     * every uncollided particle of a cell: a systematic per-cell bias */
    const float dep = __fmul_rn(om, wmc);
    mcg_fast_weight_update(wmc, dep, wres);
    if (tally_cell)
      mcg_deposit<TALLY>(tally_cell, dep, qs);
    if (dep_out)
      *dep_out = dep;
  }
  idx = neg ? idx - 1 : idx + 1;
  return true;
}

template <bool STRICT, int TALLY>
__device__ __forceinline__ void mcg_step_rest(uint64_t &seed, float &x, float &mu,
                                              float &wmc, float &inv_mu, int &idx, uint32_t &nsc,
                                              const float4 c, unsigned long long *tally_cell,
                                              int qs, const mcg_libm_tab *T,
                                              const mcg_libm_dev &LM, float *l_out = nullptr,
                                              bool *coll_out = nullptr, float *dep_out = nullptr,
                                              float *wres = nullptr)
{
  const float sig_a = c.x;
  const bool neg = mu < 0.0f;
  int inew = neg ? idx - 1 : idx + 1;
  const float edge = neg ? c.z : c.w;
  float om;
  if (STRICT) {
    /* d_edge, and the crossing's absorption, do not depend on the flight
     * sample: start them before the logarithm */
    const float a = __fsub_rn(edge, x), aa = fabsf(a);
    const float de = inv_mu == 0.0f ? MCG_MAXREAL
                     : (aa >= 0x1p-100f && aa <= 0x1p100f) ? mcg_div_by_rcp(a, mu, inv_mu)
                                                            : __fdiv_rn(a, mu);
    const float om_cross = mcg_one_minus_expf_strict(__fmul_rn(-sig_a, de), T, LM);
    /* di = sig_i > EPS ? -log(h) / sig_i : MAXREAL; the exact value is
     * only needed when the flight may end inside the cell: the certified
     * test settles almost every crossing */
    bool cross = true;
    float di = MCG_MAXREAL;
    if (c.y > MCG_EPS) {
      if (!(mcg_state_hi(seed) < mcg_cross_threshold(c.y, de))) {
        di = __fdiv_rn(-mcg_logf_strict(mcg_unit_of(seed), T, LM), c.y);
        cross = !(di < de);
      }
    } else {
      cross = !(di < de);
    }
    if (!cross) {
      inew = idx;
      x = __fadd_rn(x, __fmul_rn(di, mu));
      mu = __fsub_rn(__fmul_rn(2.0f, mcg_rnd_real(seed)), 1.0f);
      inv_mu = mcg_flight_rcp(mu);
      om = mcg_one_minus_expf_strict(__fmul_rn(-sig_a, di), T, LM);
      ++nsc;
    } else {
      x = edge;
      om = om_cross;
    }
    const float dw = __fmul_rn(om, wmc);
    wmc = __fsub_rn(wmc, dw);
    if (tally_cell)
      mcg_deposit<TALLY>(tally_cell, dw, qs);
    if (l_out) {
      *l_out = cross ? de : di;
      *coll_out = !cross;
      *dep_out = dw;
    }
  } else {
    const float de = inv_mu != 0.0f ? (edge - x) * inv_mu : MCG_MAXREAL;
    float om_cross;
    const bool coll = mcg_fast_flight(seed, sig_a, c.y, de, om_cross);
    const float di = coll ? mcg_fast_collision_distance(seed, c.y, de) : de;
    if (l_out) {
      *l_out = di;
      *coll_out = coll;
    }
    if (coll) {
      inew = idx;
      x = fmaf(di, mu, x);
      mu = fmaf(2.0f, mcg_rnd_real_fast(seed), -1.0f);
      inv_mu = mcg_flight_rcp(mu);
      om = mcg_one_minus_exp_fast(-sig_a * di);
      ++nsc;
    } else {
      x = edge;
      om = om_cross;
    }
    const float dep = __fmul_rn(om, wmc);
    mcg_fast_weight_update(wmc, dep, wres);
    if (tally_cell)
      mcg_deposit<TALLY>(tally_cell, dep, qs);
    if (dep_out)
      *dep_out = dep;
  }
  idx = inew;
}

/* THIN: the chain is optically thin (every |sig_a cell width| <= 5e-4):
 * the strict step's thin certain-crossing path, and, in both arithmetics,
 * four steps per pass of the step loop. */
template <bool STRICT, int TALLY, bool THIN>
__global__ void __launch_bounds__(1024) mcg_track_kernel(mcg_track_params P)
{
  extern __shared__ __align__(16) unsigned char smem[];
  mcg_libm_tab *T = reinterpret_cast<mcg_libm_tab *>(smem);
  unsigned long long *s_cnt = reinterpret_cast<unsigned long long *>(smem + sizeof(mcg_libm_tab));
  unsigned long long *s_tally = s_cnt + 16;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ncell = P.n_cells, lo = P.cell_lo;

  if (STRICT) {
    const float *src = reinterpret_cast<const float *>(P.libm_tab);
    float *dst = reinterpret_cast<float *>(T);
    for (int i = tid; i < (int)(sizeof(mcg_libm_tab) / 4); i += blockDim.x)
      dst[i] = src[i];
  }
  if (tid < 16)
    s_cnt[tid] = 0ull;
  if (TALLY != MCG_TALLY_GLOBAL)
    for (int i = tid; i < ncell * P.tally_copies; i += blockDim.x)
      s_tally[i] = 0ull;
  __syncthreads();
  unsigned long long *my_tally = TALLY == MCG_TALLY_GLOBAL
                                     ? P.tally
                                     : s_tally + (size_t)(warp % P.tally_copies) * ncell;

  uint64_t seed = 0;
  float x = 0.f, mu = 0.f, wmc = 0.f, inv_mu = 0.f;
  float wres = 0.f; /* fast: the weight's rounding residue (mcg_fast_weight_update) */
  int idx = 0;
  int64_t hid = -1;
  uint32_t nst = 0, nsc = 0;
  bool active = false;
  unsigned long long tot_steps = 0, tot_scat = 0;
  long long pool_next = 0, pool_end = 0;
  bool drained = false;
  const float min_w = P.min_w;
  const int qs = P.q_log2;

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
        mcg_load_particle(P, hid, seed, x, mu, wmc, idx);
        idx -= lo;
        inv_mu = mcg_flight_rcp(mu);
        wres = 0.f;
        nst = nsc = 0;
        active = true;
      }
    }
    if (!__any_sync(0xffffffffu, active))
      break;

    if (active) {
      /* up to refill_steps steps, never past the step limit; idx is the
       * cell index local to the chain, so one unsigned compare is the
       * range test of simulate_particle's loop */
      const int kmax = (int)min((uint32_t)P.refill_steps, P.max_steps - nst);
      int k = 0;
      /* four steps per loop pass on thin chains: measured 3 % faster
       * (strict) than one; on thicker chains, where crossings split between
       * the exp evaluator's paths, one (four measured 36 % slower) */
      constexpr int kUnroll = THIN ? 4 : 1;
#pragma unroll kUnroll
      for (; k < kmax;) {
        if (!((wmc >= min_w) & ((unsigned)idx < (unsigned)ncell)))
          break;
        mcg_step<STRICT, TALLY, THIN>(seed, x, mu, wmc, inv_mu, idx, nsc, __ldg(P.cells + idx),
                                      &my_tally[idx], qs, T, P.libm, nullptr, nullptr, nullptr,
                                      STRICT ? nullptr : &wres);
        ++k;
      }
      const bool going = (wmc >= min_w) & ((unsigned)idx < (unsigned)ncell);
      nst += (uint32_t)k;
      if (!going || nst >= P.max_steps) {
        /* history ends: classification of simulate_particle; a history
         * still alive in the chain here has reached the step limit */
        const bool in = (wmc >= min_w) && ((unsigned)idx < (unsigned)ncell);
        int r;
        if (in)
          r = 2;
        else if (idx == -1)
          r = -1;
        else if (idx == ncell)
          r = 1;
        else if (wmc < min_w)
          r = 0;
        else
          r = -1;
        if (P.particles) {
          unsigned long long *q = reinterpret_cast<unsigned long long *>(P.particles + hid);
          q[0] = seed;
          q[1] = (unsigned long long)__float_as_uint(x) |
                 ((unsigned long long)__float_as_uint(mu) << 32);
          q[2] = (unsigned long long)__float_as_uint(wmc) |
                 ((unsigned long long)(uint32_t)(idx + lo) << 32);
        }
        if (P.results)
          P.results[hid] = r;
        if (P.steps)
          P.steps[hid] = nst;
        if (P.scatters)
          P.scatters[hid] = nsc;
        atomicAdd(&s_cnt[MCG_CNT_HIST], 1ull);
        long long wq = mcg_to_fixed(wmc, qs);
        if (!STRICT)
          wq += mcg_to_fixed(wres, qs); /* the weight's float-float remainder */
        if (r == -1) {
          atomicAdd(&s_cnt[MCG_CNT_LEFT], 1ull);
          atomicAdd(&s_cnt[MCG_CNT_WLEFT], (unsigned long long)wq);
        } else if (r == 1) {
          atomicAdd(&s_cnt[MCG_CNT_RIGHT], 1ull);
          atomicAdd(&s_cnt[MCG_CNT_WRIGHT], (unsigned long long)wq);
        } else if (r == 0) {
          atomicAdd(&s_cnt[MCG_CNT_KILL], 1ull);
          atomicAdd(&s_cnt[MCG_CNT_WKILL], (unsigned long long)wq);
        } else {
          atomicOr(&s_cnt[MCG_CNT_ERR], 1ull);
        }
        tot_steps += nst;
        tot_scat += nsc;
        active = false;
      }
    }
  }

  /* per-thread counters -> block */
  for (int o = 16; o > 0; o >>= 1) {
    tot_steps += __shfl_down_sync(0xffffffffu, tot_steps, o);
    tot_scat += __shfl_down_sync(0xffffffffu, tot_scat, o);
  }
  if (lane == 0) {
    atomicAdd(&s_cnt[MCG_CNT_STEPS], tot_steps);
    atomicAdd(&s_cnt[MCG_CNT_SCAT], tot_scat);
  }
  __syncthreads();
  if (TALLY != MCG_TALLY_GLOBAL)
    for (int i = tid; i < ncell; i += blockDim.x) {
      unsigned long long s = 0;
      for (int c = 0; c < P.tally_copies; ++c)
        s += s_tally[(size_t)c * ncell + i];
      if (s)
        atomicAdd(&P.tally[i], s);
    }
  if (tid < MCG_CNT_N) {
    if (tid == MCG_CNT_ERR) {
      if (s_cnt[tid])
        atomicOr(&P.counters[tid], s_cnt[tid]);
    } else if (s_cnt[tid]) {
      atomicAdd(&P.counters[tid], s_cnt[tid]);
    }
  }
}

#endif
