"""The oracle against the reference's own Layer code (oracle/_ref, compiled
from the reference's src/layer.cpp and src/random.cpp) on randomised cases:
layers inside and at the borders of [0, 1], cells from vacuum to optically
thick, cross sections at and around the EPS threshold, particles anywhere
in the layer with any direction (0, -0, +-EPS, +-1 included) and weights
around the minimum.  Per particle: final 24-byte state, steps, scatters and
result of simulate_particle; per call of Layer::simulate: the float tally
bit for bit, the leaver lists in order and nb_disabled."""
import os

import numpy as np
import pytest

f32 = np.float32
REF = os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref", "libmcref.so")
pytestmark = pytest.mark.skipif(not os.path.exists(REF),
                                reason="reference not built here (oracle/_ref)")


def _case(seed):
    rng = np.random.default_rng(seed)
    m = int(rng.integers(1, 300))
    kind = seed % 4
    if kind == 0:  # a whole [0, 1] slab: both borders
        x_min, x_max, start = 0.0, 1.0, 0
    elif kind == 1:  # an interior sub-domain
        start = int(rng.integers(1, 5000))
        dx = 1.0 / (start + m + int(rng.integers(1, 5000)))
        x_min, x_max = start * dx, (start + m) * dx
    elif kind == 2:  # touching the left border only
        start, x_min, x_max = 0, 0.0, float(rng.uniform(0.05, 0.9))
    else:  # touching the right border only
        start = int(rng.integers(1, 2000))
        x_min, x_max = float(rng.uniform(0.1, 0.95)), 1.0
    width = x_max - x_min
    # optical thickness of the layer up to ~40 for scattering and absorption
    sa = rng.uniform(0, 40 / width, m) * (rng.random(m) < 0.9)
    ss = rng.uniform(0, 40 / width, m) * (rng.random(m) < 0.85)
    eps_cells = rng.random(m) < 0.1  # sig_s around the 1e-4 threshold
    ss[eps_cells] = rng.choice([0.0, 5e-5, 1e-4, 1.0001e-4, 2e-4], eps_cells.sum())
    sigs = (sa + ss).astype(f32)
    with np.errstate(invalid="ignore", divide="ignore"):
        rates = np.where(sigs > 0, sa.astype(f32) / np.maximum(sigs, f32(1e-30)), 0.5).astype(f32)
    return rng, m, f32(x_min), f32(x_max), start, sigs, rates


def _particles(rng, oracle, L, n):
    p = np.zeros(n, oracle.PARTICLE_DTYPE)
    p["seed"] = rng.integers(0, 2**63, n, dtype=np.uint64)
    cell = rng.integers(0, L.m, n)
    frac = rng.random(n)
    frac[rng.random(n) < 0.1] = 0.0  # on a cell's left edge
    x = ((cell + frac) * np.float64(L.dx) + np.float64(L.index_start) * np.float64(L.dx))
    p["x"] = x.astype(f32)
    p["index"] = cell + L.index_start
    mu = rng.uniform(-1, 1, n)
    special = rng.random(n) < 0.15
    mu[special] = rng.choice([0.0, -0.0, 1e-4, -1e-4, 1.0001e-4, 1e-5, 1.0, -1.0], special.sum())
    p["mu"] = mu.astype(f32)
    w = rng.uniform(0, 1, n)
    low = rng.random(n) < 0.05
    w[low] = rng.choice([1e-12, 9.9e-13, 2e-12, 0.0], low.sum())
    p["wmc"] = w.astype(f32)
    return p


@pytest.mark.parametrize("seed", range(12))
def test_oracle_matches_reference_per_particle(oracle, seed):
    rng, m, x_min, x_max, start, sigs, rates = _case(seed)
    L = oracle.layer_make(float(x_min), float(x_max), start, m)
    min_w = f32(1e-12)
    p = _particles(rng, oracle, L, 1500)
    ref_p = p.copy()
    tr = np.zeros(len(p), oracle.TRACE_DTYPE)
    oracle.ref().ref_trace_particles(x_min, x_max, start, m, min_w, oracle._p(sigs),
                                     oracle._p(rates), oracle._p(ref_p), len(ref_p),
                                     oracle._p(tr))
    r = oracle.layer_simulate(L, sigs, rates, float(min_w), p[::-1].copy(), len(p))
    assert r["particles"][::-1].tobytes() == ref_p.tobytes()
    t = r["traces"]  # processing order: the reversed feed's back first = p's order
    assert np.array_equal(t["steps"], tr["steps"])
    assert np.array_equal(t["scatters"], tr["scatters"])
    assert np.array_equal(t["result"], tr["result"])


@pytest.mark.parametrize("seed", range(100, 108))
def test_oracle_matches_reference_layer_simulate(oracle, seed):
    """Layer::simulate(n, 1) on part of the stored particles: float tally,
    leaver lists (processing order) and nb_disabled."""
    import ctypes as C
    rng, m, x_min, x_max, start, sigs, rates = _case(seed)
    L = oracle.layer_make(float(x_min), float(x_max), start, m)
    min_w = f32(1e-12)
    p = _particles(rng, oracle, L, 1200)
    n = 900  # the last 900 stored particles, processed from the back
    tally = np.zeros(m, f32)
    left = np.zeros(len(p), oracle.PARTICLE_DTYPE)
    right = np.zeros(len(p), oracle.PARTICLE_DTYPE)
    nl, nr, nd = C.c_int(0), C.c_int(0), C.c_int(0)
    oracle.ref().ref_layer_simulate(x_min, x_max, start, m, min_w, oracle._p(sigs),
                                    oracle._p(rates), oracle._p(p), len(p), n, 1,
                                    oracle._p(tally), oracle._p(left), C.byref(nl),
                                    oracle._p(right), C.byref(nr), C.byref(nd))
    r = oracle.layer_simulate(L, sigs, rates, float(min_w), p, n)
    assert r["tally_f32"].tobytes() == tally.tobytes()
    done = r["particles"][len(p) - n:][::-1]  # processing order
    res = r["results"]
    exp_left = done[res == -1] if not L.left_border else done[:0]
    exp_right = done[res == 1] if not L.right_border else done[:0]
    assert (nl.value, nr.value) == (len(exp_left), len(exp_right))
    assert left[:nl.value].tobytes() == exp_left.tobytes()
    assert right[:nr.value].tobytes() == exp_right.tobytes()
    disabled = int(np.count_nonzero(res == 0))
    disabled += int(np.count_nonzero(res == -1)) if L.left_border else 0
    disabled += int(np.count_nonzero(res == 1)) if L.right_border else 0
    assert nd.value == disabled
