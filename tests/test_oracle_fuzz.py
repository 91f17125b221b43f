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

from fuzz_cases import case, particles

f32 = np.float32
REF = os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref", "libmcref.so")
pytestmark = pytest.mark.skipif(not os.path.exists(REF),
                                reason="reference not built here (oracle/_ref)")


@pytest.mark.parametrize("seed", range(12))
def test_oracle_matches_reference_per_particle(oracle, seed):
    rng, m, x_min, x_max, start, sigs, rates = case(seed)
    L = oracle.layer_make(float(x_min), float(x_max), start, m)
    min_w = f32(1e-12)
    p = particles(rng, oracle.PARTICLE_DTYPE, L, 1500)
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
    rng, m, x_min, x_max, start, sigs, rates = case(seed)
    L = oracle.layer_make(float(x_min), float(x_max), start, m)
    min_w = f32(1e-12)
    p = particles(rng, oracle.PARTICLE_DTYPE, L, 1200)
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
