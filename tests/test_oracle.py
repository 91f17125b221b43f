"""CPU tests of the oracle (the checker) against the reference's golden data.

Mirrors the reference's own tests: src/test_layer.cpp (golden WA.out),
src/test_curandom.cu (RNG chain), src/test_async_serialization.cpp (Particle
layout), and per-particle histories of the reference's Layer::particle_step.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN

f32 = np.float32


def load(name):
    return np.load(os.path.join(GOLDEN, name))


def test_golden_test_layer_wa(oracle):
    """src/test_layer.cpp:41-73: byte-identical WA.out."""
    L = oracle.decompose(0.0, 1.0, 100, 1)[0]
    sigs, rates = oracle.default_sigs(L)
    x_ini = f32(np.sqrt(f32(2.0)) / f32(2.0))
    ps = oracle.create_particles(L, float(x_ini), float(f32(1.0 / 100)), 100, 5127801)
    r = oracle.layer_simulate(L, sigs, rates, 0.0, ps, 100)
    with open(os.path.join(GOLDEN, "test_layer_WA.out")) as f:
        assert oracle.format_wa(L, r["tally_f32"]) == f.read()


def test_rng_chain_kat(oracle):
    """src/test_curandom.cu:23-37: seed chain from 30061994, one rnd_real each."""
    g = load("rng_chain.npz")
    seeds = oracle.rnd_seed_chain(int(g["start"]), len(g["seeds"]))
    assert np.array_equal(seeds, g["seeds"])
    after, reals = oracle.rnd_real(seeds[:2000])
    assert np.array_equal(after, g["seeds_after"][:2000])
    assert np.array_equal(reals.view(np.uint32), g["reals"][:2000].view(np.uint32))


def test_lcg_jump_ahead(oracle):
    g = load("rng_chain.npz")
    start = int(g["start"])
    for k in (1, 2, 3, 17, 1000, 9999):
        assert oracle.lcg_skip(start, k, True) == int(g["seeds"][k - 1])


def fnv1a_signed_char(data: bytes) -> int:
    """The hash of src/test_async_serialization.cpp:6-16 with x86's signed char."""
    h = 0x811C9DC5
    for b in data:
        v = b - 256 if b >= 128 else b
        h = (h ^ (v & 0xFFFFFFFF)) & 0xFFFFFFFF
        h = (h * 16777619) & 0xFFFFFFFF
    return h - (1 << 32) if h >= (1 << 31) else h


def test_particle_layout(mcg):
    """The 24-byte Particle: same bytes as the reference's struct."""
    p = np.zeros(1, mcg.PARTICLE_DTYPE)
    p[0] = (5127801, f32(0.172634512365276), f32(123.12342351), f32(-1231.123486123), 2134512)
    assert fnv1a_signed_char(p.tobytes()) == int(load("particle_hash.npz")["hash"])


@pytest.mark.parametrize("name", ["config0", "default1000", "sublayer", "edge"])
def test_oracle_matches_reference_traces(oracle, name):
    """Per particle, bit for bit: final state, result, steps, scatters."""
    g = load(f"traces_{name}.npz")
    lt = g["layer"]
    L = oracle.layer_make(float(lt[0]), float(lt[1]), int(lt[3]), int(lt[4]))
    assert (L.dx, L.left_border, L.right_border) == (f32(lt[2]), int(lt[5]), int(lt[6]))
    init = g["initial"].astype(oracle.PARTICLE_DTYPE)
    n = len(init)
    # layer_simulate processes from the back; feed reversed so traces align
    r = oracle.layer_simulate(L, g["sigs"], g["rates"], float(g["min_w"]), init[::-1].copy(), n)
    tr = r["traces"]
    fin = r["particles"][::-1]
    assert fin.tobytes() == g["final"].astype(oracle.PARTICLE_DTYPE).tobytes()
    assert np.array_equal(tr["result"], g["result"])
    assert np.array_equal(tr["steps"], g["steps"])
    assert np.array_equal(tr["scatters"], g["scatters"])


def test_decomposed_matches_single_chain(oracle):
    """Histories across 8 layers: the oracle's exact sums agree with the
    reference's WorkerSync-driven float tallies to float accuracy."""
    g = load("decomposed_1000x8.npz")
    layers = oracle.decompose(0.0, 1.0, 1000, int(g["n_layers"]))
    r = oracle.simulate_histories(list(layers), g["sigs"], g["rates"], float(g["min_w"]),
                                  g["particles"].astype(oracle.PARTICLE_DTYPE), 2.0 ** 40)
    ref = g["tally"]
    assert np.allclose(r["tally_f64"], ref, rtol=2e-5, atol=1e-4)
    assert abs(r["tally_f64"].sum() - ref.sum()) < 1e-5 * ref.sum()
    assert np.all(r["traces"]["result"] != 2)


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle",
                                                    "_ref", "libmcref.so")),
                    reason="reference not built here (oracle/_ref)")
def test_oracle_matches_reference_decomposed_live(oracle):
    """Against the reference compiled from source, on a fresh random case."""
    rng = np.random.default_rng(7)
    m = 300
    sa = rng.uniform(0.1, 5, m).astype(np.float32)
    ss = rng.uniform(0, 10, m).astype(np.float32)
    sigs = (sa + ss).astype(np.float32)
    rates = (sa / sigs).astype(np.float32)
    L = oracle.layer_make(0.0, 1.0, 0, m)
    p = np.zeros(3000, oracle.PARTICLE_DTYPE)
    p["seed"] = rng.integers(0, 2**63, 3000, dtype=np.uint64)
    p["x"], p["mu"], p["wmc"], p["index"] = 0.0, rng.uniform(-1, 1, 3000).astype(np.float32), 1.0, 0
    p["mu"][p["mu"] < 0] *= -1
    fin = p.copy()
    tr = np.zeros(len(p), oracle.TRACE_DTYPE)
    oracle.ref().ref_trace_particles(L.x_min, L.x_max, 0, m, f32(1e-12), oracle._p(sigs),
                                     oracle._p(rates), oracle._p(fin), len(fin), oracle._p(tr))
    r = oracle.layer_simulate(L, sigs, rates, 1e-12, p[::-1].copy(), len(p))
    assert r["particles"][::-1].tobytes() == fin.tobytes()
    assert np.array_equal(r["traces"]["steps"], tr["steps"])
