"""The strict GPU tracker against the oracle on randomised single-layer cases
(the cases of tests/test_oracle_fuzz.py, where the oracle itself is checked
against the reference's compiled Layer): per particle the final 24-byte
state, steps, scatters and result; per case the int64 fixed-point tally."""
import numpy as np
import pytest

from fuzz_cases import case, particles

pytestmark = pytest.mark.gpu
f32 = np.float32
SCALE = 40


@pytest.fixture(scope="module")
def ctx(built, mcg):
    c = mcg.Context(mode="strict")
    yield c
    c.close()


@pytest.mark.parametrize("seed", range(12))
def test_gpu_matches_oracle_on_random_layers(ctx, mcg, oracle, seed):
    rng, m, x_min, x_max, start, sigs, rates = case(seed)
    L = oracle.layer_make(float(x_min), float(x_max), start, m)
    min_w = 1e-12
    p = particles(rng, mcg.PARTICLE_DTYPE, L, 1500)
    init = p.copy()
    ctx.set_layers([start], [m], [L.dx], sigs, rates, min_w)
    ctx.set_tally_scale(SCALE)
    r = ctx.simulate(p)
    ref = oracle.layer_simulate(L, sigs, rates, min_w, init[::-1].copy(), len(init))
    assert p.tobytes() == ref["particles"][::-1].tobytes()
    t = ref["traces"]
    assert np.array_equal(r["steps"], t["steps"])
    assert np.array_equal(r["scatters"], t["scatters"])
    assert np.array_equal(r["results"], t["result"])
    # the oracle's chain driver indexes cross sections and tallies by global cell
    pad = np.zeros(start, f32)
    q = oracle.simulate_histories([L], np.concatenate([pad, sigs]), np.concatenate([pad, rates]),
                                  min_w, init, 2.0 ** SCALE)
    assert np.array_equal(ctx.tally_q(), q["tally_q"][start:])
