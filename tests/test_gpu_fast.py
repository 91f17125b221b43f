"""GPU statistical parity of the fast tracker against the FP64 CPU oracle:
every per-cell tally within 3 standard errors, and the weight balance
(absorbed + leaked + cut off = born) to 1e-6 relative."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _phys0(m=100):
    xc = ((np.arange(m) + 0.5) / m).astype(np.float32)
    sa = (np.float32(0.2) + np.float32(1.8) * xc).astype(np.float32)
    sigs = (sa + np.float32(1.0)).astype(np.float32)
    return sigs, (sa / sigs).astype(np.float32)


def _phys1(nb=10000):
    xc = (np.arange(nb) + 0.5) / nb
    sa = (0.5 + 0.4 * np.sin(6 * np.pi * xc)).astype(np.float32)
    ss = (2.0 + 1.5 * np.cos(4 * np.pi * xc)).astype(np.float32)
    sigs = (sa + ss).astype(np.float32)
    return sigs, (sa / sigs).astype(np.float32)


def _check(ctx, oracle, layers, sigs, rates, n, scale):
    p = np.zeros(n, oracle.PARTICLE_DTYPE)
    p["seed"] = oracle.rnd_seed_chain(5127801, n)
    p["mu"], p["wmc"] = 1.0, 1.0
    ref = oracle.fp64_histories(layers, sigs, rates, 1e-12, p)
    ctx.simulate_source(0, n, seed_mode=0, base_seed=5127801, x0=0.0, mu0=1.0, w0=1.0)
    gpu = ctx.tally()
    var = np.maximum(ref["tally_sq"] / n - (ref["tally"] / n) ** 2, 0.0)
    se_sum = np.sqrt(var * n)  # standard error of the per-cell sum over n histories
    ok = np.abs(gpu - ref["tally"]) <= 3.0 * se_sum + 1e-9
    assert ok.all(), f"{np.count_nonzero(~ok)} cells beyond 3 SE"
    c = ctx.counters()
    out = (c["w_left_q"] + c["w_right_q"] + c["w_killed_q"]) * 2.0 ** -scale
    assert abs(gpu.sum() + out - n) <= 1e-6 * n
    return gpu, ref


@pytest.mark.parametrize("mode", ["fast", "strict"])
def test_config0_within_3se_of_fp64(built, mcg, oracle, mode):
    sigs, rates = _phys0()
    with mcg.Context(mode=mode) as ctx:
        ctx.set_layers([0], [100], [np.float32(0.01)], sigs, rates, 1e-12)
        ctx.set_tally_scale(40)
        _check(ctx, oracle, [oracle.layer_make(0.0, 1.0, 0, 100)], sigs, rates, 200000, 40)


def test_slab10k_fast_within_3se_of_fp64(built, mcg, oracle):
    sigs, rates = _phys1()
    st, m, dx, _, _ = mcg.layer_decomposition(0.0, 1.0, 10000, 64)
    with mcg.Context(mode="fast") as ctx:
        ctx.set_layers(st, m, dx, sigs, rates, 1e-12)
        ctx.set_tally_scale(40)
        _check(ctx, oracle, list(oracle.decompose(0.0, 1.0, 10000, 64)), sigs, rates, 20000, 40)


def test_flight_log2_accurate_near_one(built, mcg):
    """The fast flight's log2 (fn 5) on every value the fast uniform takes,
    (k + 1/2) 2^-23: for u = 1 - h < 2^-8, where a thin cell's collision
    probability is decided, relative error <= 2^-21 and no systematic sign
    (measured with fn 4, the hardware log2 alone is biased there: -2.9e-4
    relative on average for 2^-15 <= u < 2^-11, which moved the fast
    tallies of the 10k-cell slab by several standard errors at 1e8
    histories); above, relative error <= 2^-15."""
    import torch
    k = np.arange(1 << 23, dtype=np.float64)
    h = ((k + 0.5) * 2.0 ** -23).astype(np.float32)
    assert np.all(h.astype(np.float64) == (k + 0.5) * 2.0 ** -23)
    exact = np.log2(h.astype(np.float64))
    with mcg.Context(mode="strict") as ctx:
        ctx.set_layers([0], [1], [np.float32(1.0)], np.ones(1, np.float32),
                       np.full(1, 0.5, np.float32), 1e-12)
        ctx.simulate_source(0, 4)  # loads the strict tables the evaluator needs
        d_in = torch.from_numpy(h).cuda()
        d_out = torch.empty_like(d_in)
        torch.cuda.synchronize()  # the library runs on its own stream
        ctx.libm_eval_device(5, d_in.data_ptr(), d_out.data_ptr(), len(h))
        got = d_out.cpu().numpy().astype(np.float64)
    rel = (got - exact) / exact
    near = (1.0 - h.astype(np.float64)) < 2.0 ** -8
    assert np.abs(rel[near]).max() <= 2.0 ** -21
    assert abs(rel[near].mean()) <= 1e-7
    assert np.abs(rel[~near]).max() <= 2.0 ** -15
