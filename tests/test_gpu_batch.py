"""Batched slabs: every slab's fixed-point tally equals the oracle's (strict),
the batched launch equals one launch per slab, the autotuner keeps parity."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _oracle_slab(oracle, d, sigs, rates):
    n, m = d["n_histories"], d["n_cells"]
    p = np.zeros(n, oracle.PARTICLE_DTYPE)
    p["seed"] = oracle.rnd_seed_chain(d["base_seed"], n)
    if d["isotropic"]:
        seeds, reals = oracle.rnd_real(p["seed"])
        p["seed"] = seeds
        p["mu"] = reals if d["isotropic"] == 2 else (np.float32(2) * reals - np.float32(1))
    else:
        p["mu"] = d["mu0"]
    p["wmc"] = d["w0"]
    L = oracle.layer_make(0.0, 1.0, 0, m)
    return oracle.simulate_histories([L], sigs, rates, 1e-12, p, 2.0 ** 40)["tally_q"]


@pytest.fixture(scope="module")
def small_batch(built, mcg):
    from mc_mpi_gb300 import workloads
    return workloads.config2(n_slabs=24, seed=5, cells=(16, 300), hist=(300, 3000))


@pytest.mark.parametrize("mode", ["strict", "fast"])
def test_batch_equals_per_slab(mcg, small_batch, mode):
    slabs, sigs, rates = small_batch
    with mcg.Context(mode=mode) as ctx:
        ctx.set_tally_scale(40)
        ctx.batch_set(slabs, sigs, rates, 1e-12)
        ctx.batch_run()
        q_batch = ctx.batch_tally_q()
        c_batch = ctx.counters()
        ctx.batch_tally_reset()
        ctx.batch_run_per_slab()
        assert np.array_equal(ctx.batch_tally_q(), q_batch)
        assert ctx.counters()["steps"] == c_batch["steps"]
        assert c_batch["histories"] == sum(d["n_histories"] for d in slabs)


def test_batch_strict_matches_oracle(mcg, oracle, small_batch):
    slabs, sigs, rates = small_batch
    with mcg.Context(mode="strict") as ctx:
        ctx.set_tally_scale(40)
        ctx.batch_set(slabs, sigs, rates, 1e-12)
        ctx.batch_run()
        ctx.batch_run()  # the graph replays; tallies accumulate
        q = ctx.batch_tally_q()
    off = 0
    for d in slabs:
        m = d["n_cells"]
        ref = _oracle_slab(oracle, d, sigs[off:off + m], rates[off:off + m])
        assert np.array_equal(q[off:off + m], 2 * ref), f"slab with {m} cells differs"
        off += m


def test_batch_autotune_keeps_parity(mcg, small_batch):
    slabs, sigs, rates = small_batch
    with mcg.Context(mode="strict") as ctx:
        ctx.set_tally_scale(40)
        ctx.batch_set(slabs, sigs, rates, 1e-12)
        ctx.batch_run()
        ref = ctx.batch_tally_q()
        t = ctx.batch_autotune(0.3)
        assert t["candidates"] >= 6 and t["block"] in (256, 512, 1024)
        ctx.batch_run()
        assert np.array_equal(ctx.batch_tally_q(), ref)


@pytest.mark.parametrize("mode", ["strict", "fast"])
@pytest.mark.parametrize("k", [1, 8])
def test_batch_event_mode_equals_history(mcg, small_batch, mode, k):
    """The event-based batched form (all slabs' particles in one bank, K
    events per pass) gives the history-based form's tallies and counters."""
    slabs, sigs, rates = small_batch
    with mcg.Context(mode=mode) as ctx:
        ctx.set_tally_scale(40)
        ctx.batch_set(slabs, sigs, rates, 1e-12)
        ctx.batch_run()
        ref, c_ref = ctx.batch_tally_q(), ctx.counters()
        ctx.batch_tally_reset()
        ctx.batch_set_algorithm("event", k)
        ctx.batch_run()
        assert np.array_equal(ctx.batch_tally_q(), ref)
        c = ctx.counters()
        for key in ("histories", "steps", "scatters", "leaked_left", "leaked_right", "killed",
                    "w_left_q", "w_right_q", "w_killed_q", "error_flags"):
            assert c[key] == c_ref[key], key
