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


@pytest.mark.parametrize("mode", ["strict", "fast"])
def test_batch_deferral_equals_direct(mcg, small_batch, mode):
    """Deferring the full step until enough of a warp's lanes wait for it
    (1, 8 or 32 waiting lanes, the last only when no other lane can step)
    changes when a lane's steps run, not what they compute: tallies and
    counters equal."""
    slabs, sigs, rates = small_batch
    with mcg.Context(mode=mode) as ctx:
        ctx.set_tally_scale(40)
        ctx.batch_set(slabs, sigs, rates, 1e-12)
        ctx.batch_run()
        ref, c_ref = ctx.batch_tally_q(), ctx.counters()
        for lanes in (1, 8, 32):
            ctx.batch_tally_reset()
            ctx.batch_set_deferral(lanes)
            ctx.batch_run()
            assert np.array_equal(ctx.batch_tally_q(), ref), lanes
            c = ctx.counters()
            for key in ("histories", "steps", "scatters", "w_left_q", "w_right_q", "w_killed_q"):
                assert c[key] == c_ref[key], (lanes, key)


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


@pytest.fixture(scope="module")
def config2_ranges(built, mcg):
    """32 slabs drawn from configuration 2's full ranges: cells log-spread
    over [16, 4096] with both ends forced (4096 cells is the largest
    shared-memory tally of the batched kernel), L ~ U[0.5, 5], sigma_a ~
    U[0.1, 5], sigma_s ~ U[0, 10] per cell, and in every fourth slab a few
    cells whose interaction cross section sits at and around the reference's
    EPS (src/layer.cpp:137: sig_i <= 1e-4 means no collision), including 0;
    300 histories per slab from beam (mu = 1), half-isotropic (mu in [0, 1))
    and isotropic (mu in [-1, 1)) sources."""
    from mc_mpi_gb300 import workloads
    rng = np.random.default_rng(22)
    cells = np.unique(np.round(np.exp(rng.uniform(np.log(16), np.log(4096), 30)))).astype(int)
    cells = [16, 4096] + [int(c) for c in cells][: 30]
    slabs, sigs, rates, eps_cells = [], [], [], 0
    for s, m in enumerate(cells):
        L = float(rng.uniform(0.5, 5.0))
        sa = rng.uniform(0.1, 5.0, m).astype(np.float32)
        ss = rng.uniform(0.0, 10.0, m).astype(np.float32)
        if s % 4 == 1:
            k = rng.choice(m, size=min(m, 12), replace=False)
            near = np.float32(1e-4) / np.float32(L)
            ss[k] = np.array([0.0, near, np.nextafter(near, np.float32(0)),
                              np.nextafter(near, np.float32(1)), 0.5 * near, 2 * near,
                              1e-6, 3e-5, near * 0.999, near * 1.001, 1e-8, 5e-5],
                             np.float32)[: len(k)]
        g, r = workloads.sigs_rates(sa, ss, L)
        sig_i = g * (np.float32(1.0) - r.astype(np.float64)).astype(np.float32)
        eps_cells += int(np.count_nonzero(sig_i <= np.float32(1e-4)))
        sigs.append(g)
        rates.append(r)
        slabs.append(dict(n_cells=m, n_histories=300, base_seed=5127801 + 104729 * s,
                          seed_mode=0, isotropic=(0, 2, 1)[s % 3], mu0=1.0, w0=1.0))
    assert eps_cells >= 16  # the EPS branch is reachable in several slabs
    return slabs, np.concatenate(sigs), np.concatenate(rates)


@pytest.mark.parametrize("algorithm", ["history", "deferred", "event"])
def test_batch_config2_ranges_match_oracle(mcg, oracle, config2_ranges, algorithm):
    """Strict batched tallies of slabs across configuration 2's ranges equal
    the oracle's per slab, bit for bit, for the history-based and the
    event-based batched forms and for one launch per slab."""
    slabs, sigs, rates = config2_ranges
    with mcg.Context(mode="strict") as ctx:
        ctx.set_tally_scale(40)
        ctx.batch_set(slabs, sigs, rates, 1e-12)
        if algorithm == "event":
            ctx.batch_set_algorithm("event", 4)
        if algorithm == "deferred":
            ctx.batch_set_deferral(True)
        ctx.batch_run()
        q = ctx.batch_tally_q()
        ctx.batch_tally_reset()
        ctx.batch_run_per_slab()
        q_per_slab = ctx.batch_tally_q()
    assert np.array_equal(q, q_per_slab)
    off = 0
    for d in slabs:
        m = d["n_cells"]
        ref = _oracle_slab(oracle, d, sigs[off:off + m], rates[off:off + m])
        assert np.array_equal(q[off:off + m], ref), f"slab with {m} cells differs"
        off += m
