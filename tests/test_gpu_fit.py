"""Batched inverse fit (configuration 4 physics at reduced size): recover
per-cell absorption cross sections of several slabs from their absorption
tallies by Adam on batched forward+adjoint steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_inverse_fit_recovers_sigma_a(mcg):
    from mc_mpi_gb300 import workloads
    slabs, hidden, sig_s = workloads.config4(n_slabs=8, cells=(64, 256), histories=200_000)
    tslabs = [dict(d, n_histories=2_000_000, base_seed=d["base_seed"] + 1) for d in slabs]
    sigs = (hidden + sig_s).astype(np.float32)
    rates = (hidden / sigs).astype(np.float32)
    with mcg.Context(mode="fast") as ctx:
        ctx.batch_set(tslabs, sigs, rates, 1e-12)
        ctx.batch_run()
        tally = ctx.batch_tally()
        n_per_cell = np.concatenate([np.full(d["n_cells"], d["n_histories"]) for d in tslabs])
        target = tally / n_per_cell
        ctx.fit_set(slabs, np.ones_like(hidden), sig_s, target, max_steps=200)
        ctx.fit_run(150, lr=1e-2)
        sig, loss = ctx.fit_read()
    err0 = np.linalg.norm(1.0 - hidden) / np.linalg.norm(hidden)
    err = np.linalg.norm(sig - hidden) / np.linalg.norm(hidden)
    assert len(loss) == 150
    assert err < 0.35 * err0, f"relative L2 error {err:.3f} (start {err0:.3f})"
    assert loss[-10:].mean() < 0.1 * loss[0]


def test_fit_gradient_matches_adjoint(mcg):
    """The fit's fused forward+adjoint kernel against the adjoint form
    (mcg_adjoint_run, whose gradients are checked against the FP64 CPU
    estimator and finite differences) on the same histories, cross sections
    and loss weights: the absorbed weight per history bit for bit (both are
    exact fixed-point sums of the same deposits) and dF/dsig_a within the
    rounding of their fp32 accumulations (a relative 1e-4 of the largest
    component)."""
    rng = np.random.default_rng(12)
    m, n, seed = 300, 200_000, 5127801 + 17
    sig_a = rng.uniform(0.5, 2.0, m).astype(np.float32)
    sig_s = np.full(m, 1.5, np.float32)
    w = rng.standard_normal(m)
    slab = dict(n_cells=m, n_histories=n, base_seed=seed, seed_mode=0, isotropic=0, mu0=1.0,
                w0=1.0)
    with mcg.Context(mode="fast") as ctx:
        ctx.fit_set([slab], sig_a, sig_s, np.zeros(m), max_steps=4)
        t_fit, g_fit = ctx.fit_gradient(w)
        # the fit's own state is untouched: an Adam step still runs
        ctx.fit_run(1)
        assert len(ctx.fit_read()[1]) == 1
    with mcg.Context(mode="fast") as ctx:
        ctx.set_layers_xs([0], [m], [np.float32(1.0 / m)], sig_a, sig_s, 1e-12)
        ctx.adjoint_set_weights(w.astype(np.float32))
        ctx.adjoint_reset()
        ctx.adjoint_run(0, n, with_gradient=True, seed_mode=0, base_seed=seed)
        _, g_adj, _ = ctx.adjoint_read()
        t_adj = ctx.tally() / n
    assert np.array_equal(t_fit, t_adj)
    scale = np.abs(g_adj).max()
    assert scale > 0
    assert np.abs(g_fit - g_adj).max() <= 1e-4 * scale, np.abs(g_fit - g_adj).max() / scale
