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
