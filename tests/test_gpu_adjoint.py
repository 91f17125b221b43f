"""Adjoint gradients of a tally loss (configuration 3 physics: 1000 cells on
[0, 2], sigma_a ~ U[0.2, 2], sigma_s ~ U[0.5, 5], loss weights ~ N(0, 1)).

* the forward pass of the adjoint kernel produces the tracker's tally bit for
  bit;
* gradients agree with the FP64 CPU estimator within standard errors
  (batch means over independent history batches);
* central finite differences with common random numbers (h = 1e-3
  relative) on 32 random cells agree with the adjoint within their standard
  error.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

M, L = 1000, 2.0


def _problem(seed=3):
    rng = np.random.default_rng(seed)
    sa = rng.uniform(0.2, 2.0, M).astype(np.float32)
    ss = rng.uniform(0.5, 5.0, M).astype(np.float32)
    w = rng.standard_normal(M).astype(np.float32)
    return (sa * np.float32(L)).astype(np.float32), (ss * np.float32(L)).astype(np.float32), w


def _sr(sig_a, sig_s):
    sigs = (sig_a + sig_s).astype(np.float32)
    return sigs, (sig_a / sigs).astype(np.float32)


def _ctx(mcg, mode, sig_a, sig_s, w):
    ctx = mcg.Context(mode=mode)
    ctx.set_layers_xs([0], [M], [np.float32(1.0 / M)], sig_a, sig_s, 1e-12)
    ctx.adjoint_set_weights(w)
    return ctx


@pytest.mark.parametrize("mode", ["strict", "fast"])
def test_forward_tally_equals_tracker(mcg, mode):
    sig_a, sig_s, w = _problem()
    ctx = _ctx(mcg, mode, sig_a, sig_s, w)
    ctx.simulate_source(0, 50000)
    ref = ctx.tally_q()
    for with_grad in (False, True):
        ctx.adjoint_reset()
        ctx.adjoint_run(0, 50000, with_gradient=with_grad)
        assert np.array_equal(ctx.tally_q(), ref)
        loss, _, _ = ctx.adjoint_read()
        assert abs(loss - (ctx.tally() * w).sum() / 50000) < 1e-6
    ctx.close()


def test_adjoint_matches_fp64_estimator(mcg, oracle):
    sig_a, sig_s, w = _problem()
    ctx = _ctx(mcg, "fast", sig_a, sig_s, w)
    K, nb = 8, 25000
    gpu_a, gpu_s, cpu_a, cpu_s = [], [], [], []
    lay = [oracle.layer_make(0.0, 1.0, 0, M)]
    sa64, ss64 = sig_a.astype(np.float64), sig_s.astype(np.float64)
    for b in range(K):
        ctx.adjoint_reset()
        ctx.adjoint_run(b * nb, nb)
        _, ga, gs = ctx.adjoint_read()
        gpu_a.append(ga)
        gpu_s.append(gs)
        p = np.zeros(nb, oracle.PARTICLE_DTYPE)
        p["seed"] = oracle.rnd_seed_chain(oracle.lcg_skip(5127801, b * nb, True), nb)
        p["mu"], p["wmc"] = 1.0, 1.0
        _, ca, cs = oracle.fp64_adjoint(lay, sa64, ss64, w, 1e-12, p)
        cpu_a.append(ca / nb)
        cpu_s.append(cs / nb)
    ctx.close()
    for g, c in ((gpu_a, cpu_a), (gpu_s, cpu_s)):
        g, c = np.array(g), np.array(c)
        se = np.sqrt(g.var(axis=0, ddof=1) / K + c.var(axis=0, ddof=1) / K) + 1e-12
        z = np.abs(g.mean(0) - c.mean(0)) / se
        assert np.mean(z <= 3.0) >= 0.98, f"{np.mean(z > 3.0):.3%} of cells beyond 3 SE"
        assert z.max() <= 5.0


def _particles(oracle, first, n):
    p = np.zeros(n, oracle.PARTICLE_DTYPE)
    p["seed"] = oracle.rnd_seed_chain(oracle.lcg_skip(5127801, first, True), n)
    p["mu"], p["wmc"] = 1.0, 1.0
    return p


def _fd64(oracle, sig_a, sig_s, w, p, which, c, h):
    """Central difference of the FP64 loss (common random numbers: the same
    histories on both sides), per history."""
    lay = [oracle.layer_make(0.0, 1.0, 0, M)]
    out = []
    for sign in (+1, -1):
        a2, s2 = sig_a.astype(np.float64), sig_s.astype(np.float64)
        t = a2 if which == "a" else s2
        t[c] = float(np.float32(t[c] * (1.0 + sign * h)))
        loss, _, _ = oracle.fp64_adjoint(lay, a2, s2, w, 1e-12, p, with_gradient=False)
        out.append((loss / len(p), t[c]))
    (fp, xp), (fm, xm) = out
    return (fp - fm) / (xp - xm)


def test_finite_differences_common_random_numbers(mcg, oracle):
    """Central differences (h = 1e-3 relative) with common random numbers on
    32 random cells, taken on the FP64 forward: at this h the float32
    forward's own rounding (a deposit is quantised to the weight's ulp, ~3e-5
    of itself) would swamp the difference.
      sigma_a does not move the flights, so FD and the pathwise adjoint agree
      tightly on the same histories;
      sigma_s moves them (a flight near the face flips between crossing and
      collision), so FD and the likelihood-ratio adjoint are two estimators of
      the same derivative, compared within batch-means standard errors."""
    sig_a, sig_s, w = _problem()
    cells = np.random.default_rng(11).choice(M, 32, replace=False)
    h = 1e-3
    ctx = _ctx(mcg, "fast", sig_a, sig_s, w)
    # sigma_a: one batch of 20000 histories, tight agreement
    p = _particles(oracle, 0, 20000)
    ctx.adjoint_reset()
    ctx.adjoint_run(0, 20000)
    _, ga, _ = ctx.adjoint_read()
    fd_a = np.array([_fd64(oracle, sig_a, sig_s, w, p, "a", c, h) for c in cells])
    scale = np.abs(ga[cells]).max()
    assert np.allclose(ga[cells], fd_a, rtol=2e-3, atol=2e-4 * scale), \
        f"max rel dev {np.max(np.abs(ga[cells] - fd_a) / (np.abs(fd_a) + 1e-3 * scale)):.2e}"
    # sigma_s: K batches, z-scores of the difference of the two estimators
    K, nb = 8, 10000
    adj, fd = np.zeros((K, 32)), np.zeros((K, 32))
    for b in range(K):
        ctx.adjoint_reset()
        ctx.adjoint_run(b * nb, nb)
        adj[b] = ctx.adjoint_read()[2][cells]
        pb = _particles(oracle, b * nb, nb)
        fd[b] = [_fd64(oracle, sig_a, sig_s, w, pb, "s", c, h) for c in cells]
    ctx.close()
    se = np.sqrt(adj.var(axis=0, ddof=1) / K + fd.var(axis=0, ddof=1) / K) + 1e-12
    z = np.abs(adj.mean(0) - fd.mean(0)) / se
    assert np.mean(z <= 3.0) >= 0.9 and z.max() <= 5.0, f"z = {np.round(z, 2)}"
