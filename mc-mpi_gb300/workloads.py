"""Synthetic workloads of the benchmark configurations (seeded, reproducible).

The reference has no dataset; every input is generated from the formulas of
the configuration it stands for.  Cross sections are fp32 at cell centres;
a slab [0, L] is mapped onto the reference's Layer on [0, 1] by scaling its
cross sections by L (sigs = (sigma_a + sigma_s) L, rates = sigma_a / (sigma_a
+ sigma_s)), which leaves every optical depth, hence every tally, unchanged.
"""
import numpy as np

BASE_SEED = 5127801  # the seed decompose_domain uses (src/layer.cpp:36)


def sigs_rates(sigma_a, sigma_s, length=1.0):
    sa = np.asarray(sigma_a, np.float32)
    ss = np.asarray(sigma_s, np.float32)
    tot = (sa + ss).astype(np.float32)
    rates = np.where(tot > 0, sa / np.where(tot > 0, tot, 1), 0).astype(np.float32)
    return (tot * np.float32(length)).astype(np.float32), rates


def config0(m=100):
    """100 cells on [0, 1]: sigma_a = 0.2 + 1.8 x, sigma_s = 1."""
    xc = ((np.arange(m, dtype=np.float64) + 0.5) / m).astype(np.float32)
    return sigs_rates(np.float32(0.2) + np.float32(1.8) * xc, np.ones(m, np.float32))


def config1(nb=10000):
    """10,000 cells: sigma_a = 0.5 + 0.4 sin(6 pi x), sigma_s = 2 + 1.5 cos(4 pi x)."""
    xc = (np.arange(nb, dtype=np.float64) + 0.5) / nb
    return sigs_rates(0.5 + 0.4 * np.sin(6 * np.pi * xc), 2.0 + 1.5 * np.cos(4 * np.pi * xc))


def config2(n_slabs=4096, seed=2, cells=(16, 4096), hist=(1e3, 1e6), scale_histories=1.0):
    """Batched slabs: cells ~ U{16..4096}, L ~ U[0.5, 5], per-cell sigma_a ~
    U[0.1, 5], sigma_s ~ U[0, 10], histories log-uniform in [1e3, 1e6];
    sources at x = 0 with mu = 1 (even slabs) or mu ~ U[0, 1) (odd slabs).
    Returns (slab dicts, sigs, rates)."""
    rng = np.random.default_rng(seed)
    slabs, sigs, rates = [], [], []
    for s in range(n_slabs):
        m = int(rng.integers(cells[0], cells[1] + 1))
        L = float(rng.uniform(0.5, 5.0))
        sa = rng.uniform(0.1, 5.0, m).astype(np.float32)
        ss = rng.uniform(0.0, 10.0, m).astype(np.float32)
        n = int(round(np.exp(rng.uniform(np.log(hist[0]), np.log(hist[1]))) * scale_histories))
        g, r = sigs_rates(sa, ss, L)
        sigs.append(g)
        rates.append(r)
        slabs.append(dict(n_cells=m, n_histories=max(n, 1), base_seed=BASE_SEED + 7919 * s,
                          seed_mode=0, isotropic=0 if s % 2 == 0 else 2, mu0=1.0, w0=1.0,
                          length=L))
    return slabs, np.concatenate(sigs), np.concatenate(rates)


def config3(m=1000, length=2.0, seed=3):
    """Differentiation: m cells on [0, L], sigma_a ~ U[0.2, 2], sigma_s ~
    U[0.5, 5], loss weights ~ N(0, 1).  Returns the step's cross sections on
    the unit slab (sigma * L) and the weights."""
    rng = np.random.default_rng(seed)
    sa = rng.uniform(0.2, 2.0, m).astype(np.float32)
    ss = rng.uniform(0.5, 5.0, m).astype(np.float32)
    w = rng.standard_normal(m).astype(np.float32)
    L = np.float32(length)
    return (sa * L).astype(np.float32), (ss * L).astype(np.float32), w


def config4(n_slabs=64, cells=(64, 1024), seed=4, histories=1_000_000):
    """Inverse fit: n_slabs slabs on [0, 1], cells ~ U{64..1024}; hidden
    sigma_a(x) = 1 + 0.8 sin(2 pi k x + phi), k ~ U{1..4}, phi ~ U[0, 2 pi);
    sigma_s = 1.5; sources at x = 0, mu = 1.  Returns (slab dicts with
    `histories` per step, hidden sigma_a, sigma_s)."""
    rng = np.random.default_rng(seed)
    slabs, hidden, sig_s = [], [], []
    for s in range(n_slabs):
        m = int(rng.integers(cells[0], cells[1] + 1))
        k = int(rng.integers(1, 5))
        phi = float(rng.uniform(0.0, 2.0 * np.pi))
        xc = (np.arange(m, dtype=np.float64) + 0.5) / m
        hidden.append((1.0 + 0.8 * np.sin(2.0 * np.pi * k * xc + phi)).astype(np.float32))
        sig_s.append(np.full(m, 1.5, np.float32))
        slabs.append(dict(n_cells=m, n_histories=histories, base_seed=BASE_SEED + 104729 * s,
                          seed_mode=0, isotropic=0, mu0=1.0, w0=1.0))
    return slabs, np.concatenate(hidden), np.concatenate(sig_s)
