"""Randomised single-layer cases shared by the oracle-vs-reference tests
(CPU) and the GPU-vs-oracle tests: layers inside and at the borders of
[0, 1], cells from vacuum to optically thick, cross sections at and around
the EPS threshold, particles anywhere in the layer with any direction (0,
-0, +-EPS, +-1 included) and weights around the minimum."""
import numpy as np

f32 = np.float32


def case(seed):
    rng = np.random.default_rng(seed)
    m = int(rng.integers(1, 300))
    kind = seed % 4
    if kind == 0:  # a whole [0, 1] slab: both borders
        x_min, x_max, start = 0.0, 1.0, 0
    elif kind == 1:  # an interior sub-domain
        start = int(rng.integers(1, 5000))
        dx = 1.0 / (start + m + int(rng.integers(1, 5000)))
        x_min, x_max = start * dx, (start + m) * dx
    elif kind == 2:  # touching the left border only
        start, x_min, x_max = 0, 0.0, float(rng.uniform(0.05, 0.9))
    else:  # touching the right border only
        start = int(rng.integers(1, 2000))
        x_min, x_max = float(rng.uniform(0.1, 0.95)), 1.0
    width = x_max - x_min
    # optical thickness of the layer up to ~40 for scattering and absorption
    sa = rng.uniform(0, 40 / width, m) * (rng.random(m) < 0.9)
    ss = rng.uniform(0, 40 / width, m) * (rng.random(m) < 0.85)
    eps_cells = rng.random(m) < 0.1  # sig_s around the 1e-4 threshold
    ss[eps_cells] = rng.choice([0.0, 5e-5, 1e-4, 1.0001e-4, 2e-4], eps_cells.sum())
    sigs = (sa + ss).astype(f32)
    with np.errstate(invalid="ignore", divide="ignore"):
        rates = np.where(sigs > 0, sa.astype(f32) / np.maximum(sigs, f32(1e-30)), 0.5).astype(f32)
    return rng, m, f32(x_min), f32(x_max), start, sigs, rates


def particles(rng, dtype, L, n):
    p = np.zeros(n, dtype)
    p["seed"] = rng.integers(0, 2**63, n, dtype=np.uint64)
    cell = rng.integers(0, L.m, n)
    frac = rng.random(n)
    frac[rng.random(n) < 0.1] = 0.0  # on a cell's left edge
    x = ((cell + frac) * np.float64(L.dx) + np.float64(L.index_start) * np.float64(L.dx))
    p["x"] = x.astype(f32)
    p["index"] = cell + L.index_start
    mu = rng.uniform(-1, 1, n)
    special = rng.random(n) < 0.15
    mu[special] = rng.choice([0.0, -0.0, 1e-4, -1e-4, 1.0001e-4, 1e-5, 1.0, -1.0], special.sum())
    p["mu"] = mu.astype(f32)
    w = rng.uniform(0, 1, n)
    low = rng.random(n) < 0.05
    w[low] = rng.choice([1e-12, 9.9e-13, 2e-12, 0.0], low.sum())
    p["wmc"] = w.astype(f32)
    return p
