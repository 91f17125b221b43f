"""The synthetic inputs stand in for the benchmark configurations: their
shapes, sizes and value distributions follow the configurations' formulas
(slab counts, cell-count and length ranges, cross-section ranges, history
counts, source directions), and the benchmark's own slab is configuration 1."""
import numpy as np

f32 = np.float32


def test_config0_and_config1_formulas(mcg):
    from mc_mpi_gb300 import workloads
    import bench
    sigs, rates = workloads.config0()
    xc = ((np.arange(100) + 0.5) / 100).astype(f32)
    sa = (f32(0.2) + f32(1.8) * xc).astype(f32)
    assert np.array_equal(sigs, (sa + f32(1.0)).astype(f32))
    assert np.allclose(rates * sigs, sa, rtol=1e-6)
    s1, r1 = workloads.config1()
    b1, br1 = bench.physics()
    assert np.array_equal(s1, b1) and np.array_equal(r1, br1)
    assert len(s1) == 10000


def test_config2_shapes_and_ranges(mcg):
    from mc_mpi_gb300 import workloads
    slabs, sigs, rates = workloads.config2()
    assert len(slabs) == 4096
    cells = np.array([d["n_cells"] for d in slabs])
    hist = np.array([d["n_histories"] for d in slabs])
    length = np.array([d["length"] for d in slabs])
    assert cells.min() >= 16 and cells.max() <= 4096
    assert abs(cells.mean() - 2056) < 60  # U{16..4096}
    assert length.min() >= 0.5 and length.max() <= 5.0
    assert hist.min() >= 1000 and hist.max() <= 1_000_000
    # log-uniform on [1e3, 1e6]: mean (1e6 - 1e3) / ln(1e3) ~ 1.45e5
    assert 5.0e8 < hist.sum() < 6.9e8
    assert len(sigs) == len(rates) == cells.sum()
    # per-cell sigma_a ~ U[0.1, 5], sigma_s ~ U[0, 10], scaled by the slab's length
    per_len = np.concatenate([np.full(c, L, np.float32) for c, L in zip(cells, length)])
    tot = sigs / per_len
    sa = tot * rates
    assert sa.min() >= 0.1 * (1 - 1e-5) and sa.max() <= 5.0 * (1 + 1e-5)
    assert (tot - sa).min() >= -1e-4 and (tot - sa).max() <= 10.0 * (1 + 1e-5)
    iso = np.array([d["isotropic"] for d in slabs])
    assert np.count_nonzero(iso == 0) == 2048 and np.count_nonzero(iso == 2) == 2048
    # distinct seeds per slab
    assert len({d["base_seed"] for d in slabs}) == 4096


def test_config3_and_config4(mcg):
    from mc_mpi_gb300 import workloads
    sa, ss, w = workloads.config3()
    assert len(sa) == len(ss) == len(w) == 1000
    assert sa.min() >= 0.2 * 2 and sa.max() <= 2.0 * 2  # sigma * L, L = 2
    assert ss.min() >= 0.5 * 2 and ss.max() <= 5.0 * 2
    assert abs(float(w.mean())) < 0.1 and abs(float(w.std()) - 1.0) < 0.1
    slabs, hidden, sig_s = workloads.config4()
    assert len(slabs) == 64
    cells = np.array([d["n_cells"] for d in slabs])
    assert cells.min() >= 64 and cells.max() <= 1024 and len(hidden) == cells.sum()
    assert hidden.min() >= 0.2 - 1e-6 and hidden.max() <= 1.8 + 1e-6
    assert np.all(sig_s == f32(1.5))
    assert all(d["n_histories"] == 1_000_000 for d in slabs)
