#!/usr/bin/env python3
"""Regenerate the golden fixtures of tests/golden/ from the REFERENCE's own
code: oracle/_ref/libmcref.so, i.e. lkskstlr/mc-mpi's src/layer.cpp and
src/random.cpp compiled in place by `make -C oracle ref` (needs the reference
checkout, so this runs where the reference is mounted, not on the GPU machine).

Fixtures:
  test_layer_WA.out   Layer::dump_WA of src/test_layer.cpp's case (100 cells,
                      100 particles, x_ini = sqrt(2)/2, min weight 0): equal
                      to the reference's data/test_layer_target_WA.out.
  rng_chain.npz       10000 rnd_seed values from 30061994 (the start of
                      src/test_curandom.cu) and one rnd_real step of each.
  particle_hash.npz   FNV-1a hash of src/test_async_serialization.cpp's
                      particle as the reference lays it out.
  traces_*.npz        per-particle histories through the reference's public
                      Layer::particle_step with simulate_particle's loop:
                      initial and final particles, result, steps, scatters
                      (traces_edge: the step's special cases, see
                      edge_case_physics and edge_case_particles).
  decomposed_*.npz    reference float tallies of a decomposed slab driven by
                      the WorkerSync cycle over Layer::simulate.
"""
import ctypes as C
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

f32 = np.float32


def physics_config0(m):
    """sigma_a = 0.2 + 1.8 x, sigma_s = 1.0 at cell centres (fp32)."""
    xc = ((np.arange(m, dtype=np.float64) + 0.5) / m).astype(np.float32)
    sa = (f32(0.2) + f32(1.8) * xc).astype(np.float32)
    ss = np.full(m, 1.0, np.float32)
    return sigs_rates(sa, ss)


def sigs_rates(sa, ss):
    sig = (sa + ss).astype(np.float32)
    rate = (sa / sig).astype(np.float32)
    return sig, rate


def chain_particles(n, x0, mu0, w0, cell0, base=5127801):
    seeds = np.empty(n, np.uint64)
    s = C.c_uint64(base)
    for i in range(n):
        seeds[i] = O.lib().orc_rnd_seed(C.byref(s))
    p = np.zeros(n, O.PARTICLE_DTYPE)
    p["seed"] = seeds
    p["x"] = x0
    p["mu"] = mu0
    p["wmc"] = w0
    p["index"] = cell0
    return p


def ref_traces(name, L, sigs, rates, min_w, particles):
    R = O.ref()
    fin = particles.copy()
    tr = np.zeros(len(particles), O.TRACE_DTYPE)
    R.ref_trace_particles(L.x_min, L.x_max, L.index_start, L.m, min_w, O._p(sigs), O._p(rates),
                          O._p(fin), len(fin), O._p(tr))
    np.savez_compressed(os.path.join(HERE, f"traces_{name}.npz"), layer=np.array(L.as_tuple()),
                        sigs=sigs, rates=rates, min_w=np.float32(min_w), initial=particles,
                        final=fin, result=tr["result"], steps=tr["steps"],
                        scatters=tr["scatters"])
    print(f"traces_{name}: n={len(fin)} mean steps {tr['steps'].mean():.1f}")


def edge_case_physics(m):
    """Cells cycling through the step's special cases: vacuum (sigs = 0),
    pure absorber (rate 1, sig_i = 0), sig_i on the EPS threshold
    (2e-4 * 0.5), optically thick scatterer and absorber (exp arguments
    below -17.5), and an ordinary cell."""
    kinds = [(0.0, 0.5), (3.0, 1.0), (2e-4, 0.5), (5000.0, 0.3), (2000.0, 0.99), (2.5, 0.2)]
    sigs = np.array([kinds[i % 6][0] for i in range(m)], np.float32)
    rates = np.array([kinds[i % 6][1] for i in range(m)], np.float32)
    return sigs, rates


def edge_case_particles(L, n, base=424242):
    """Particles mixing ordinary starts with the special ones: directions 0,
    -0, +-1e-4 (the EPS threshold), 1e-5, +-1; positions exactly on cell
    edges (either neighbouring index) and one ulp past them; indices just
    outside the layer; weights at, below and far below the minimum."""
    rng = np.random.default_rng(7)
    p = chain_particles(n, 0.0, 1.0, 1.0, L.index_start, base)
    cells = rng.integers(L.index_start, L.index_start + L.m, n)
    frac = rng.random(n).astype(np.float32)
    x = ((cells.astype(np.float32) + frac) * f32(L.dx)).astype(np.float32)
    idx = cells.astype(np.int32)
    mu = rng.uniform(-1.0, 1.0, n).astype(np.float32)
    w = np.ones(n, np.float32)
    special_mu = np.array([0.0, -0.0, 1e-4, -1e-4, 1.0001e-4, 1e-5, 1.0, -1.0], np.float32)
    k = rng.integers(0, 10, n)
    pick = k < 3
    mu[pick] = special_mu[rng.integers(0, len(special_mu), pick.sum())]
    edge = k == 3                        # on the left edge of the cell
    x[edge] = (cells[edge].astype(np.float32) * f32(L.dx)).astype(np.float32)
    edge_r = k == 4                      # on the same edge, owned by the cell before
    x[edge_r] = (cells[edge_r].astype(np.float32) * f32(L.dx)).astype(np.float32)
    idx[edge_r] = np.maximum(cells[edge_r] - 1, L.index_start)
    past = k == 5                        # one ulp past the left edge, inwards and out
    e = (cells[past].astype(np.float32) * f32(L.dx)).astype(np.float32)
    x[past] = np.where(rng.random(past.sum()) < 0.5, np.nextafter(e, f32(-1)),
                       np.nextafter(e, f32(2))).astype(np.float32)
    low = k == 6
    w[low] = np.array([1e-12, 9e-13, 0.0, 1.5e-12], np.float32)[rng.integers(0, 4, low.sum())]
    out = k == 7
    idx[out] = np.array([L.index_start - 1, L.index_start + L.m, L.index_start - 5],
                        np.int32)[rng.integers(0, 3, out.sum())]
    p["x"], p["mu"], p["wmc"], p["index"] = x, mu, w, idx
    return p


def main():
    if not O.ref_available():
        O.build()
    R = O.ref()
    R.ref_rng_chain.argtypes = [C.c_uint64, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    R.ref_particle_hash.restype = C.c_int

    # 1. golden WA.out of src/test_layer.cpp
    buf = C.create_string_buffer(1 << 20)
    with tempfile.TemporaryDirectory() as d:
        n = R.ref_test_layer_wa(d.encode(), buf, 1 << 20, 1)
    assert n > 0
    with open(os.path.join(HERE, "test_layer_WA.out"), "w") as f:
        f.write(buf.value.decode())

    # 2. RNG chain of src/test_curandom.cu
    n = 10000
    s0 = np.zeros(n, np.uint64)
    s1 = np.zeros(n, np.uint64)
    r = np.zeros(n, np.float32)
    R.ref_rng_chain(30061994, n, O._p(s0), O._p(s1), O._p(r))
    np.savez_compressed(os.path.join(HERE, "rng_chain.npz"), start=np.uint64(30061994), seeds=s0,
                        seeds_after=s1, reals=r)

    # 3. particle wire layout
    np.savez_compressed(os.path.join(HERE, "particle_hash.npz"),
                        hash=np.int32(R.ref_particle_hash()))

    # 4. per-particle traces
    # 4a. configuration 0 physics: 100 cells, from x=0 mu=1 w=1, min weight 1e-12
    L = O.layer_make(0.0, 1.0, 0, 100)
    sigs, rates = physics_config0(100)
    ref_traces("config0", L, sigs, rates, 1e-12, chain_particles(4000, 0.0, 1.0, 1.0, 0))
    # 4b. the reference's default physics with its own particle source
    L = O.decompose(0.0, 1.0, 1000, 1)[0]
    sigs, rates = O.default_sigs(L)
    x_ini = f32(np.sqrt(f32(2.0)) / f32(2.0))
    ps = O.create_particles(L, float(x_ini), float(f32(1.0 / 2000)), 2000, 5127801)
    ref_traces("default1000", L, sigs, rates, 0.0, ps)
    # 4c. a middle sub-domain (cells 157..313 of a 10000-cell slab in 64 layers)
    layers = O.decompose(0.0, 1.0, 10000, 64)
    L = layers[1]
    xc = ((np.arange(L.index_start, L.index_start + L.m) + 0.5) / 10000.0)
    sa = (0.5 + 0.4 * np.sin(6 * np.pi * xc)).astype(np.float32)
    ss = (2.0 + 1.5 * np.cos(4 * np.pi * xc)).astype(np.float32)
    sigs, rates = sigs_rates(sa, ss)
    ps = chain_particles(2000, float(f32(L.index_start) * L.dx), 1.0, 1.0, L.index_start)
    ref_traces("sublayer", L, sigs, rates, 1e-12, ps)

    # 4d. edge cases of particle_step / simulate_particle on a middle
    # sub-domain (cells 60..119 of 240 in 4 layers)
    L = O.decompose(0.0, 1.0, 240, 4)[1]
    sigs, rates = edge_case_physics(L.m)
    ref_traces("edge", L, sigs, rates, 1e-12, edge_case_particles(L, 4000))

    # 5. decomposed slab: reference float tallies (WorkerSync cycle)
    nb, P, N = 1000, 8, 4000
    xc = ((np.arange(nb) + 0.5) / nb)
    sa = (0.5 + 0.4 * np.sin(6 * np.pi * xc)).astype(np.float32)
    ss = (2.0 + 1.5 * np.cos(4 * np.pi * xc)).astype(np.float32)
    sigs, rates = sigs_rates(sa, ss)
    ps = chain_particles(N, 0.0, 1.0, 1.0, 0)
    tally = np.zeros(nb, np.float64)
    cycles = R.ref_decomposed(0.0, 1.0, nb, P, 1e-12, O._p(sigs), O._p(rates), O._p(ps), N, 500, 1,
                              O._p(tally))
    np.savez_compressed(os.path.join(HERE, "decomposed_1000x8.npz"), sigs=sigs, rates=rates,
                        particles=ps, tally=tally, n_layers=np.int32(P), cycles=np.int32(cycles),
                        min_w=np.float32(1e-12))
    print("decomposed: cycles", cycles, "total", tally.sum())


if __name__ == "__main__":
    main()
