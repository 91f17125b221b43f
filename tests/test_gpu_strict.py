"""GPU parity of the strict tracker against the oracle and the reference's
golden data: bit-exact per particle, exact fixed-point tallies.

Mirrors src/test_layer.cpp (golden WA.out through the GPU Layer),
src/test_culayer.cu (cusimulate vs CPU) and src/test_curandom.cu (RNG)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
f32 = np.float32
SCALE = 40


def load(name):
    return np.load(os.path.join(GOLDEN, name))


@pytest.fixture(scope="module")
def ctx(built, mcg):
    c = mcg.Context(mode="strict")
    yield c
    c.close()


def oracle_q(oracle, layers, sigs, rates, min_w, particles):
    return oracle.simulate_histories(list(layers), sigs, rates, min_w, particles, 2.0 ** SCALE)


@pytest.mark.parametrize("name", ["config0", "default1000", "sublayer", "edge"])
def test_golden_traces_bit_exact(ctx, mcg, name):
    g = load(f"traces_{name}.npz")
    lt = g["layer"]
    ctx.set_layers([int(lt[3])], [int(lt[4])], [f32(lt[2])], g["sigs"], g["rates"],
                   float(g["min_w"]))
    p = g["initial"].astype(mcg.PARTICLE_DTYPE).copy()
    r = ctx.simulate(p)
    assert p.tobytes() == g["final"].astype(mcg.PARTICLE_DTYPE).tobytes()
    assert np.array_equal(r["results"], g["result"])
    assert np.array_equal(r["steps"], g["steps"])
    assert np.array_equal(r["scatters"], g["scatters"])


@pytest.mark.parametrize("name", ["config0", "edge"])
def test_tally_fixed_point_exact(ctx, mcg, oracle, name):
    """The int64 tally equals the oracle's sum of llrint(dw * 2^S)."""
    g = load(f"traces_{name}.npz")
    lt = g["layer"]
    L = oracle.layer_make(float(lt[0]), float(lt[1]), int(lt[3]), int(lt[4]))
    ctx.set_layers([int(lt[3])], [int(lt[4])], [f32(lt[2])], g["sigs"], g["rates"], 1e-12)
    p = g["initial"].astype(mcg.PARTICLE_DTYPE).copy()
    ctx.simulate(p)
    # the oracle's chain driver indexes cross sections and tallies by global cell
    s0 = int(lt[3])
    pad = np.zeros(s0, np.float32)
    ref = oracle_q(oracle, [L], np.concatenate([pad, g["sigs"]]),
                   np.concatenate([pad, g["rates"]]), 1e-12, g["initial"])
    assert np.array_equal(ctx.tally_q(), ref["tally_q"][s0:])
    c = ctx.counters()
    assert c["histories"] == len(p) and c["steps"] == int(g["steps"].sum())
    assert c["scatters"] == int(g["scatters"].sum())


def test_decomposed_chain_bit_exact(ctx, mcg, oracle):
    """64 sub-domains of a 10000-cell slab (per-layer dx, as decompose_domain)
    in one context: per-particle and tally parity with the oracle's
    layer-by-layer hand-over."""
    nb, P, N = 10000, 64, 3000
    st, m, dx, _, _ = mcg.layer_decomposition(0.0, 1.0, nb, P)
    xc = (np.arange(nb) + 0.5) / nb
    sa = (0.5 + 0.4 * np.sin(6 * np.pi * xc)).astype(np.float32)
    ss = (2.0 + 1.5 * np.cos(4 * np.pi * xc)).astype(np.float32)
    sigs = (sa + ss).astype(np.float32)
    rates = (sa / sigs).astype(np.float32)
    ctx.set_layers(st, m, dx, sigs, rates, 1e-12)
    p = np.zeros(N, mcg.PARTICLE_DTYPE)
    p["seed"] = oracle.rnd_seed_chain(5127801, N)
    p["x"], p["mu"], p["wmc"], p["index"] = 0.0, 1.0, 1.0, 0
    init = p.copy()
    r = ctx.simulate(p)
    layers = oracle.decompose(0.0, 1.0, nb, P)
    ref = oracle_q(oracle, layers, sigs, rates, 1e-12, init)
    assert p.tobytes() == ref["particles"].tobytes()
    assert np.array_equal(r["steps"], ref["traces"]["steps"])
    assert np.array_equal(r["results"], ref["traces"]["result"])
    assert np.array_equal(ctx.tally_q(), ref["tally_q"])


def test_source_mode_matches_host_particles(ctx, mcg, oracle):
    """Device-born particles (seed chain jump-ahead) = host-built particles."""
    nb = 100
    g = load("traces_config0.npz")
    ctx.set_layers([0], [nb], [f32(1.0 / nb)], g["sigs"], g["rates"], 1e-12)
    ctx.simulate_source(0, 4000, seed_mode=0, base_seed=5127801, x0=0.0, mu0=1.0, w0=1.0)
    q_src = ctx.tally_q()
    c = ctx.counters()
    assert c["steps"] == int(g["steps"].sum())
    ctx.tally_reset()
    p = g["initial"].astype(mcg.PARTICLE_DTYPE).copy()
    ctx.simulate(p)
    assert np.array_equal(ctx.tally_q(), q_src)


def test_golden_wa_through_gpu_layer(mcg):
    """src/test_layer.cpp through the GPU Layer: WA.out byte-identical."""
    x_ini = f32(np.sqrt(f32(2.0)) / f32(2.0))
    layer = mcg.decompose_domain(0.0, 1.0, x_ini, 1, 0, 100, 100, 0.0)
    layer.simulate(-1)
    with open(os.path.join(GOLDEN, "test_layer_WA.out")) as f:
        assert layer.format_WA() == f.read()
    assert layer.nb_disabled == 100


def test_cusimulate_dropin(mcg, oracle):
    """src/test_culayer.cu: 1000 cells, default physics, every particle's final
    state written back, tallies within 1e-4 of the CPU (exact here)."""
    n, m = 20000, 1000
    L = oracle.decompose(0.0, 1.0, m, 1)[0]
    sigs, rates = oracle.default_sigs(L)
    x_ini = f32(np.sqrt(f32(2.0)) / f32(2.0))
    ps = oracle.create_particles(L, float(x_ini), float(f32(1.0 / n)), n, 5127801)
    cpu = oracle.layer_simulate(L, sigs, rates, 0.0, ps[::-1].copy(), n)
    gp = ps.astype(mcg.PARTICLE_DTYPE).copy()
    w = np.zeros(m, np.float32)
    mcg.cusimulate(gp, sigs, rates, w, 0, m, L.dx)
    assert gp.tobytes() == cpu["particles"][::-1].tobytes()
    assert np.max(np.abs(w - cpu["tally_f32"])) < 1e-4


def test_layer_api_simulate_batches(mcg, oracle):
    """Layer.simulate(n) consumes from the back, classifies leavers in
    processing order and accumulates weights_absorbed."""
    layer = mcg.Layer(0.25, 0.5, 25, 25, 1e-12)
    rng = np.random.default_rng(3)
    p = np.zeros(5000, mcg.PARTICLE_DTYPE)
    p["seed"] = rng.integers(0, 2**63, 5000, dtype=np.uint64)
    p["x"] = f32(0.3)
    p["mu"] = rng.uniform(-1, 1, 5000).astype(np.float32)
    p["wmc"] = 1.0
    p["index"] = 30
    layer.particles = p.copy()
    layer.simulate(3000)
    assert len(layer.particles) == 2000
    L = oracle.layer_make(0.25, 0.5, 25, 25)
    ref = oracle.layer_simulate(L, layer.sigs, layer.absorption_rates, 1e-12, p.copy(), 3000)
    res = ref["results"]
    proc = ref["particles"][len(p) - 3000:][::-1]
    assert layer.particles_left.tobytes() == proc[res == -1].tobytes()
    assert layer.particles_right.tobytes() == proc[res == 1].tobytes()
    assert layer.nb_disabled == int(np.count_nonzero(res == 0))
    assert np.allclose(layer.weights_absorbed, ref["tally_f32"], rtol=1e-5, atol=1e-6)


def test_simulate_pinned_buffers_in_place(ctx, mcg, oracle):
    """mcg_simulate on page-locked host buffers (read and written in place by
    the GPU) equals the staged path on pageable copies of the same
    particles, byte for byte, results, steps and tallies included."""
    import ctypes as C
    import torch
    nb, P, N = 10000, 64, 20000
    st, m, dx, _, _ = mcg.layer_decomposition(0.0, 1.0, nb, P)
    xc = (np.arange(nb) + 0.5) / nb
    sa = (0.5 + 0.4 * np.sin(6 * np.pi * xc)).astype(np.float32)
    ss = (2.0 + 1.5 * np.cos(4 * np.pi * xc)).astype(np.float32)
    sigs = (sa + ss).astype(np.float32)
    ctx.set_layers(st, m, dx, sigs, (sa / sigs).astype(np.float32), 1e-12)
    p = np.zeros(N, mcg.PARTICLE_DTYPE)
    p["seed"] = oracle.rnd_seed_chain(77, N)
    p["mu"], p["wmc"] = 1.0, 1.0
    staged = p.copy()
    ctx.tally_reset()
    r0 = ctx.simulate(staged)
    q0 = ctx.tally_q()
    hp = torch.from_numpy(p.view(np.uint8).copy()).pin_memory()
    hr = torch.full((N,), 9, dtype=torch.int32).pin_memory()
    hs = torch.zeros(N, dtype=torch.int64).pin_memory()
    hc = torch.zeros(N, dtype=torch.int64).pin_memory()
    ctx.tally_reset()
    rc = ctx.lib.mcg_simulate(ctx.h, C.c_void_p(hp.data_ptr()), N, C.c_void_p(hr.data_ptr()),
                              C.c_void_p(hs.data_ptr()), C.c_void_p(hc.data_ptr()))
    assert rc == 0, ctx.lib.mcg_last_error().decode()
    assert hp.numpy().tobytes() == staged.tobytes()
    assert np.array_equal(hr.numpy(), r0["results"])
    assert np.array_equal(hs.numpy(), r0["steps"])
    assert np.array_equal(hc.numpy(), r0["scatters"])
    assert np.array_equal(ctx.tally_q(), q0)


@pytest.mark.parametrize("mode", ["strict", "fast"])
def test_tally_independent_of_launch_shape(mcg, oracle, mode):
    """The fixed-point tally is a sum of integers: every launch shape (block
    size, blocks per SM, refill interval) and tally privatisation (64-bit
    shared, 32-bit shared with carry, global) gives the same bits and the
    same counters."""
    st, m, dx, sigs, rates = _slab(mcg, 2000, 16)
    with mcg.Context(mode=mode) as ctx:
        ctx.set_layers(st, m, dx, sigs, rates, 1e-12)
        ref = ref_c = None
        for block, bps, refill in ((0, 0, 0), (256, 2, 1), (1024, 1, 32), (512, 0, 8)):
            for tmode in (0, 1, 2):
                ctx.set_launch(block, bps, refill)
                ctx.set_tally_mode(tmode)
                ctx.tally_reset()
                ctx.simulate_source(0, 20000)
                q, c = ctx.tally_q(), ctx.counters()
                if ref is None:
                    ref, ref_c = q, c
                assert np.array_equal(q, ref), (block, bps, refill, tmode)
                assert c == ref_c, (block, bps, refill, tmode)


def test_rnd_real_device_kat(ctx, oracle):
    """src/test_curandom.cu: device rnd_real == CPU, seeds and floats."""
    import torch
    g = load("rng_chain.npz")
    seeds = torch.tensor(g["seeds"].view(np.int64), device="cuda")
    reals = torch.empty(len(g["seeds"]), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()  # the library runs on its own stream
    ctx.rnd_real_device(seeds.data_ptr(), reals.data_ptr(), len(g["seeds"]))
    assert np.array_equal(seeds.cpu().numpy().view(np.uint64), g["seeds_after"])
    assert np.array_equal(reals.cpu().numpy().view(np.uint32), g["reals"].view(np.uint32))


@pytest.mark.parametrize("fn", [0, 1, 3])
def test_strict_libm_exhaustive(ctx, oracle, fn):
    """Every logf argument in (0, 1] and every expf argument in [-17.5, 89):
    the GPU equals the host C library bit for bit.  fn 3 forces the exp
    evaluator's general path for every argument, the small-argument range
    included: the two paths are interchangeable, which lets the batched and
    adjoint kernels choose the path per warp."""
    import torch
    if fn == 0:
        ranges = [(1, 0x3F800000 + 1)]
    else:
        neg_hi = int(np.array([-17.5], np.float32).view(np.uint32)[0])
        pos_hi = int(np.array([89.0], np.float32).view(np.uint32)[0])
        ranges = [(0x80000000, neg_hi + 1), (0, pos_hi)]
    chunk = 1 << 26
    bad = 0
    for a, b in ranges:
        for s in range(a, b, chunk):
            e = min(s + chunk, b)
            u = np.arange(s, e, dtype=np.uint64).astype(np.uint32)
            x = u.view(np.float32)
            d_in = torch.from_numpy(x).cuda()
            d_out = torch.empty_like(d_in)
            ctx.libm_eval_device(fn, d_in.data_ptr(), d_out.data_ptr(), len(x))
            gpu = d_out.cpu().numpy().view(np.uint32)
            host = oracle.libm_array(min(fn, 1), x).view(np.uint32)
            bad += int(np.count_nonzero(gpu != host))
    assert bad == 0


def test_cross_bound_ex2_exhaustive(ctx):
    """The strict tracker's certain-crossing test assumes the hardware 2^x
    never exceeds the exact value by more than 2^-20 relative.  Checked for
    every float argument in [-150, 0] (below, the result must be 0)."""
    import torch
    chunk = 1 << 26
    worst = 0.0
    a, b = 0x80000000, int(np.array([-150.0], np.float32).view(np.uint32)[0]) + 1
    for s in range(a, b, chunk):
        e = min(s + chunk, b)
        u = torch.arange(s, e, dtype=torch.int64, device="cuda")
        x = (u - (1 << 32)).to(torch.int32).view(torch.float32)
        out = torch.empty_like(x)
        torch.cuda.synchronize()  # the library runs on its own stream
        ctx.libm_eval_device(2, x.data_ptr(), out.data_ptr(), x.numel())
        exact = torch.exp2(x.double())
        rel = (out.double() - exact) / exact
        worst = max(worst, float(rel.max()))
    assert worst <= 2.0 ** -20, worst
    # arguments below -150 (every 4099th float, and -inf) give 0
    u = torch.arange(b, 0xFF800001, 4099, dtype=torch.int64, device="cuda")
    u = torch.cat([u, torch.tensor([0xFF800000], dtype=torch.int64, device="cuda")])
    x = (u - (1 << 32)).to(torch.int32).view(torch.float32)
    out = torch.empty_like(x)
    torch.cuda.synchronize()
    ctx.libm_eval_device(2, x.data_ptr(), out.data_ptr(), x.numel())
    assert float(out.max()) == 0.0


@pytest.mark.parametrize("mode", [0, 1])
def test_division_by_cached_reciprocal(ctx, mode):
    """The strict tracker divides by RN(1/mu) cached per flight: equal to the
    IEEE quotient for all 2^46 significand pairs (mode 0) and for random
    pairs over the tracker's exponent range (mode 1)."""
    n = 1 << 30
    checked, bad, example = ctx.verify_division(mode, n)
    assert checked == (1 << 46 if mode == 0 else n)
    assert bad == 0, hex(example)


def _slab(mcg, nb, P):
    from mc_mpi_gb300 import workloads
    sigs, rates = workloads.config1(nb)
    st, m, dx, _, _ = mcg.layer_decomposition(0.0, 1.0, nb, P)
    return st, m, dx, sigs, rates


@pytest.mark.parametrize("mode", ["strict", "fast"])
@pytest.mark.parametrize("k", [1, 16])
def test_event_mode_identical_to_history(mcg, oracle, mode, k):
    """The event-based tracker (SoA buffers, compaction) gives the history
    tracker's results particle by particle."""
    st, m, dx, sigs, rates = _slab(mcg, 2000, 16)
    p = np.zeros(3000, mcg.PARTICLE_DTYPE)
    p["seed"] = oracle.rnd_seed_chain(99, 3000)
    p["mu"], p["wmc"] = 1.0, 1.0
    with mcg.Context(mode=mode) as ctx:
        ctx.set_layers(st, m, dx, sigs, rates, 1e-12)
        a = p.copy()
        ra = ctx.simulate(a)
        qa, ca = ctx.tally_q(), ctx.counters()
        ctx.tally_reset()
        ctx.set_algorithm("event", k)
        b = p.copy()
        rb = ctx.simulate(b)
        assert a.tobytes() == b.tobytes()
        for key in ("results", "steps", "scatters"):
            assert np.array_equal(ra[key], rb[key])
        assert np.array_equal(ctx.tally_q(), qa)
        assert ctx.counters() == ca


@pytest.mark.parametrize("k", [1, 4])
def test_event_mode_edge_cases(ctx, mcg, k):
    """The event-based tracker on the reference's edge-case traces: per
    particle bit-exact, like the history tracker."""
    g = load("traces_edge.npz")
    lt = g["layer"]
    ctx.set_layers([int(lt[3])], [int(lt[4])], [f32(lt[2])], g["sigs"], g["rates"],
                   float(g["min_w"]))
    ctx.set_algorithm("event", k)
    try:
        p = g["initial"].astype(mcg.PARTICLE_DTYPE).copy()
        r = ctx.simulate(p)
    finally:
        ctx.set_algorithm("history", 1)
    assert p.tobytes() == g["final"].astype(mcg.PARTICLE_DTYPE).tobytes()
    assert np.array_equal(r["results"], g["result"])
    assert np.array_equal(r["steps"], g["steps"])
    assert np.array_equal(r["scatters"], g["scatters"])


@pytest.mark.parametrize("per_cycle", [500, 65536])
def test_worker_handover_queues_match_fused(mcg, per_cycle):
    """The workers' cycle with per-sub-domain queues (64 sub-domains) gives
    the fused tracker's tallies exactly."""
    st, m, dx, sigs, rates = _slab(mcg, 10000, 64)
    with mcg.Context(mode="strict") as ctx:
        ctx.set_layers(st, m, dx, sigs, rates, 1e-12)
        ctx.simulate_source(0, 4000)
        fused = ctx.tally_q()
        steps = ctx.counters()["steps"]
        ctx.tally_reset()
        cycles, hand = ctx.worker_run(4000, per_cycle=per_cycle, queue_capacity=1 << 16)
        assert np.array_equal(ctx.tally_q(), fused)
        assert ctx.counters()["steps"] == steps
        assert cycles > 10 and hand > 4000


@pytest.mark.parametrize("mode", ["strict", "fast"])
def test_async_worker_matches_fused(mcg, mode):
    """The asynchronous workers (one persistent launch, a shared-memory ring
    per block and bounded global rings per sub-domain) give the fused
    tracker's tallies and step counts exactly, on repeated calls that reuse
    the context's rings, with any ring capacity (the admission of newborns
    keeps every ring within it)."""
    st, m, dx, sigs, rates = _slab(mcg, 10000, 64)
    with mcg.Context(mode=mode) as ctx:
        ctx.set_layers(st, m, dx, sigs, rates, 1e-12)
        ctx.simulate_source(0, 20000)
        fused = ctx.tally_q()
        c_fused = ctx.counters()
        for _ in range(2):
            ctx.tally_reset()
            hand = ctx.worker_run_async(20000)
            assert np.array_equal(ctx.tally_q(), fused)
            c = ctx.counters()
            assert c["steps"] == c_fused["steps"] and c["scatters"] == c_fused["scatters"]
            assert c["histories"] == 20000 and hand > 20000
        # a ring capacity of 4 admits only 32 histories at a time (no ring
        # can overflow): slow, with the same tallies
        ctx.tally_reset()
        ctx.simulate_source(0, 1000)
        small = ctx.tally_q()
        ctx.tally_reset()
        ctx.worker_run_async(1000, queue_capacity=4)
        assert np.array_equal(ctx.tally_q(), small)
        ctx.tally_reset()
        ctx.worker_run_async(0)
        assert ctx.tally_q().sum() == 0
        ctx.worker_run_async(20000)
        assert np.array_equal(ctx.tally_q(), fused)


@pytest.mark.parametrize("mode", ["strict", "fast"])
def test_workers_on_a_thick_chain_match_fused(mcg, mode):
    """Both worker forms on a chain too thick for the thin-cell step (1000
    cells on [0, 2], sigma_a up to 4 per unit, 8 sub-domains: the strict
    full-exp instances) give the fused tracker's tallies exactly."""
    from mc_mpi_gb300 import workloads
    sig_a, sig_s, _ = workloads.config3()
    sigs, rates = workloads.sigs_rates(sig_a, sig_s)
    st, m, dx, _, _ = mcg.layer_decomposition(0.0, 1.0, 1000, 8)
    with mcg.Context(mode=mode) as ctx:
        ctx.set_layers(st, m, dx, sigs, rates, 1e-12)
        ctx.simulate_source(0, 5000)
        fused = ctx.tally_q()
        ctx.tally_reset()
        ctx.worker_run_async(5000)
        assert np.array_equal(ctx.tally_q(), fused)
        ctx.tally_reset()
        ctx.worker_run(5000, per_cycle=1000, queue_capacity=1 << 14)
        assert np.array_equal(ctx.tally_q(), fused)


def test_worker_matches_reference_workersync_tally(mcg):
    """Against the reference's own Layer::simulate driven by the WorkerSync
    cycle (golden fixture): float tallies agree to float accuracy."""
    g = load("decomposed_1000x8.npz")
    st, m, dx, _, _ = mcg.layer_decomposition(0.0, 1.0, 1000, int(g["n_layers"]))
    with mcg.Context(mode="strict") as ctx:
        ctx.set_layers(st, m, dx, g["sigs"], g["rates"], float(g["min_w"]))
        ctx.worker_run(len(g["particles"]), per_cycle=500, queue_capacity=1 << 14)
        t = ctx.tally()
    assert np.allclose(t, g["tally"], rtol=2e-5, atol=1e-4)
