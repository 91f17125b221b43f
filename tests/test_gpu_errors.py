"""Error behaviour of the C ABI on the GPU: every failure is a status code
with a message (the reference asserts, calls exit() or MPI_Abort), and the
context stays usable afterwards.  Failures are provoked on the host side
(bad arguments, missing state, a step limit, a too small hand-over queue, a
refused libm table); nothing here faults the GPU."""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
f32 = np.float32


def _rc(mcg, name, *args):
    lib = mcg.load_library()
    return getattr(lib, name)(*args), lib.mcg_last_error().decode()


def _slab(ctx, nb=200):
    xc = (np.arange(nb) + 0.5) / nb
    sa = (0.5 + 0.4 * np.sin(6 * np.pi * xc)).astype(np.float32)
    ss = (2.0 + 1.5 * np.cos(4 * np.pi * xc)).astype(np.float32)
    sigs = (sa + ss).astype(np.float32)
    ctx.set_layers([0], [nb], [f32(1.0 / nb)], sigs, (sa / sigs).astype(np.float32), 1e-12)


def test_bad_arguments_and_missing_state(built, mcg):
    with mcg.Context(mode="strict") as ctx:
        p = np.zeros(4, mcg.PARTICLE_DTYPE)
        # no layers yet
        rc, msg = _rc(mcg, "mcg_simulate", ctx.h, p.ctypes.data_as(C.c_void_p), 4, None, None, None)
        assert rc == 5 and "no layers" in msg  # MCG_ERR_STATE
        rc, _ = _rc(mcg, "mcg_tally_read", ctx.h, None, None)
        assert rc == 5
        _slab(ctx)
        rc, _ = _rc(mcg, "mcg_simulate", ctx.h, None, 4, None, None, None)
        assert rc == 1  # MCG_ERR_ARG: particles missing
        rc, _ = _rc(mcg, "mcg_simulate", ctx.h, p.ctypes.data_as(C.c_void_p), -1, None, None, None)
        assert rc == 1
        rc, _ = _rc(mcg, "mcg_set_step_limit", ctx.h, 0)
        assert rc == 1
        rc, _ = _rc(mcg, "mcg_set_algorithm", ctx.h, 7, 1)
        assert rc == 1
        # the context still works
        p["seed"] = np.arange(1, 5, dtype=np.uint64)
        p["mu"], p["wmc"] = 1.0, 1.0
        ctx.simulate(p)
        assert ctx.counters()["histories"] == 4


def test_step_limit_reports_and_recovers(built, mcg):
    """A history still alive at the step limit ends with result 2 and the
    call returns MCG_ERR_LIMIT (the reference has no limit: its loop would
    run on); the other histories finish normally."""
    with mcg.Context(mode="strict") as ctx:
        _slab(ctx)
        p = np.zeros(64, mcg.PARTICLE_DTYPE)
        p["seed"] = np.arange(1, 65, dtype=np.uint64) * np.uint64(7919)
        p["mu"], p["wmc"] = 1.0, 1.0
        ref = p.copy()
        r_ref = ctx.simulate(ref)
        longest = int(r_ref["steps"].max())
        ctx.set_tally_scale(40)
        rc, _ = _rc(mcg, "mcg_set_step_limit", ctx.h, max(1, longest - 1))
        assert rc == 0
        q = p.copy()
        res = np.zeros(64, np.int32)
        steps = np.zeros(64, np.int64)
        rc, msg = _rc(mcg, "mcg_simulate", ctx.h, q.ctypes.data_as(C.c_void_p), 64,
                      res.ctypes.data_as(C.c_void_p), steps.ctypes.data_as(C.c_void_p), None)
        assert rc == 7 and "step limit" in msg  # MCG_ERR_LIMIT
        hit = steps >= longest - 1
        assert np.all(res[hit & (res != r_ref["results"])] == 2)
        assert np.array_equal(res[~hit], r_ref["results"][~hit])
        # back to the default limit: the same call succeeds again
        assert _rc(mcg, "mcg_set_step_limit", ctx.h, 1 << 28)[0] == 0
        ctx.tally_reset()
        ctx.simulate(p.copy())


def test_worker_queue_overflow_is_reported(built, mcg):
    """The reference aborts on a full hand-over buffer; here the call returns
    MCG_ERR_OVERFLOW and the context stays usable."""
    xs = mcg.layer_decomposition(0.0, 1.0, 1000, 8)
    st, m, dx = xs[0], xs[1], xs[2]
    xc = (np.arange(1000) + 0.5) / 1000
    sa = (0.5 + 0.4 * np.sin(6 * np.pi * xc)).astype(np.float32)
    ss = (2.0 + 1.5 * np.cos(4 * np.pi * xc)).astype(np.float32)
    sigs = (sa + ss).astype(np.float32)
    with mcg.Context(mode="strict") as ctx:
        ctx.set_layers(st, m, dx, sigs, (sa / sigs).astype(np.float32), 1e-12)
        with pytest.raises(mcg.MCGError) as e:
            ctx.worker_run(4000, per_cycle=4000, queue_capacity=8)
        assert e.value.code == 3  # MCG_ERR_OVERFLOW
        ctx.tally_reset()
        cycles, hand = ctx.worker_run(4000, per_cycle=500, queue_capacity=1 << 14)
        assert cycles > 0 and hand > 0


def test_libm_table_refused(built, mcg, tmp_path):
    """A strict context refuses a libm table that is not the one this build
    and this C library produce (MCG_ERR_TABLES), instead of using it."""
    bad = tmp_path / "libm_exceptions.bin"
    good = os.path.join(os.path.dirname(built.LIB), "libm_exceptions.bin")
    data = bytearray(open(good, "rb").read())
    data[64] ^= 0xFF  # the fingerprint
    bad.write_bytes(bytes(data))
    old = os.environ.get("MCG_LIBM_TABLE")
    os.environ["MCG_LIBM_TABLE"] = str(bad)
    try:
        h = C.c_void_p()
        rc, msg = _rc(mcg, "mcg_create", 0, 0, C.byref(h))
        if rc == 0:  # the table is loaded at the first strict launch
            ctx = mcg.Context.__new__(mcg.Context)
            ctx.lib, ctx.h = mcg.load_library(), h
            _slab(ctx)
            p = np.zeros(4, mcg.PARTICLE_DTYPE)
            p["seed"] = np.arange(1, 5, dtype=np.uint64)
            p["mu"], p["wmc"] = 1.0, 1.0
            rc, msg = _rc(mcg, "mcg_simulate", h, p.ctypes.data_as(C.c_void_p), 4, None, None,
                          None)
            mcg.load_library().mcg_destroy(h)
        assert rc == 6 and "rebuild" in msg  # MCG_ERR_TABLES
    finally:
        if old is None:
            del os.environ["MCG_LIBM_TABLE"]
        else:
            os.environ["MCG_LIBM_TABLE"] = old


@pytest.mark.parametrize("fail_at", [0, 1, 2])
def test_failed_layer_setup_leaves_no_geometry(built, mcg, fail_at):
    """A device allocation that fails part-way through mcg_set_layers (made
    to fail on the host, without touching the GPU) leaves the context with no
    geometry: launches and tally reads return MCG_ERR_STATE instead of
    indexing buffers sized for another chain; a new set-up recovers it and
    gives the same tallies as a fresh context."""
    lib = mcg.load_library()
    p = np.zeros(64, mcg.PARTICLE_DTYPE)
    p["seed"] = np.arange(1, 65, dtype=np.uint64) * np.uint64(104729)
    p["mu"], p["wmc"] = 1.0, 1.0
    with mcg.Context(mode="strict") as ref:
        _slab(ref, 300)
        ref.simulate(p.copy())
        q_ref = ref.tally_q()
    with mcg.Context(mode="strict") as ctx:
        _slab(ctx, 200)
        ctx.simulate(p.copy())
        lib.mcg_testing_fail_allocation(fail_at)
        try:
            with pytest.raises(mcg.MCGError) as e:
                _slab(ctx, 300)
            assert e.value.code == 2  # MCG_ERR_CUDA
        finally:
            lib.mcg_testing_fail_allocation(-1)
        rc, msg = _rc(mcg, "mcg_simulate", ctx.h, p.copy().ctypes.data_as(C.c_void_p), 64, None,
                      None, None)
        assert rc == 5 and "no layers" in msg
        assert _rc(mcg, "mcg_tally_read", ctx.h, None, None)[0] == 5
        _slab(ctx, 300)
        ctx.simulate(p.copy())
        assert np.array_equal(ctx.tally_q(), q_ref)


@pytest.mark.parametrize("fail_at", [0, 3, 4])
def test_failed_batch_setup_leaves_no_slabs(built, mcg, fail_at):
    """The same for mcg_batch_set: a failed allocation leaves no slabs set
    (MCG_ERR_STATE), and a new set-up runs as on a fresh context."""
    lib = mcg.load_library()
    rng = np.random.default_rng(11)
    slabs = [dict(n_cells=int(c), n_histories=500, seed_mode=1, isotropic=s % 2,
                  base_seed=1000 + 7919 * s, mu0=1.0, w0=1.0)
             for s, c in enumerate(rng.integers(16, 200, 6))]
    tot = sum(d["n_cells"] for d in slabs)
    sigs = rng.uniform(0.5, 5.0, tot).astype(np.float32)
    rates = rng.uniform(0.1, 0.9, tot).astype(np.float32)
    with mcg.Context(mode="strict") as ref:
        ref.batch_set(slabs, sigs, rates, 1e-12)
        ref.batch_run()
        q_ref = ref.batch_tally_q()
    with mcg.Context(mode="strict") as ctx:
        ctx.batch_set(slabs[:3], sigs[: sum(d["n_cells"] for d in slabs[:3])],
                      rates[: sum(d["n_cells"] for d in slabs[:3])], 1e-12)
        ctx.batch_run()
        lib.mcg_testing_fail_allocation(fail_at)
        try:
            with pytest.raises(mcg.MCGError) as e:
                ctx.batch_set(slabs, sigs, rates, 1e-12)
            assert e.value.code == 2
        finally:
            lib.mcg_testing_fail_allocation(-1)
        rc, msg = _rc(mcg, "mcg_batch_run", ctx.h)
        assert rc == 5 and "no slabs" in msg
        ctx.batch_set(slabs, sigs, rates, 1e-12)
        ctx.batch_run()
        assert np.array_equal(ctx.batch_tally_q(), q_ref)
