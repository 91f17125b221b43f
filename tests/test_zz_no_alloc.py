"""The allocation-free entry point mcg_simulate_fast_noalloc against the
context path (fast mode, mcg_set_layers + mcg_simulate_device).

Callers that may not allocate device memory (host codes whose allocator owns
the GPU) use the no-allocation variant; it must give the same particles,
results and fixed-point tally as the regular path, bit for bit, and keep
doing so on consecutive calls that reuse its fixed scratch.  This file is
collected last so that a failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bind(lib):
    fn = lib.mcg_simulate_fast_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.c_float, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    return fn


def _case(mcg, oracle, nb, n, seed_offset):
    P = 16
    st, m, dx, _, _ = mcg.layer_decomposition(0.0, 1.0, nb, P)
    xc = (np.arange(nb) + 0.5) / nb
    sa = (0.5 + 0.4 * np.sin(6 * np.pi * xc)).astype(np.float32)
    ss = (2.0 + 1.5 * np.cos(4 * np.pi * xc)).astype(np.float32)
    sigs = (sa + ss).astype(np.float32)
    rates = (sa / sigs).astype(np.float32)
    p = np.zeros(n, mcg.PARTICLE_DTYPE)
    p["seed"] = oracle.rnd_seed_chain(oracle.lcg_skip(5127801, seed_offset, True), n)
    p["x"], p["mu"], p["wmc"], p["index"] = 0.0, 1.0, 1.0, 0
    return st, m, dx, sigs, rates, p


# 200 cells: 256-thread blocks with one tally copy per warp; 2000 cells:
# 1024-thread blocks with one copy per block; 16,384 cells: the largest
# chain the fixed scratch holds.
@pytest.mark.parametrize("nb", [200, 2000, 16384])
def test_noalloc_matches_context_path_twice(built, mcg, oracle, nb):
    import torch
    lib = mcg.load_library()
    fn = _bind(lib)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)
    ctx = mcg.Context(mode="fast")
    # the second call passes no result array
    for call, (offset, with_results) in enumerate(((0, True), (50000, False))):
        st, m, dx, sigs, rates, p = _case(mcg, oracle, nb, 40000, offset)
        n, total = len(p), int(m.sum())
        assert total == nb
        # regular path
        ctx.set_layers(st, m, dx, sigs, rates, 1e-12)
        ctx.set_tally_scale(36)
        d_ref = torch.from_numpy(p.view(np.uint8).copy()).cuda()
        r_ref = torch.zeros(n, dtype=torch.int32, device="cuda")
        ctx.simulate_device_ptr(d_ref.data_ptr(), n, r_ref.data_ptr())
        q_ref = ctx.tally_q()
        # allocation-free path on the same particles
        d_na = torch.from_numpy(p.view(np.uint8).copy()).cuda()
        r_na = torch.zeros(n, dtype=torch.int32, device="cuda")
        q_na = torch.full((total,), -7, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        rc = fn(len(m), ptr(st), ptr(m), ptr(dx), ptr(sigs), ptr(rates), 1e-12, 36,
                C.c_void_p(d_na.data_ptr()), n,
                C.c_void_p(r_na.data_ptr()) if with_results else None,
                C.c_void_p(q_na.data_ptr()))
        assert rc == 0, lib.mcg_last_error().decode()
        assert torch.equal(d_na, d_ref), f"call {call}: final particles differ"
        if with_results:
            assert torch.equal(r_na, r_ref), f"call {call}: results differ"
        assert np.array_equal(q_na.cpu().numpy(), q_ref), f"call {call}: tallies differ"
        assert q_ref.sum() > 0
    ctx.close()


def test_noalloc_empty_call_clears_tally(built, mcg, oracle):
    """n = 0 runs no kernel, but the output tally is still overwritten with
    the (zero) tally of the call, not the previous call's."""
    import torch
    lib = mcg.load_library()
    fn = _bind(lib)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)
    st, m, dx, sigs, rates, p = _case(mcg, oracle, 300, 2000, 0)
    d = torch.from_numpy(p.view(np.uint8).copy()).cuda()
    q = torch.zeros(300, dtype=torch.int64, device="cuda")
    rc = fn(len(m), ptr(st), ptr(m), ptr(dx), ptr(sigs), ptr(rates), 1e-12, 36,
            C.c_void_p(d.data_ptr()), len(p), None, C.c_void_p(q.data_ptr()))
    assert rc == 0, lib.mcg_last_error().decode()
    assert int(q.sum()) > 0
    q.fill_(-7)
    rc = fn(len(m), ptr(st), ptr(m), ptr(dx), ptr(sigs), ptr(rates), 1e-12, 36,
            None, 0, None, C.c_void_p(q.data_ptr()))
    assert rc == 0, lib.mcg_last_error().decode()
    assert not q.any()


def test_noalloc_rejects_oversized_chain(built, mcg):
    lib = mcg.load_library()
    fn = _bind(lib)
    m = np.array([20000], np.int32)
    st = np.zeros(1, np.int32)
    dx = np.array([1.0 / 20000], np.float32)
    sigs = np.ones(20000, np.float32)
    rates = np.full(20000, 0.5, np.float32)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)
    dummy = C.c_void_p(8)  # never dereferenced: the size check fails first
    rc = fn(1, ptr(st), ptr(m), ptr(dx), ptr(sigs), ptr(rates), 0.0, 36, dummy, 0, None, dummy)
    assert rc == 1
    assert "exceeds the fixed scratch" in lib.mcg_last_error().decode()
    # a layer count whose running total would overflow 32 bits is rejected
    # at the first layer past the limit
    big = np.full(3, 2**31 - 1, np.int32)
    starts = np.zeros(3, np.int32)
    rc = fn(3, ptr(starts), ptr(big), ptr(dx), ptr(sigs), ptr(rates), 0.0, 36, dummy, 0, None,
            dummy)
    assert rc == 1
