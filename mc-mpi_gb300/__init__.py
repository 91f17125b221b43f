"""mc-mpi_gb300: GB300 particle-history tracker for the mc-mpi hot path.

Python mirror of the reference's Layer API over the C ABI of
libmcgb300.so (include/mcgb300.h).  The computation always runs on the GPU:
loading fails loudly when the library is missing, and there is no CPU path.

  ctx = Context(mode="strict")           # bit-exact with the CPU reference
  ctx.set_slab(0.0, 1.0, nb_cells=100, n_layers=1, sigs=..., rates=..., min_w=1e-12)
  res = ctx.simulate(particles)          # numpy PARTICLE_DTYPE array, in place
  tally = ctx.tally()                    # per-cell absorbed weight (float64)

Layer / decompose_domain mirror include/layer/layer.hpp of the reference.
"""
import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libmcgb300.so")

PARTICLE_DTYPE = np.dtype(
    [("seed", "<u8"), ("x", "<f4"), ("mu", "<f4"), ("wmc", "<f4"), ("index", "<i4")], align=True
)
assert PARTICLE_DTYPE.itemsize == 24

MODE_STRICT = 0
MODE_FAST = 1
OK = 0
STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_OVERFLOW", 4: "ERR_TIMEOUT",
          5: "ERR_STATE", 6: "ERR_TABLES", 7: "ERR_LIMIT"}


class MCGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class Source(C.Structure):
    _fields_ = [("seed_mode", C.c_int32), ("isotropic", C.c_int32), ("base_seed", C.c_uint64),
                ("x0", C.c_float), ("mu0", C.c_float), ("w0", C.c_float), ("cell0", C.c_int32)]


class Slab(C.Structure):
    _fields_ = [("n_cells", C.c_int32), ("seed_mode", C.c_int32), ("isotropic", C.c_int32),
                ("reserved", C.c_int32), ("base_seed", C.c_uint64), ("n_histories", C.c_int64),
                ("mu0", C.c_float), ("w0", C.c_float)]


class Tuning(C.Structure):
    _fields_ = [("block", C.c_int32), ("tally_mode", C.c_int32), ("item_histories", C.c_int64),
                ("sample_ms", C.c_float), ("candidates", C.c_int32), ("algorithm", C.c_int32),
                ("steps_per_pass", C.c_int32), ("defer", C.c_int32)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class Counters(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("histories", "steps", "scatters", "leaked_left",
                                         "leaked_right", "killed", "w_left_q", "w_right_q",
                                         "w_killed_q", "error_flags")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


_lib = None


def load_library(path=None):
    """Load libmcgb300.so; raises if it was not built (no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise MCGError(5, f"{p} missing: run build() (mc-mpi_gb300/build.py) first")
    L = C.CDLL(p)
    vp, i32, i64, f32 = C.c_void_p, C.c_int32, C.c_int64, C.c_float
    sig = {
        "mcg_last_error": (C.c_char_p, []),
        "mcg_version": (C.c_char_p, []),
        "mcg_create": (C.c_int, [C.c_int, C.c_int, C.POINTER(vp)]),
        "mcg_destroy": (C.c_int, [vp]),
        "mcg_set_mode": (C.c_int, [vp, C.c_int]),
        "mcg_set_layers": (C.c_int, [vp, C.c_int, vp, vp, vp, vp, vp, f32]),
        "mcg_set_slab": (C.c_int, [vp, f32, f32, i32, i32, vp, vp, f32]),
        "mcg_set_layers_xs": (C.c_int, [vp, C.c_int, vp, vp, vp, vp, vp, f32]),
        "mcg_set_tally_scale": (C.c_int, [vp, i32]),
        "mcg_tally_reset": (C.c_int, [vp]),
        "mcg_tally_read": (C.c_int, [vp, vp, vp]),
        "mcg_simulate": (C.c_int, [vp, vp, i64, vp, vp, vp]),
        "mcg_simulate_device": (C.c_int, [vp, vp, i64, vp, vp, vp]),
        "mcg_simulate_source": (C.c_int, [vp, C.POINTER(Source), i64, i64]),
        "mcg_create_particles": (C.c_int, [vp, C.POINTER(Source), i64, i64, vp]),
        "mcg_worker_run": (C.c_int, [vp, C.POINTER(Source), i64, i32, i64, vp, vp]),
        "mcg_worker_run_async": (C.c_int, [vp, C.POINTER(Source), i64, i64, vp]),
        "mcg_counters_read": (C.c_int, [vp, C.POINTER(Counters)]),
        "mcg_last_kernel_ms": (C.c_int, [vp, C.POINTER(C.c_float)]),
        "mcg_set_launch": (C.c_int, [vp, i32, i32, i32]),
        "mcg_set_step_limit": (C.c_int, [vp, i64]),
        "mcg_set_tally_mode": (C.c_int, [vp, i32]),
        "mcg_set_algorithm": (C.c_int, [vp, i32, i32]),
        "mcg_cusimulate": (C.c_int, [C.c_int, vp, vp, vp, vp, C.c_int, C.c_int, f32]),
        "mcg_rnd_real_device": (C.c_int, [vp, vp, vp, i64]),
        "mcg_adjoint_set_weights": (C.c_int, [vp, vp]),
        "mcg_adjoint_reset": (C.c_int, [vp]),
        "mcg_adjoint_run": (C.c_int, [vp, C.POINTER(Source), i64, i64, i32]),
        "mcg_adjoint_read": (C.c_int, [vp, vp, vp, vp]),
        "mcg_fit_set": (C.c_int, [vp, i32, vp, vp, vp, vp, f32, i32]),
        "mcg_fit_run": (C.c_int, [vp, i32, f32, f32, f32, f32, f32]),
        "mcg_fit_read": (C.c_int, [vp, vp, vp, vp]),
        "mcg_fit_release": (C.c_int, [vp]),
        "mcg_fit_gradient": (C.c_int, [vp, vp, vp, vp]),
        "mcg_batch_set": (C.c_int, [vp, i32, vp, vp, vp, f32]),
        "mcg_batch_run": (C.c_int, [vp]),
        "mcg_batch_run_per_slab": (C.c_int, [vp]),
        "mcg_batch_tally_reset": (C.c_int, [vp]),
        "mcg_batch_tally_read": (C.c_int, [vp, vp, vp]),
        "mcg_batch_set_launch": (C.c_int, [vp, i32, i64, i32]),
        "mcg_batch_autotune": (C.c_int, [vp, C.c_double, C.POINTER(Tuning)]),
        "mcg_batch_set_algorithm": (C.c_int, [vp, i32, i32]),
        "mcg_batch_set_deferral": (C.c_int, [vp, i32]),
        "mcg_libm_eval_device": (C.c_int, [vp, C.c_int, vp, vp, i64]),
        "mcg_testing_fail_allocation": (C.c_int, [i32]),
        "mcg_measure_conversion_rates": (C.c_int, [vp, vp]),
        "mcg_verify_division": (C.c_int, [vp, C.c_int, C.c_uint64] + [C.POINTER(C.c_uint64)] * 3),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = L
    return L


def _check(rc):
    if rc != OK:
        raise MCGError(rc, load_library().mcg_last_error().decode())


def _device_inputs_ready():
    """The library works on its own non-blocking stream: before a call that
    reads device memory written through torch, wait for torch's stream."""
    import sys
    torch = sys.modules.get("torch")
    if torch is not None and torch.cuda.is_initialized():
        torch.cuda.current_stream().synchronize()


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def layer_decomposition(x_min, x_max, nb_cells, world_size):
    """decompose_domain for every rank (src/layer.cpp:17-42) + the Layer
    constructor's dx (src/layer.cpp:44-48), float32 arithmetic as the
    reference.  Returns (index_start[], m[], dx[], x_min[], x_max[])."""
    f = np.float32
    cpl, extra = nb_cells // world_size, nb_cells % world_size
    gdx = f(f(x_max) - f(x_min)) / f(nb_cells)
    st, ms, dxs, x0s, x1s = [], [], [], [], []
    for r in range(world_size):
        m = cpl + (1 if r < extra else 0)
        s = r * cpl + min(r, extra)
        x0 = f(x_min) + f(s) * gdx
        x1 = f(x_min) + f(s + m) * gdx
        st.append(s)
        ms.append(m)
        dxs.append(f(f(x1 - x0) / f(m)))
        x0s.append(x0)
        x1s.append(x1)
    return (np.array(st, np.int32), np.array(ms, np.int32), np.array(dxs, np.float32),
            np.array(x0s, np.float32), np.array(x1s, np.float32))


class Context:
    """One device context (include/mcgb300.h: mcg_create ... mcg_destroy)."""

    def __init__(self, mode="strict", device=0):
        self.lib = load_library()
        self.h = C.c_void_p()
        m = MODE_STRICT if mode in ("strict", MODE_STRICT) else MODE_FAST
        _check(self.lib.mcg_create(device, m, C.byref(self.h)))
        self.n_cells = 0
        self.log2_scale = 40

    def close(self):
        if self.h:
            self.lib.mcg_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_mode(self, mode):
        _check(self.lib.mcg_set_mode(self.h, MODE_STRICT if mode == "strict" else MODE_FAST))

    def set_layers(self, index_start, m, dx, sigs, rates, min_w):
        index_start = np.ascontiguousarray(index_start, np.int32)
        m = np.ascontiguousarray(m, np.int32)
        dx = np.ascontiguousarray(dx, np.float32)
        sigs = np.ascontiguousarray(sigs, np.float32)
        rates = np.ascontiguousarray(rates, np.float32)
        _check(self.lib.mcg_set_layers(self.h, len(m), _ptr(index_start), _ptr(m), _ptr(dx),
                                       _ptr(sigs), _ptr(rates), float(min_w)))
        self.n_cells = int(m.sum())

    def set_layers_xs(self, index_start, m, dx, sig_a, sig_s, min_w):
        index_start = np.ascontiguousarray(index_start, np.int32)
        m = np.ascontiguousarray(m, np.int32)
        dx = np.ascontiguousarray(dx, np.float32)
        sig_a = np.ascontiguousarray(sig_a, np.float32)
        sig_s = np.ascontiguousarray(sig_s, np.float32)
        _check(self.lib.mcg_set_layers_xs(self.h, len(m), _ptr(index_start), _ptr(m), _ptr(dx),
                                          _ptr(sig_a), _ptr(sig_s), float(min_w)))
        self.n_cells = int(m.sum())

    def set_slab(self, x_min, x_max, nb_cells, n_layers=1, sigs=None, rates=None, min_w=0.0):
        s = None if sigs is None else np.ascontiguousarray(sigs, np.float32)
        r = None if rates is None else np.ascontiguousarray(rates, np.float32)
        _check(self.lib.mcg_set_slab(self.h, float(x_min), float(x_max), int(nb_cells),
                                     int(n_layers), _ptr(s), _ptr(r), float(min_w)))
        self.n_cells = int(nb_cells)

    def set_tally_scale(self, log2_scale):
        _check(self.lib.mcg_set_tally_scale(self.h, int(log2_scale)))
        self.log2_scale = int(log2_scale)

    def tally_reset(self):
        _check(self.lib.mcg_tally_reset(self.h))

    def tally(self):
        out = np.zeros(self.n_cells, np.float64)
        _check(self.lib.mcg_tally_read(self.h, None, _ptr(out)))
        return out

    def tally_q(self):
        out = np.zeros(self.n_cells, np.int64)
        _check(self.lib.mcg_tally_read(self.h, _ptr(out), None))
        return out

    def counters(self):
        c = Counters()
        _check(self.lib.mcg_counters_read(self.h, C.byref(c)))
        return c.as_dict()

    def last_kernel_ms(self):
        v = C.c_float()
        _check(self.lib.mcg_last_kernel_ms(self.h, C.byref(v)))
        return v.value

    def set_launch(self, block=0, blocks_per_sm=0, refill_steps=0):
        _check(self.lib.mcg_set_launch(self.h, block, blocks_per_sm, refill_steps))

    def set_algorithm(self, algorithm="history", steps_per_pass=1):
        _check(self.lib.mcg_set_algorithm(self.h, 0 if algorithm == "history" else 1,
                                          int(steps_per_pass)))

    def set_tally_mode(self, mode):
        _check(self.lib.mcg_set_tally_mode(self.h, int(mode)))

    def simulate(self, particles, want_steps=True):
        """Histories of host particles (PARTICLE_DTYPE, updated in place).
        Returns dict(results, steps, scatters)."""
        assert particles.dtype == PARTICLE_DTYPE and particles.flags.c_contiguous
        n = len(particles)
        res = np.zeros(n, np.int32)
        steps = np.zeros(n, np.int64) if want_steps else None
        scat = np.zeros(n, np.int64) if want_steps else None
        _check(self.lib.mcg_simulate(self.h, _ptr(particles), n, _ptr(res), _ptr(steps), _ptr(scat)))
        return dict(results=res, steps=steps, scatters=scat)

    def simulate_device_ptr(self, d_particles, n, d_results=None, d_steps=None, d_scatters=None):
        _device_inputs_ready()
        _check(self.lib.mcg_simulate_device(self.h, C.c_void_p(d_particles), int(n),
                                            C.c_void_p(d_results) if d_results else None,
                                            C.c_void_p(d_steps) if d_steps else None,
                                            C.c_void_p(d_scatters) if d_scatters else None))

    def simulate_source(self, first, n, seed_mode=0, base_seed=5127801, x0=0.0, mu0=1.0,
                        w0=1.0, isotropic=0, cell0=0):
        src = Source(seed_mode, isotropic, base_seed, x0, mu0, w0, cell0)
        _check(self.lib.mcg_simulate_source(self.h, C.byref(src), int(first), int(n)))

    # -- adjoint --
    def adjoint_set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        _check(self.lib.mcg_adjoint_set_weights(self.h, _ptr(w)))

    def adjoint_reset(self):
        _check(self.lib.mcg_adjoint_reset(self.h))

    def adjoint_run(self, first, n, with_gradient=True, seed_mode=0, base_seed=5127801, x0=0.0,
                    mu0=1.0, w0=1.0, isotropic=0, cell0=0):
        src = Source(seed_mode, isotropic, base_seed, x0, mu0, w0, cell0)
        _check(self.lib.mcg_adjoint_run(self.h, C.byref(src), int(first), int(n),
                                        1 if with_gradient else 0))

    def adjoint_read(self):
        loss = C.c_double()
        ga = np.zeros(self.n_cells, np.float64)
        gs = np.zeros(self.n_cells, np.float64)
        _check(self.lib.mcg_adjoint_read(self.h, C.byref(loss), _ptr(ga), _ptr(gs)))
        return loss.value, ga, gs

    # -- batched inverse fit --
    @staticmethod
    def _slab_array(slabs):
        arr = (Slab * len(slabs))()
        for i, d in enumerate(slabs):
            arr[i] = Slab(int(d["n_cells"]), int(d.get("seed_mode", 0)), int(d.get("isotropic", 0)),
                          0, int(d["base_seed"]), int(d["n_histories"]), float(d.get("mu0", 1.0)),
                          float(d.get("w0", 1.0)))
        return arr

    def fit_set(self, slabs, sig_a0, sig_s, target, min_w=1e-12, max_steps=1000):
        arr = self._slab_array(slabs)
        sig_a0 = np.ascontiguousarray(sig_a0, np.float32)
        sig_s = np.ascontiguousarray(sig_s, np.float32)
        target = np.ascontiguousarray(target, np.float64)
        _check(self.lib.mcg_fit_set(self.h, len(slabs), C.cast(arr, C.c_void_p), _ptr(sig_a0),
                                    _ptr(sig_s), _ptr(target), float(min_w), int(max_steps)))
        self.fit_cells, self.fit_max_steps = len(sig_a0), int(max_steps)

    def fit_run(self, n_steps, lr=1e-2, beta1=0.9, beta2=0.999, eps=1e-8, sig_min=1e-3):
        _check(self.lib.mcg_fit_run(self.h, int(n_steps), lr, beta1, beta2, eps, sig_min))

    def fit_read(self):
        sig = np.zeros(self.fit_cells, np.float32)
        loss = np.zeros(self.fit_max_steps, np.float64)
        st = C.c_int32()
        _check(self.lib.mcg_fit_read(self.h, _ptr(sig), _ptr(loss), C.byref(st)))
        return sig, loss[:st.value]

    def fit_gradient(self, weights):
        """(weight absorbed per history, dF/dsig_a per history) of one
        forward+adjoint launch of the fit's kernel with loss weights w."""
        w = np.ascontiguousarray(weights, np.float64)
        t = np.zeros(len(w), np.float64)
        g = np.zeros(len(w), np.float64)
        _check(self.lib.mcg_fit_gradient(self.h, _ptr(w), _ptr(t), _ptr(g)))
        return t, g

    # -- batched slabs --
    def batch_set(self, slabs, sigs, rates, min_w):
        """slabs: list of dicts(n_cells, n_histories, base_seed, seed_mode, isotropic, mu0, w0);
        sigs/rates: concatenated per-cell arrays (slab order)."""
        arr = (Slab * len(slabs))()
        for i, d in enumerate(slabs):
            arr[i] = Slab(int(d["n_cells"]), int(d.get("seed_mode", 0)), int(d.get("isotropic", 0)),
                          0, int(d["base_seed"]), int(d["n_histories"]), float(d.get("mu0", 1.0)),
                          float(d.get("w0", 1.0)))
        sigs = np.ascontiguousarray(sigs, np.float32)
        rates = np.ascontiguousarray(rates, np.float32)
        _check(self.lib.mcg_batch_set(self.h, len(slabs), C.cast(arr, C.c_void_p), _ptr(sigs),
                                      _ptr(rates), float(min_w)))
        self.batch_cells = int(sum(int(d["n_cells"]) for d in slabs))

    def batch_run(self):
        _check(self.lib.mcg_batch_run(self.h))

    def batch_run_per_slab(self):
        _check(self.lib.mcg_batch_run_per_slab(self.h))

    def batch_tally_reset(self):
        _check(self.lib.mcg_batch_tally_reset(self.h))

    def batch_tally_q(self):
        out = np.zeros(self.batch_cells, np.int64)
        _check(self.lib.mcg_batch_tally_read(self.h, _ptr(out), None))
        return out

    def batch_tally(self):
        out = np.zeros(self.batch_cells, np.float64)
        _check(self.lib.mcg_batch_tally_read(self.h, None, _ptr(out)))
        return out

    def batch_set_launch(self, block=0, item_histories=0, tally_mode=-1):
        _check(self.lib.mcg_batch_set_launch(self.h, block, item_histories, tally_mode))

    def batch_set_deferral(self, defer):
        """0/False: off; True: 8 waiting lanes; 1..32: that many."""
        lanes = 8 if defer is True else int(defer)
        _check(self.lib.mcg_batch_set_deferral(self.h, lanes))

    def batch_set_algorithm(self, algorithm="history", steps_per_pass=0):
        _check(self.lib.mcg_batch_set_algorithm(self.h, 0 if algorithm == "history" else 1,
                                                int(steps_per_pass)))

    def batch_autotune(self, sample_fraction=0.02):
        t = Tuning()
        _check(self.lib.mcg_batch_autotune(self.h, float(sample_fraction), C.byref(t)))
        return t.as_dict()

    def worker_run(self, n, per_cycle=65536, queue_capacity=1 << 20, seed_mode=0,
                   base_seed=5127801, x0=0.0, mu0=1.0, w0=1.0, isotropic=0, cell0=0):
        """The workers' cycle with on-device hand-over queues; returns
        (cycles, handoffs)."""
        src = Source(seed_mode, isotropic, base_seed, x0, mu0, w0, cell0)
        cyc, hand = C.c_int64(), C.c_int64()
        _check(self.lib.mcg_worker_run(self.h, C.byref(src), int(n), int(per_cycle),
                                       int(queue_capacity), C.byref(cyc), C.byref(hand)))
        return cyc.value, hand.value

    def worker_run_async(self, n, queue_capacity=0, seed_mode=0, base_seed=5127801, x0=0.0,
                         mu0=1.0, w0=1.0, isotropic=0, cell0=0):
        """The asynchronous workers (one persistent launch, bounded on-device
        rings); returns the number of hand-overs.  queue_capacity 0: three
        times the GPU's resident threads per ring, which admits twice the
        resident threads in flight and can never overflow."""
        src = Source(seed_mode, isotropic, base_seed, x0, mu0, w0, cell0)
        hand = C.c_int64()
        _check(self.lib.mcg_worker_run_async(self.h, C.byref(src), int(n), int(queue_capacity),
                                             C.byref(hand)))
        return hand.value

    def rnd_real_device(self, d_seeds, d_reals, n):
        _device_inputs_ready()
        _check(self.lib.mcg_rnd_real_device(self.h, C.c_void_p(d_seeds), C.c_void_p(d_reals), n))

    def verify_division(self, mode, n=0):
        """(pairs checked, mismatches, one mismatching pair's bits) of the
        cached-reciprocal division against the IEEE quotient."""
        c, m, x = C.c_uint64(), C.c_uint64(), C.c_uint64()
        _check(self.lib.mcg_verify_division(self.h, mode, n, C.byref(c), C.byref(m), C.byref(x)))
        return c.value, m.value, x.value

    def conversion_rates(self):
        """Measured conversions/s: u64->f32, f32->s64, u32->f32, f32->u32."""
        r = np.zeros(4, np.float64)
        _check(self.lib.mcg_measure_conversion_rates(self.h, _ptr(r)))
        return dict(zip(("u64_f32", "f32_s64", "u32_f32", "f32_u32"), r.tolist()))

    def libm_eval_device(self, fn, d_in, d_out, n):
        _device_inputs_ready()
        _check(self.lib.mcg_libm_eval_device(self.h, fn, C.c_void_p(d_in), C.c_void_p(d_out), n))


def cusimulate(particles, sigs, absorption_rates, weights_absorbed, min_index, max_index, dx):
    """The reference GPU seam (include/culayer/culayer.hpp:6-13) over
    mcg_cusimulate; particles and weights_absorbed are updated in place."""
    lib = load_library()
    sigs = np.ascontiguousarray(sigs, np.float32)
    absorption_rates = np.ascontiguousarray(absorption_rates, np.float32)
    assert weights_absorbed.dtype == np.float32 and particles.dtype == PARTICLE_DTYPE
    _check(lib.mcg_cusimulate(len(particles), _ptr(particles), _ptr(sigs), _ptr(absorption_rates),
                              _ptr(weights_absorbed), int(min_index), int(max_index),
                              float(np.float32(dx))))


from .layer import Layer, decompose_domain  # noqa: E402,F401
