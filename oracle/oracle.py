"""ctypes bindings of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, and only as the checker.  It wraps:
  * liboracle.so - the plain-C restatement of the reference's Layer path
    (oracle/mcoracle.c, each function cites src/layer.cpp / src/random.cpp);
  * _ref/libmcref.so - the reference's own src/layer.cpp + src/random.cpp
    compiled in place with oracle/ref_harness.cpp, where it could be built.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libmcref.so")

PARTICLE_DTYPE = np.dtype(
    [("seed", "<u8"), ("x", "<f4"), ("mu", "<f4"), ("wmc", "<f4"), ("index", "<i4")], align=True
)
assert PARTICLE_DTYPE.itemsize == 24
TRACE_DTYPE = np.dtype([("result", "<i4"), ("pad", "<i4"), ("steps", "<i8"), ("scatters", "<i8")])


class Layer(C.Structure):
    _fields_ = [
        ("x_min", C.c_float), ("x_max", C.c_float), ("dx", C.c_float),
        ("index_start", C.c_int32), ("m", C.c_int32),
        ("left_border", C.c_int32), ("right_border", C.c_int32),
    ]

    def as_tuple(self):
        return (self.x_min, self.x_max, self.dx, self.index_start, self.m,
                self.left_border, self.right_border)


def build(ref=None):
    """Compile liboracle.so (and _ref/ when the reference sources exist)."""
    env = dict(os.environ)
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True, env=env)
    ref_root = ref or os.environ.get("MCG_REFERENCE", "/root/reference")
    if os.path.isfile(os.path.join(ref_root, "src", "layer.cpp")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_root}"], check=True, env=env)


_lib = None
_ref = None


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.orc_rnd_real.restype = C.c_float
        L.orc_rnd_real.argtypes = [C.POINTER(C.c_uint64)]
        L.orc_rnd_seed.restype = C.c_uint64
        L.orc_rnd_seed.argtypes = [C.POINTER(C.c_uint64)]
        L.orc_lcg_skip.restype = C.c_uint64
        L.orc_lcg_skip.argtypes = [C.c_uint64, C.c_uint64, C.c_int]
        L.orc_decompose.argtypes = [C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, C.POINTER(Layer)]
        L.orc_layer_make.argtypes = [C.c_float, C.c_float, C.c_int, C.c_int, C.POINTER(Layer)]
        L.orc_default_sigs.argtypes = [C.POINTER(Layer), C.c_void_p, C.c_void_p]
        L.orc_create_particles.restype = C.c_int
        L.orc_create_particles.argtypes = [C.POINTER(Layer), C.c_float, C.c_float, C.c_int,
                                           C.c_uint64, C.c_void_p]
        L.orc_layer_simulate.argtypes = [C.POINTER(Layer), C.c_void_p, C.c_void_p, C.c_float,
                                         C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_float, C.c_void_p]
        L.orc_simulate_histories.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                             C.c_float, C.c_void_p, C.c_int, C.c_void_p,
                                             C.c_void_p, C.c_float, C.c_void_p,
                                             C.POINTER(C.c_int64), C.c_int]
        L.orc_format_wa.restype = C.c_int
        L.orc_format_wa.argtypes = [C.POINTER(Layer), C.c_void_p, C.c_char_p, C.c_int]
        L.orc_fp64_adjoint.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_double, C.c_void_p, C.c_int, C.POINTER(C.c_double),
                                       C.c_void_p, C.c_void_p, C.c_int]
        L.orc_libm_array.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_longlong]
        L.orc_fp64_histories.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                         C.c_double, C.c_void_p, C.c_int, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_int]
        _lib = L
    return _lib


def ref_available():
    return os.path.exists(REF_LIB)


def ref():
    global _ref
    if _ref is None:
        R = C.CDLL(REF_LIB)
        R.ref_trace_particles.argtypes = [C.c_float, C.c_float, C.c_int, C.c_int, C.c_float,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        R.ref_layer_simulate.argtypes = [C.c_float, C.c_float, C.c_int, C.c_int, C.c_float,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                         C.c_int, C.c_void_p, C.c_void_p, C.POINTER(C.c_int),
                                         C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        R.ref_test_layer_wa.restype = C.c_int
        R.ref_test_layer_wa.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_int]
        R.ref_decomposed.restype = C.c_int
        R.ref_decomposed.argtypes = [C.c_float, C.c_float, C.c_int, C.c_int, C.c_float,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                     C.c_int, C.c_void_p]
        _ref = R
    return _ref


# ---------------------------------------------------------------- helpers
def rnd_seed_chain(seed, n):
    """n successive rnd_seed values starting from `seed` (src/random.cpp:24-29)."""
    s = C.c_uint64(seed)
    out = np.empty(n, np.uint64)
    L = lib()
    for i in range(n):
        out[i] = L.orc_rnd_seed(C.byref(s))
    return out


def rnd_real(seeds):
    """One rnd_real step per seed; returns (new seeds, floats)."""
    L = lib()
    seeds = np.array(seeds, np.uint64)
    reals = np.empty(len(seeds), np.float32)
    for i in range(len(seeds)):
        s = C.c_uint64(int(seeds[i]))
        reals[i] = L.orc_rnd_real(C.byref(s))
        seeds[i] = s.value
    return seeds, reals


def lcg_skip(seed, n, seed_chain):
    return int(lib().orc_lcg_skip(seed, n, 1 if seed_chain else 0))


def decompose(x_min, x_max, nb_cells, world_size):
    out = (Layer * world_size)()
    for r in range(world_size):
        lib().orc_decompose(x_min, x_max, nb_cells, world_size, r, C.byref(out[r]))
    return out


def layer_make(x_min, x_max, index_start, m):
    L = Layer()
    lib().orc_layer_make(x_min, x_max, index_start, m, C.byref(L))
    return L


def default_sigs(L):
    sigs = np.empty(L.m, np.float32)
    rates = np.empty(L.m, np.float32)
    lib().orc_default_sigs(C.byref(L), _p(sigs), _p(rates))
    return sigs, rates


def create_particles(L, x_ini, wmc, n, seed):
    out = np.zeros(n, PARTICLE_DTYPE)
    k = lib().orc_create_particles(C.byref(L), x_ini, wmc, n, seed, _p(out))
    return out[:k]


def layer_simulate(L, sigs, rates, min_w, particles, n, q_scale=0.0, tally_f32=None):
    """Layer::simulate(n) (one call, one thread).  Returns dict."""
    particles = np.ascontiguousarray(particles).copy()
    n_total = len(particles)
    n = min(n, n_total)
    results = np.zeros(n, np.int32)
    t32 = np.zeros(L.m, np.float32) if tally_f32 is None else tally_f32
    tq = np.zeros(L.m, np.int64)
    t64 = np.zeros(L.m, np.float64)
    tr = np.zeros(n, TRACE_DTYPE)
    lib().orc_layer_simulate(C.byref(L), _p(sigs), _p(rates), min_w, _p(particles), n_total, n,
                             _p(results), _p(t32), _p(tq), _p(t64), q_scale, _p(tr))
    return dict(particles=particles, results=results, tally_f32=t32, tally_q=tq, tally_f64=t64,
                traces=tr)


def simulate_histories(layers, sigs, rates, min_w, particles, q_scale, nthreads=0):
    layers_arr = (Layer * len(layers))(*layers)
    particles = np.ascontiguousarray(particles).copy()
    total = layers[-1].index_start + layers[-1].m
    tq = np.zeros(total, np.int64)
    t64 = np.zeros(total, np.float64)
    tr = np.zeros(len(particles), TRACE_DTYPE)
    hand = C.c_int64(0)
    lib().orc_simulate_histories(C.cast(layers_arr, C.c_void_p), len(layers), _p(sigs), _p(rates),
                                 min_w, _p(particles), len(particles), _p(tq), _p(t64), q_scale,
                                 _p(tr), C.byref(hand), nthreads)
    return dict(particles=particles, tally_q=tq, tally_f64=t64, traces=tr, handoffs=hand.value)


def fp64_histories(layers, sigs, rates, min_w, particles, nthreads=0):
    layers_arr = (Layer * len(layers))(*layers)
    total = layers[-1].index_start + layers[-1].m
    t = np.zeros(total, np.float64)
    t2 = np.zeros(total, np.float64)
    leak = np.zeros(2, np.float64)
    particles = np.ascontiguousarray(particles)
    lib().orc_fp64_histories(C.cast(layers_arr, C.c_void_p), len(layers), _p(sigs), _p(rates),
                             float(min_w), _p(particles), len(particles), _p(t), _p(t2), _p(leak),
                             nthreads)
    return dict(tally=t, tally_sq=t2, leak=leak)


def format_wa(L, tally_f32):
    buf = C.create_string_buffer(1 << 20)
    n = lib().orc_format_wa(C.byref(L), _p(np.ascontiguousarray(tally_f32, np.float32)), buf,
                            1 << 20)
    assert n >= 0
    return buf.value.decode()


def libm_array(fn, x):
    """Host C library logf (fn 0) or expf (fn 1) of a float32 array."""
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty_like(x)
    lib().orc_libm_array(fn, _p(x), _p(out), len(x))
    return out


def fp64_adjoint(layers, sig_a, sig_s, w, min_w, particles, nthreads=0, with_gradient=True):
    """Sums over the histories of the loss and of dG/dsig_a, dG/dsig_s (FP64);
    with_gradient=False runs the forward pass only (gradients returned as 0)."""
    layers_arr = (Layer * len(layers))(*layers)
    total = layers[-1].index_start + layers[-1].m
    sa = np.ascontiguousarray(sig_a, np.float64)
    ss = np.ascontiguousarray(sig_s, np.float64)
    ww = np.ascontiguousarray(w, np.float64)
    ga = np.zeros(total, np.float64)
    gs = np.zeros(total, np.float64)
    loss = C.c_double(0.0)
    particles = np.ascontiguousarray(particles)
    lib().orc_fp64_adjoint(C.cast(layers_arr, C.c_void_p), len(layers), _p(sa), _p(ss), _p(ww),
                           float(min_w), _p(particles), len(particles), C.byref(loss),
                           _p(ga) if with_gradient else None, _p(gs) if with_gradient else None,
                           nthreads)
    return loss.value, ga, gs
