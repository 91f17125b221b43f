"""Python mirror of the reference's Layer (include/layer/layer.hpp:14-110,
src/layer.cpp) whose simulate() runs on the GPU through the C ABI.

Public members carry the reference's names and meaning: weights_absorbed,
particles, particles_left, particles_right, nb_disabled, sigs,
absorption_rates, particle_min_weight, dx, left_border, right_border, seed,
x_ini, wmc, nb_particles_create.  Arrays of particles are numpy arrays of
PARTICLE_DTYPE (the 24-byte Particle of include/types/particle.hpp).
"""
import ctypes as C
import ctypes.util

import numpy as np

from . import PARTICLE_DTYPE, Context, Source, _check, _ptr, load_library

MAX_PARTICLES_VECTOR = 1000000  # src/layer.cpp:15
EPS_PRECISION = np.float32(1e-4)  # include/types/types.hpp:15

_libm = C.CDLL(ctypes.util.find_library("m") or "libm.so.6")
_libm.expf.restype = C.c_float
_libm.expf.argtypes = [C.c_float]

f32 = np.float32


class Layer:
    """Layer(x_min, x_max, index_start, m, particle_min_weight) - src/layer.cpp:44-69."""

    def __init__(self, x_min, x_max, index_start, m, particle_min_weight, mode="strict",
                 context=None):
        self.x_min, self.x_max = f32(x_min), f32(x_max)
        self.m, self.index_start = int(m), int(index_start)
        self.dx = f32(f32(self.x_max - self.x_min) / f32(m))
        self.left_border = bool(abs(self.x_min) < EPS_PRECISION)
        self.right_border = bool(abs(float(self.x_max) - 1.0) < float(EPS_PRECISION))
        self.particle_min_weight = f32(particle_min_weight)
        # sigs[i] = expf(-x_mid), x_mid = x_min + i*dx + 0.5*dx (double), rates 0.5
        self.sigs = np.empty(self.m, np.float32)
        for i in range(self.m):
            x_mid = f32(float(f32(self.x_min + f32(i) * self.dx)) + 0.5 * float(self.dx))
            self.sigs[i] = _libm.expf(float(-x_mid))
        self.absorption_rates = np.full(self.m, 0.5, np.float32)
        self.weights_absorbed = np.zeros(self.m, np.float32)
        self.particles = np.zeros(0, PARTICLE_DTYPE)
        self.particles_left = np.zeros(0, PARTICLE_DTYPE)
        self.particles_right = np.zeros(0, PARTICLE_DTYPE)
        self.nb_disabled = 0
        self.seed = 0
        self.x_ini = f32(0)
        self.wmc = f32(0)
        self.nb_particles_create = 0
        self._ctx = context or Context(mode=mode)
        self._uploaded = None

    # -- particle source (src/layer.cpp:71-121) --
    def create_particles(self, x_ini, wmc, n, seed):
        x_ini = f32(x_ini)
        if x_ini > self.x_min and x_ini < self.x_max:
            self.x_ini, self.wmc = x_ini, f32(wmc)
            self.nb_particles_create = int(n)
            self.seed = int(seed)
            self._created = 0
            self._create(MAX_PARTICLES_VECTOR)

    def nb_active(self):
        return len(self.particles) + self.nb_particles_create

    def _create(self, n):
        if self.nb_particles_create <= 0:
            return
        n = max(MAX_PARTICLES_VECTOR - len(self.particles), n)
        n = min(self.nb_particles_create, n)
        self.nb_particles_create -= n
        # particle k of the chain: k-th rnd_seed from self.seed; mu from its own stream
        src = Source(0, 1, self.seed, float(self.x_ini), 0.0, float(self.wmc),
                     int(self.x_ini / self.dx))
        out = np.zeros(n, PARTICLE_DTYPE)
        _check(load_library().mcg_create_particles(self._ctx.h, C.byref(src), self._created, n,
                                                   _ptr(out)))
        self._created += n
        self.particles = np.concatenate([self.particles, out])

    # -- Layer::simulate (src/layer.cpp:220-361) --
    def simulate(self, nb_particles, nthread=-1, use_gpu=True):
        """nthread and use_gpu are accepted for signature compatibility; the
        histories always run on the GPU."""
        if nb_particles == -1 or nb_particles > MAX_PARTICLES_VECTOR:
            self._simulate_helper(nb_particles)
        if len(self.particles) < nb_particles and self.nb_particles_create > 0:
            self._create(nb_particles)
        nb = min(len(self.particles), nb_particles)
        if nb <= 0:
            return
        self._upload()
        batch = np.ascontiguousarray(self.particles[len(self.particles) - nb:][::-1])
        self._ctx.tally_reset()
        res = self._ctx.simulate(batch, want_steps=False)["results"]
        self.weights_absorbed += self._ctx.tally().astype(np.float32)
        self.particles_left = np.concatenate([self.particles_left, batch[res == -1]])
        self.particles_right = np.concatenate([self.particles_right, batch[res == 1]])
        self.nb_disabled += int(np.count_nonzero(res == 0))
        self.particles = self.particles[: len(self.particles) - nb]
        if self.left_border:
            self.nb_disabled += len(self.particles_left)
            self.particles_left = self.particles_left[:0]
        if self.right_border:
            self.nb_disabled += len(self.particles_right)
            self.particles_right = self.particles_right[:0]

    def _simulate_helper(self, nb_particles):
        if nb_particles == -1:
            while len(self.particles) > 0 or self.nb_particles_create > 0:
                self.simulate(MAX_PARTICLES_VECTOR)
        while nb_particles > 0 and (len(self.particles) > 0 or self.nb_particles_create > 0):
            k = min(nb_particles, MAX_PARTICLES_VECTOR)
            self.simulate(k)
            nb_particles -= k

    def _upload(self):
        key = (self.sigs.tobytes(), self.absorption_rates.tobytes(), float(self.particle_min_weight))
        if key != self._uploaded:
            self._ctx.set_layers([self.index_start], [self.m], [self.dx], self.sigs,
                                 self.absorption_rates, self.particle_min_weight)
            self._uploaded = key

    # -- Layer::dump_WA (src/layer.cpp:363-380) --
    def dump_WA(self, path="WA.out"):
        with open(path, "w") as f:
            f.write(self.format_WA())

    def format_WA(self):
        lines = []
        for i in range(self.m):
            x = float(f32(self.x_min + f32(i) * self.dx)) + 0.5 * float(self.dx)
            lines.append("%.4e %.3e\n" % (x, float(f32(self.weights_absorbed[i] / self.dx))))
        return "".join(lines)


def decompose_domain(x_min, x_max, x_ini, world_size, world_rank, nb_cells, nb_particles,
                     particle_min_weight, mode="strict"):
    """src/layer.cpp:17-42."""
    cpl, extra = nb_cells // world_size, nb_cells % world_size
    m = cpl + (1 if world_rank < extra else 0)
    start = world_rank * cpl + min(world_rank, extra)
    dx = f32(f32(f32(x_max) - f32(x_min)) / f32(nb_cells))
    cell_ini = int(f32(f32(x_ini) - f32(x_min)) / dx)
    layer = Layer(f32(x_min) + f32(start) * dx, f32(x_min) + f32(start + m) * dx, start, m,
                  particle_min_weight, mode=mode)
    if start <= cell_ini < start + m:
        layer.create_particles(x_ini, f32(1.0 / nb_particles), nb_particles, 5127801)
    return layer
