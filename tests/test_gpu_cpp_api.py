"""The C++ API (mc-mpi_gb300/host/include: Layer, decompose_domain, Worker,
cusimulate) used the way the reference's own tests use theirs: compiled C++
programs linked against libmcgb300.so."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, PKG_DIR, ROOT

pytestmark = pytest.mark.gpu
CPP = os.path.join(ROOT, "tests", "cpp")


def _build(built, name, out_dir):
    exe = os.path.join(out_dir, name)
    libdir = os.path.dirname(built.LIB)
    subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(PKG_DIR, "host", "include"),
                    os.path.join(CPP, name + ".cpp"), "-L" + libdir, "-lmcgb300",
                    "-Wl,-rpath," + libdir, "-o", exe], check=True)
    return exe


def test_cpp_layer_golden_wa(built, tmp_path):
    exe = _build(built, "test_layer_gpu", str(tmp_path))
    r = subprocess.run([exe, os.path.join(GOLDEN, "test_layer_WA.out")], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_cpp_particle_step_composes(built, tmp_path):
    exe = _build(built, "test_steps_gpu", str(tmp_path))
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_cpp_worker_outputs(built, mcg, tmp_path):
    cfg = tmp_path / "config.yaml"
    cfg.write_text("x_min: 0.0\nx_max: 1.0\nx_ini: 7.071067690849304199e-01\n"
                   "particle_min_weight: 1e-12\nnb_cells: 1000\nnb_particles: 20000\n"
                   "cycle_time: 1.e-05\nnb_particles_per_cycle: 500\nnthread: 1\n"
                   "statistics_cycle_time: 1.e-1\n")
    exe = _build(built, "test_worker_gpu", str(tmp_path))
    r = subprocess.run([exe, str(cfg)], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = (tmp_path / "out" / "weights.csv").read_text().splitlines()
    assert rows[0] == "proc, x, weight" and len(rows) == 1001
    procs = [int(x.split(",")[0]) for x in rows[1:]]
    assert procs[0] == 0 and procs[-1] == 7 and procs == sorted(procs)
    assert (tmp_path / "out" / "config.yaml").read_text().startswith("# Read from config")
    assert len((tmp_path / "WA.out").read_text().splitlines()) == 125
    # out/stats.csv in WorkerSync's columns, one row per sub-domain
    stats = (tmp_path / "out" / "stats.csv").read_text().splitlines()
    assert stats[0] == ("rank, starttime, endtime, time_comp, time_send, time_recv, "
                        "time_idle, nb_cycles, ")
    assert len(stats) == 9
    for r, row in enumerate(stats[1:]):
        f = [x.strip() for x in row.split(",")]
        assert int(f[0]) == r and len(f) == 9 and f[8] == ""
        assert float(f[2]) >= float(f[1]) > 0 and float(f[3]) > 0 and int(f[7]) > 0
    # the same problem through the fused tracker: identical absorbed weights
    w = np.array([float(x.split(",")[2]) for x in rows[1:]])
    st, m, dx, _, _ = mcg.layer_decomposition(0.0, 1.0, 1000, 8)
    sigs = np.concatenate([_default_sigs(mcg, st[r], m[r], dx[r]) for r in range(8)])
    with mcg.Context(mode="strict") as ctx:
        ctx.set_layers(st, m, dx, sigs, np.full(1000, 0.5, np.float32), 1e-12)
        x_ini = np.float32(7.071067690849304199e-01)
        ctx.simulate_source(0, 20000, seed_mode=0, base_seed=5127801, x0=float(x_ini), mu0=0.0,
                            w0=float(np.float32(1.0 / 20000)), isotropic=1,
                            cell0=int(x_ini / dx[5]))
        fused = ctx.tally().astype(np.float32) / dx[0]
    assert np.allclose(w, fused, rtol=1e-6, atol=1e-9)


def _default_sigs(mcg, start, m, dx):
    import ctypes
    import ctypes.util
    libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
    libm.expf.restype = ctypes.c_float
    libm.expf.argtypes = [ctypes.c_float]
    f = np.float32
    gdx = f(f(1.0) / f(1000))
    x0 = f(f(start) * gdx)
    out = np.empty(m, np.float32)
    for i in range(m):
        x_mid = f(float(f(x0 + f(i) * f(dx))) + 0.5 * float(dx))
        out[i] = libm.expf(float(-x_mid))
    return out
