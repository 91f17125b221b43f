"""Host logic that needs no GPU: the domain decomposition of the Python
binding against the oracle, and the C++ config loader (options_from_config)
against the reference's parsing rules (src/yaml_loader.cpp:4-41,
src/worker.cpp:315-333)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import PKG_DIR, ROOT

CONFIG = ("x_min: 0.000000000000000000e+00\nx_max: 1.000000000000000000e+00\n"
          "x_ini: 7.071067690849304199e-01\nparticle_min_weight: 9.999999960041972003e-13\n"
          "nb_cells: 1000\nnb_particles: 100000\ncycle_time: 1.e-05\n"
          "nb_particles_per_cycle: 500\nnthread: 1\nstatistics_cycle_time: 1.e-1\n")


@pytest.mark.parametrize("x_min,x_max,cells,ranks", [
    (0.0, 1.0, 10000, 64), (0.0, 1.0, 1000, 8), (0.0, 1.0, 100, 1), (0.0, 1.0, 37, 5),
    (0.0, 2.0, 1000, 7), (-1.5, 3.25, 4099, 13), (0.0, 1.0, 64, 64)])
def test_layer_decomposition_matches_oracle(mcg, oracle, x_min, x_max, cells, ranks):
    """decompose_domain + the Layer constructor's dx (src/layer.cpp:17-48):
    start index, cell count, dx and the layer bounds, bit for bit."""
    st, m, dx, x0, x1 = mcg.layer_decomposition(x_min, x_max, cells, ranks)
    ref = oracle.decompose(x_min, x_max, cells, ranks)
    f = np.float32
    assert int(m.sum()) == cells and st[0] == 0
    for r in range(ranks):
        L = ref[r]
        assert (st[r], m[r]) == (L.index_start, L.m)
        assert f(dx[r]).tobytes() == f(L.dx).tobytes()
        assert f(x0[r]).tobytes() == f(L.x_min).tobytes()
        assert f(x1[r]).tobytes() == f(L.x_max).tobytes()


@pytest.fixture(scope="module")
def config_exe(built, tmp_path_factory):
    out = tmp_path_factory.mktemp("cfg")
    exe = str(out / "test_config_cpu")
    libdir = os.path.dirname(built.LIB)
    subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(PKG_DIR, "host", "include"),
                    os.path.join(ROOT, "tests", "cpp", "test_config_cpu.cpp"), "-L" + libdir,
                    "-lmcgb300", "-Wl,-rpath," + libdir, "-o", exe], check=True)
    return exe


def _load(exe, tmp_path, text, ranks=8):
    cfg = tmp_path / "config.yaml"
    cfg.write_bytes(text.encode())
    r = subprocess.run([exe, str(cfg), str(ranks)], capture_output=True, text=True)
    vals = dict(line.split(" ", 1) for line in r.stdout.splitlines())
    return r.returncode, vals, r.stderr


def test_config_loader_reads_the_reference_keys(config_exe, tmp_path):
    rc, v, err = _load(config_exe, tmp_path, CONFIG)
    assert rc == 0, err
    assert v["world_size"] == "8" and v["nb_cells"] == "1000"
    assert v["nb_particles"] == "100000" and v["nb_particles_per_cycle"] == "500"
    assert v["nthread"] == "1"
    f = np.float32
    assert f(float(v["x_ini"])) == f(0.7071067690849304199)
    assert f(float(v["particle_min_weight"])) == f(9.999999960041972003e-13)
    assert float(v["cycle_time"]) == 1e-5 and float(v["statistics_cycle_time"]) == 0.1
    # CRLF line ends: the reference keeps the '\r' in the value, which the
    # number parsers ignore
    rc2, v2, _ = _load(config_exe, tmp_path, CONFIG.replace("\n", "\r\n"))
    assert rc2 == 0 and v2 == v


def test_config_loader_first_key_wins(config_exe, tmp_path):
    rc, v, err = _load(config_exe, tmp_path, CONFIG + "nb_cells: 77\n")
    assert rc == 0, err
    assert v["nb_cells"] == "1000"
    rc, v, err = _load(config_exe, tmp_path, "nb_cells: 77\n" + CONFIG)
    assert rc == 0 and v["nb_cells"] == "77"


def test_config_loader_errors(config_exe, tmp_path):
    # a line without ':' (an empty line included) is a format error
    rc, _, err = _load(config_exe, tmp_path, CONFIG + "\n")
    assert rc != 0 and "not correctly formatted" in err
    rc, _, err = _load(config_exe, tmp_path, CONFIG.replace("nthread: 1\n", ""))
    assert rc != 0 and "nthread" in err
    r = subprocess.run([config_exe, str(tmp_path / "missing.yaml"), "1"], capture_output=True,
                       text=True)
    assert r.returncode != 0 and "Couldn't open" in r.stderr


@pytest.mark.parametrize("name", sorted(f[:-4] for f in os.listdir(os.path.join(ROOT, "tests", "cpp"))
                                        if f.endswith(".cpp")))
def test_cpp_programs_build_against_the_api(built, tmp_path, name):
    """Every C++ test program (the GPU ones included) compiles and links
    against the installed headers and libmcgb300.so: the C++ API the
    reference's callers use stays in step with the library."""
    libdir = os.path.dirname(built.LIB)
    r = subprocess.run(["g++", "-O0", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                        "-I" + os.path.join(PKG_DIR, "host", "include"),
                        os.path.join(ROOT, "tests", "cpp", name + ".cpp"), "-L" + libdir,
                        "-lmcgb300", "-Wl,-rpath," + libdir, "-o", str(tmp_path / name)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
