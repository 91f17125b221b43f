"""Build libmcgb300.so (sm_103a) and the host-libm exception table.

Outputs go to mc-mpi_gb300/_build/:
  libmcgb300.so        the C-ABI library (include/mcgb300.h) and the C++ Layer
                       API (host/include/*.hpp)
  libm_tablegen        generator of the strict-mode host-libm table
  libm_exceptions.bin  the table, regenerated when missing or made against
                       another C library (fingerprint check)
"""
import concurrent.futures as cf
import ctypes
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libmcgb300.so")
TABLE = os.path.join(OUT, "libm_exceptions.bin")
GEN = os.path.join(OUT, "libm_tablegen")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["mcg_api.cu", "mcg_misc.cu", "mcg_noalloc.cu", "mcg_batch.cu",
              "mcg_adjoint.cu", "mcg_event.cu", "mcg_worker.cu", "mcg_fit.cu"]
HOST_SOURCES = ["layer.cpp", "random.cpp", "worker.cpp"]


def _run(cmd, **kw):
    r = subprocess.run(cmd, capture_output=True, text=True, **kw)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _deps():
    out = []
    for d in (CSRC, HOST, os.path.join(ROOT, "include")):
        for base, _, files in os.walk(d):
            out += [os.path.join(base, f) for f in files
                    if f.endswith((".cu", ".cuh", ".h", ".hpp", ".cpp", ".inc"))]
    return out


def build_library(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    deps = _deps()
    if _newer(LIB, deps):
        return LIB
    flags = ["-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
             "-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "-I" + os.path.join(HOST, "include")]
    objs = []

    def compile_one(src):
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        if src.endswith(".cu"):
            cmd = [NVCC, *flags, "-c", src, "-o", obj]
        else:
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
                   "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
                   "-I" + os.path.join(HOST, "include"),
                   "-I/usr/local/cuda/include", "-c", src, "-o", obj]
        _run(cmd)
        return obj

    srcs = [os.path.join(CSRC, s) for s in CU_SOURCES] + [os.path.join(HOST, s) for s in HOST_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    _run([NVCC, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart_static", "-ldl", "-lrt",
          "-lpthread"])
    os.replace(LIB + ".tmp", LIB)
    if verbose:
        print("built", LIB)
    return LIB


def _table_is_current():
    """True when the table exists and was made against this host's libm."""
    if not os.path.exists(TABLE):
        return False
    try:
        if not os.path.exists(GEN):
            return False
        r = subprocess.run([GEN, "--fingerprint-matches", TABLE], capture_output=True)
        return r.returncode == 0
    except OSError:
        return False


def build_tables(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(CSRC, "libm_tablegen.cpp")
    hdrs = [os.path.join(CSRC, f) for f in ("exact_libm.h", "libm_tables.inc", "libm_file.h")]
    if not _newer(GEN, [src] + hdrs):
        _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-I" + CSRC, src,
              "-o", GEN])
        if os.path.exists(TABLE):
            os.remove(TABLE)
    if _table_is_current():
        return TABLE
    r = _run([GEN, TABLE + ".tmp"])
    os.replace(TABLE + ".tmp", TABLE)
    if verbose:
        sys.stdout.write(r.stdout)
    return TABLE


def build(verbose=False):
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_library, verbose)
        f2 = ex.submit(build_tables, verbose)
        f1.result()
        f2.result()
    # the library must load and export its entry points
    ctypes.CDLL(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
