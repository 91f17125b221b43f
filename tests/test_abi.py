"""CPU tests of the C ABI: the library builds, loads and exports every entry
point declared in include/mcgb300.h.  No compute call is made here."""
import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import ROOT


def declared_functions():
    with open(os.path.join(ROOT, "include", "mcgb300.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_ ]*?[\s\*]+(\w+)\s*\(", text, re.M)
    return sorted(set(n for n in names if not n.startswith("__")))


def test_header_declares_the_abi():
    names = declared_functions()
    for must in ("mcg_create", "mcg_destroy", "mcg_set_layers", "mcg_simulate", "cusimulate",
                 "mcg_tally_read", "mcg_simulate_source"):
        assert must in names


def test_library_exports_every_declared_symbol(built):
    out = subprocess.run(["nm", "-D", "--defined-only", built.LIB], capture_output=True,
                         text=True, check=True).stdout
    exported = set(line.split()[-1] for line in out.splitlines() if line.strip())
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"declared but not exported: {missing}"


def test_library_loads_and_reports(built, mcg):
    lib = mcg.load_library()
    assert lib.mcg_version().decode().startswith("mcgb300")


def test_no_gpu_fails_loudly(built, mcg):
    """Without a GPU the context cannot be created and says why (no fallback)."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(mcg.MCGError):
        mcg.Context(mode="fast")


def test_strict_table_built(built):
    assert os.path.exists(built.TABLE)
    r = subprocess.run([built.GEN, "--fingerprint-matches", built.TABLE])
    assert r.returncode == 0
