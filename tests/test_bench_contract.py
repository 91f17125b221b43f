"""bench.py's reference arm on the CPU: the oracle port of Layer::simulate
over the 10,000-cell slab on the host cores, printing the benchmark's JSON
line (same metric and workload as the GPU arm); under torchrun only rank 0
prints."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def _run(extra_env=None):
    env = dict(os.environ)
    env.update(extra_env or {})
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True,
                       env=env, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout.strip().splitlines()


def test_reference_arm_prints_the_contract_line(oracle):
    import bench
    lines = _run()
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == "histories/s"
    assert line["config"]["workload"] == bench.WORKLOAD
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert (line["steps"], line["warmup"], line["n_gpus"]) == (1, 0, 1)
    assert line["higher_is_better"] is True and line["vs_baseline"] is None
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly():
    assert _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}) == []


def test_conversion_roofline_arithmetic():
    """64-bit conversions of the strict tracker: two per scatter (flight
    sample and new direction), none per certain crossing; none in the fast
    tracker; the peak is the smaller of the two measured 64-bit rates."""
    import bench
    rates = {"u64_f32": 6e11, "f32_s64": 5.9e11, "u32_f32": 1e13, "f32_u32": 4.6e12}
    r = bench.conversion_roofline(10, 2, 1e-10, "strict", rates)
    assert r["achieved"] == 4 / 1e-10 and r["peak"] == 5.9e11
    assert abs(r["frac"] - 4 / 1e-10 / 5.9e11) < 1e-12
    assert bench.conversion_roofline(10, 2, 1.0, "fast", rates)["achieved"] == 0
