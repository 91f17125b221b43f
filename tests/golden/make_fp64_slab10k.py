#!/usr/bin/env python3
"""Generate the FP64 statistical fixture of the benchmark's slab.

Workload: slab [0, 1] in 10,000 cells decomposed into 64 sub-domains
(decompose_domain), sigma_a = 0.5 + 0.4 sin(6 pi x), sigma_s = 2 + 1.5 cos(4 pi x)
at cell centres (fp32), particles born at x = 0, mu = 1, weight 1, seeds the
rnd_seed chain from 5127801 (histories 0 .. n-1, the source the GPU tests
run through mcg_simulate_source), minimum weight 1e-12.

The oracle's FP64 restatement of the physics (orc_fp64_histories: double
arithmetic, log/expm1, the same LCG draws, on the reference's float cell
faces) runs every history; per cell it
keeps the sum of the absorbed weight and the sum over histories of the
square of each history's absorbed weight, so the per-cell standard error
of the sum is exact.  Chunks of 1e6 histories are accumulated; a fixture is
written each time the count reaches one of the requested sizes:

    python tests/golden/make_fp64_slab10k.py 10000000 100000000

writes fp64_slab10k_1e7.npz after 1e7 histories and fp64_slab10k_1e8.npz
after 1e8 (about 55 minutes on 8 x86 cores).  The fixture does not depend on
the host C library beyond double-precision rounding, so it serves the GPU
box, where the statistical tests of the fast arithmetic read it.
"""
import math
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

NB, LAYERS, BASE_SEED, MIN_W = 10000, 64, 5127801, 1e-12
CHUNK = 1_000_000


def physics():
    xc = (np.arange(NB) + 0.5) / NB
    sa = (0.5 + 0.4 * np.sin(6 * np.pi * xc)).astype(np.float32)
    ss = (2.0 + 1.5 * np.cos(4 * np.pi * xc)).astype(np.float32)
    sigs = (sa + ss).astype(np.float32)
    return sigs, (sa / sigs).astype(np.float32)


def fixture_name(n):
    e = int(round(math.log10(n)))
    assert 10 ** e == n, "sizes are powers of ten"
    return os.path.join(HERE, f"fp64_slab10k_1e{e}.npz")


def main(sizes):
    O.build()
    sizes = sorted(int(float(s)) for s in sizes)
    sigs, rates = physics()
    layers = list(O.decompose(0.0, 1.0, NB, LAYERS))
    tally = np.zeros(NB)
    tally_sq = np.zeros(NB)
    leak = np.zeros(2)
    done = 0
    t0 = time.time()
    while done < sizes[-1]:
        n = min(CHUNK, sizes[-1] - done)
        for s in sizes:
            if done < s < done + n:
                n = s - done
        p = np.zeros(n, O.PARTICLE_DTYPE)
        p["seed"] = O.rnd_seed_chain(O.lcg_skip(BASE_SEED, done, True), n)
        p["x"], p["mu"], p["wmc"], p["index"] = 0.0, 1.0, 1.0, 0
        r = O.fp64_histories(layers, sigs, rates, MIN_W, p)
        tally += r["tally"]
        tally_sq += r["tally_sq"]
        leak += r["leak"]
        done += n
        print(f"{done} histories, {time.time() - t0:.0f} s", flush=True)
        if done in sizes:
            np.savez_compressed(fixture_name(done), n=done, tally=tally, tally_sq=tally_sq,
                                leak=leak, base_seed=BASE_SEED)
            print("wrote", fixture_name(done), flush=True)


if __name__ == "__main__":
    main(sys.argv[1:] or ["10000000"])
