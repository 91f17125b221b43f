"""Host logic of the multi-GPU path on CPU: world_size-2 gloo ranks shard the
histories, compute their tallies (with the oracle standing in for each
rank's GPU) and reduce them exactly; the result equals one rank doing all."""
import os
import socket

import numpy as np
import pytest


def test_shard_covers_everything(mcg):
    from mc_mpi_gb300 import dist
    for n in (0, 1, 7, 1000, 10**8 + 3):
        for ws in (1, 2, 3, 8):
            ranges = [dist.shard(n, ws, r) for r in range(ws)]
            assert sum(c for _, c in ranges) == n
            pos = 0
            for f, c in ranges:
                assert f == pos
                pos += c
    with pytest.raises(ValueError):
        dist.shard(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out_dir):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "oracle"))
    sys.path.insert(0, os.path.join(root, "tests"))
    import torch
    import torch.distributed as tdist
    from conftest import import_package
    import oracle as O
    import_package()
    from mc_mpi_gb300 import dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    n_total, m = 3001, 100
    first, count = dist.shard(n_total, world, rank)
    xc = ((np.arange(m) + 0.5) / m).astype(np.float32)
    sa = (np.float32(0.2) + np.float32(1.8) * xc).astype(np.float32)
    sigs = (sa + np.float32(1.0)).astype(np.float32)
    rates = (sa / sigs).astype(np.float32)
    p = np.zeros(count, O.PARTICLE_DTYPE)
    p["seed"] = O.rnd_seed_chain(O.lcg_skip(5127801, first, True), count)
    p["mu"], p["wmc"] = 1.0, 1.0
    r = O.simulate_histories([O.layer_make(0.0, 1.0, 0, m)], sigs, rates, 1e-12, p, 2.0 ** 40,
                             nthreads=1)
    t = torch.from_numpy(r["tally_q"].copy())
    dist.allreduce_tally(t)

    # the code path of the benchmark's multi-rank check: dist.sharded_tally
    # with each rank's share run by a callable (the GPU source there, the
    # oracle standing in for it here)
    def run_shard(f, c):
        pp = np.zeros(c, O.PARTICLE_DTYPE)
        pp["seed"] = O.rnd_seed_chain(O.lcg_skip(5127801, f, True), c)
        pp["mu"], pp["wmc"] = 1.0, 1.0
        return O.simulate_histories([O.layer_make(0.0, 1.0, 0, m)], sigs, rates, 1e-12, pp,
                                    2.0 ** 40, nthreads=1)["tally_q"]

    t2 = dist.sharded_tally(run_shard, n_total, world, rank)
    np.save(os.path.join(out_dir, f"count{rank}.npy"), np.array([count]))
    if rank == 0:
        np.save(os.path.join(out_dir, "reduced.npy"), t.numpy())
        np.save(os.path.join(out_dir, "sharded.npy"), t2.numpy())
    tdist.destroy_process_group()


def test_two_rank_gloo_reduction_is_exact(mcg, oracle, tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    reduced = np.load(tmp_path / "reduced.npy")
    m = 100
    xc = ((np.arange(m) + 0.5) / m).astype(np.float32)
    sa = (np.float32(0.2) + np.float32(1.8) * xc).astype(np.float32)
    sigs = (sa + np.float32(1.0)).astype(np.float32)
    rates = (sa / sigs).astype(np.float32)
    p = np.zeros(3001, oracle.PARTICLE_DTYPE)
    p["seed"] = oracle.rnd_seed_chain(5127801, 3001)
    p["mu"], p["wmc"] = 1.0, 1.0
    whole = oracle.simulate_histories([oracle.layer_make(0.0, 1.0, 0, m)], sigs, rates, 1e-12, p,
                                      2.0 ** 40)
    assert np.array_equal(reduced, whole["tally_q"])
    assert np.array_equal(np.load(tmp_path / "sharded.npy"), whole["tally_q"])
    # the two ranks ran different shards (1501 and 1500 histories)
    assert [int(np.load(tmp_path / f"count{r}.npy")[0]) for r in (0, 1)] == [1501, 1500]
