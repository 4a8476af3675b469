"""Multi-rank host path on CPU (gloo, world size 2).

The path shards by frequency: every rank solves its own block of the sweep
with a replicated model, and only the step time is reduced (max over ranks).
This checks, without a GPU, that the sharding in bench.py covers the sweep
without overlap, that per-rank results gathered over gloo equal a single
process's (the oracle's FP64 solve stands in for the device solve here), and
that the max-over-ranks timing reduction behaves.
"""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_path):
    sys.path.insert(0, ROOT)
    import importlib
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from tests.conftest import load_package
    load_package()
    meshes = importlib.import_module("elpaso_core_gb300.meshes")
    from oracle import oracle as orc
    d = meshes.plate(6, 4, 0.3, 0.2, 0.002)
    s = orc.System(d)
    S = 3
    mine = np.concatenate([bench.sweep(rank, world, k, S) for k in range(2)])
    xs = np.stack([s.solve(2 * np.pi * f) for f in mine])
    t = torch.tensor([float(rank + 1)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    freqs = [None] * world
    sols = [None] * world
    dist.all_gather_object(freqs, mine.tolist())
    dist.all_gather_object(sols, xs)
    if rank == 0:
        np.savez(out_path, freqs=np.array(freqs, dtype=object), sols=np.array(sols, dtype=object), tmax=t.item())
    dist.barrier()
    dist.destroy_process_group()


def test_frequency_sharding_over_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    out = str(tmp_path / "gather.npz")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    r = np.load(out, allow_pickle=True)
    assert r["tmax"] == 2.0
    freqs = [np.asarray(f) for f in r["freqs"]]
    allf = np.concatenate(freqs)
    assert len(np.unique(allf)) == len(allf) == 12          # no frequency solved twice
    sys.path.insert(0, ROOT)
    import bench
    single = np.concatenate([bench.sweep(0, 1, k, 3) for k in range(4)])
    assert sorted(allf.tolist()) == sorted(single.tolist())   # same frequencies as one rank
    import importlib
    from tests.conftest import load_package
    load_package()
    meshes = importlib.import_module("elpaso_core_gb300.meshes")
    from oracle import oracle as orc
    s = orc.System(meshes.plate(6, 4, 0.3, 0.2, 0.002))
    for f_list, xs in zip(freqs, r["sols"]):
        for f, x in zip(f_list, xs):
            assert np.allclose(x, s.solve(2 * np.pi * f), rtol=1e-12, atol=0)
