"""The multi-GPU path of bench.py is replicas over disjoint seed ranges with a max-over-ranks
timing reduction and no data-path collective.  Here two gloo ranks on CPU run the same
sharding (with the CPU oracle standing in for the GPU) and must reproduce the single-process
result over the union of their seeds."""
import os
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, runs, out_dir):
    import sys

    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch
    import torch.distributed as dist

    import bench
    import jne_oracle

    dist.init_process_group("gloo", rank=rank, world_size=world)
    s0 = bench.replica_seed_first(rank, runs)
    eig = jne_oracle.c_eigs_seeded(3, 2, 64, s0, runs)
    slowest = bench.reduce_max(dist, float(rank + 1), "cpu")
    parts = [torch.zeros((runs, eig.shape[1]), dtype=torch.float64) for _ in range(world)]
    dist.all_gather(parts, torch.from_numpy(eig))
    if rank == 0:
        np.save(os.path.join(out_dir, "gathered.npy"), torch.cat(parts).numpy())
        np.save(os.path.join(out_dir, "slowest.npy"), np.array([slowest]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_cover_the_seed_range_once(oracle, tmp_path):
    import torch.multiprocessing as mp

    world, runs = 2, 24
    mp.start_processes(_worker, args=(world, _free_port(), runs, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    gathered = np.load(tmp_path / "gathered.npy")
    whole = oracle.c_eigs_seeded(3, 2, 64, 1, world * runs)
    assert np.array_equal(gathered, whole)
    assert float(np.load(tmp_path / "slowest.npy")[0]) == world
