"""bench.py --gpus N runs N independent replicas (one seeded scene per rank,
no collective on the data path); its whole-job figures are the slowest
rank's time and the sum of all ranks' units.  Two gloo ranks on the CPU."""
import os
import socket

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from automs_gb300 import scenes
    elapsed = [120.5, 98.25][rank]
    units = [5_291_998, 5_100_001][rank]
    t, u = bench.aggregate_over_ranks(torch, dist, "cpu", elapsed, units)
    c = scenes.coverage_config("coverage-tiny", seed=rank)
    out[rank] = (t, u, float(np.asarray(c["tris"], np.float64).sum()))
    dist.destroy_process_group()


def test_two_replicas_aggregate():
    world = 2
    with mp.get_context("spawn").Manager() as m:  # no fork of this threaded process
        out = m.dict()
        mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world,
                           start_method="spawn")
        res = dict(out)
    for r in range(world):
        t, u, _ = res[r]
        assert t == 120.5 and u == 5_291_998 + 5_100_001
    # the replicas trace different seeded scenes
    assert res[0][2] != res[1][2]


def test_single_process_passthrough():
    import bench
    assert bench.aggregate_over_ranks(torch, None, "cpu", 3.5, 7) == (3.5, 7)
