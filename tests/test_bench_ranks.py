"""bench.py's multi-rank host logic on CPU ranks (gloo, world size 2): every rank renders a
disjoint sample range of the same workload, the timing is the maximum over ranks, and the
reported value counts the paths of all ranks. The GPU side of a rank is a replica of the
single-GPU path, with no collective on the data path."""
import os
import socket

import pytest
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        my_time = 1.0 + rank            # rank 1 is the slow one
        out[rank] = (bench.rank_sample_base(rank), bench.max_over_ranks(my_time, "cpu"))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_disjoint_samples_and_max_timing():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    bases = [res[r][0] for r in range(world)]
    assert all(res[r][1] == 2.0 for r in range(world))          # both ranks see the slowest time
    warmup, steps, spp = 3, 10, bench.SPP
    ranges = [(b, b + (warmup + steps) * spp) for b in bases]
    assert ranges[0][1] <= ranges[1][0]                            # disjoint sample ranges
    v = bench.whole_job_value(world, steps, bench.WIDTH * bench.HEIGHT * spp, 2.0)
    assert v == pytest.approx(world * steps * bench.WIDTH * bench.HEIGHT * spp / 2.0 / 1e6)
