"""The multi-rank logic of bench.py on CPU ranks (gloo, world size 2): the
step time is the largest over the replicas, the rate the whole job's, and
the reference arm does its work on rank 0 only."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = [1.5, 4.25][rank]
    ms = bench.max_over_ranks(local_ms, world)
    out[rank] = (ms, bench.aggregate_rate(ms, world))
    dist.barrier()
    dist.destroy_process_group()


def test_slowest_rank_sets_the_step(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    port = _free_port()
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        ms, rate = res[rank]
        assert ms == 4.25
        assert abs(rate - 2 * 1000.0 / 4.25) < 1e-9


def test_one_rank_is_its_own_maximum():
    import bench
    assert bench.max_over_ranks(3.0, 1) == 3.0
    assert bench.aggregate_rate(2.0, 1) == 500.0


def test_reference_arm_works_on_rank_0_only(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("RANK", "1")
    bench.run_reference(None)      # returns before touching its arguments
    assert capsys.readouterr().out == ""
