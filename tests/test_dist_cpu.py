"""The multi-process path of bench.py on CPU (gloo, world size 2): proofs are
independent, so ranks run replicas and only the timing is reduced (the
slowest rank's time, max over ranks); the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=2)
    ws, r, local = bench.dist_info()
    out[rank] = (ws, r, local, bench.barrier_and_max(1.5 + rank, ws))
    dist.destroy_process_group()


def test_two_rank_max_over_ranks():
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0] == (2, 0, 0, 2.5)
    assert res[1] == (2, 1, 1, 2.5)


def test_reference_arm_only_on_rank_zero(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        steps, warmup, gpus = 1, 0, 2
    bench.run_reference_arm(A, 2, 1)  # rank 1: returns without work or output
    assert capsys.readouterr().out == ""
