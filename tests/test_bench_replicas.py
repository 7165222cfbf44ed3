"""Replicas on N GPUs (bench.py --gpus N under torchrun): the path does not
shard, so every rank runs its own copy of the workload and the job's rate is
world x per-rank units over the slowest rank's time.  Checked here with two
gloo ranks on the CPU (no GPU involved)."""
import importlib.util
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    b = _bench()
    t = b.max_over_ranks(1.0 + rank, dist)          # rank 1 is the slow replica
    out[rank] = (t, b.job_rate(1000, t, world))
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_replicas_take_the_slowest_time_and_add_their_work():
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, _free_port(), out), nprocs=2, join=True)
        got = dict(out)
    assert got[0] == got[1] == (2.0, 1000.0)        # 2 x 1000 units in 2 s


def test_single_process_is_its_own_max():
    b = _bench()
    assert b.max_over_ranks(3.5, None) == 3.5
    assert b.job_rate(10, 2.0, 1) == pytest.approx(5.0)
