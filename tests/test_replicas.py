"""Multi-GPU bench logic on CPU: replicas with no collective on the data path, the
job's time is the slowest rank's (max over ranks), and the reference arm runs on
rank 0 only.  world_size-2 `gloo` process groups on 127.0.0.1."""
import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local = [1.5, 2.5][rank]
    value, t = bench.replica_rate(local, steps=3, device="cpu")
    q.put((rank, value, t))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_rate_takes_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, t in out:
        assert t == 2.5
        assert value == pytest.approx(2 * 3 / 2.5)


def test_replica_rate_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_rate(2.0, steps=4) == (2.0, 2.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    # rank 1 returns before reading its arguments, the oracle or a workload
    bench.run_reference(None, bench.SHAPE)
    assert capsys.readouterr().out == ""
