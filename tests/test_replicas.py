"""bench.py --gpus N runs N independent replicas (the path does not shard):
the whole-job rate sums every rank's corners over the slowest rank's step
time.  Checked with world_size 2 on the gloo backend (CPU), and the
reference arm exits without work on ranks other than 0."""
import os
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    ms, value = bench.replica_rate(1.0 + rank, 1000, ws, "cpu")
    dist.destroy_process_group()
    q.put((rank, ms, value))


def test_replica_rate_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in out:
        assert ms == 2.0                      # max over ranks
        assert value == pytest.approx(2 * 1000 / 2.0e-3)


def test_reference_arm_other_ranks_do_nothing(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        steps, warmup, gpus = 1, 3, 2
    bench.run_reference(A())
    assert capsys.readouterr().out == ""
