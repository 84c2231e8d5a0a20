"""Multi-rank host logic of bench.py on CPU with gloo (world size 2).

Every rank runs an independent replica; the reported time is the maximum over
ranks and the whole-job value sums the replicas.
"""

import os
import socket
import sys

import torch
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    bench.init_dist(ws, "gloo")
    t = bench.max_over_ranks(10.0 * (rank + 1), ws, torch.device("cpu"))
    bench.barrier(ws)
    out[rank] = t
    torch.distributed.destroy_process_group()


def test_max_over_ranks_gloo():
    ws = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, out)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    assert dict(out) == {0: 20.0, 1: 20.0}


def test_reference_arm_only_rank0_prints(capsys, monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        steps, gpus = 1, 2

    called = []
    monkeypatch.setattr(bench, "cpu_oracle_rate", lambda *a, **k: called.append(1))
    bench.reference_arm(A(), 2, 1)
    assert called == [] and capsys.readouterr().out == ""
