"""Multi-GPU is replicas only: every rank solves its own copy of the workload,
no collective touches the data path, and bench.py reports the slowest rank.
These CPU tests run the rank logic with two gloo ranks on 127.0.0.1."""
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


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "dplus-dev_gb300"))
    import torch.distributed as dist
    import bench
    from dpx import workloads as W
    r, w, lr = bench.rank_info()
    dist.init_process_group("gloo", rank=r, world_size=w)
    # replicas: every rank builds the same seeded mix and request stream
    mix = [(s.atoms, s.layers, round(s.qmax, 12)) for s in W.batch_mix(16)]
    stream = [(x.kind, round(x.arrival_s, 12)) for x in W.request_stream(12, helix_copies_n=500)]
    t = bench.max_over_ranks(10.0 * (rank + 1), w)
    pair = bench.max_over_ranks([1.0 + rank, 5.0 - rank], w)
    bench.barrier_sync(w)
    dist.destroy_process_group()
    q.put((r, w, lr, mix, stream, t, pair))


def test_two_gloo_replicas_agree_and_report_the_slowest_rank():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, l0, mix0, st0, t0, p0), (r1, w1, l1, mix1, st1, t1, p1) = res
    assert (r0, r1, w0, w1, l0, l1) == (0, 1, 2, 2, 0, 1)
    assert mix0 == mix1 and st0 == st1  # identical replica workloads
    assert t0 == t1 == 20.0  # the slowest rank's time
    assert p0 == p1 == [2.0, 5.0]
