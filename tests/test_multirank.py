"""Multi-rank plumbing of bench.py on CPU (gloo, world size 2): the timing
barrier, max-over-ranks and the rank-0-only reference arm. Cases are
independent, so ranks share no data; only these host collectives exist."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    import torch.distributed as dist

    class A:
        pass

    w, r, _ = bench.dist_setup(A())
    bench.barrier(w)
    m = bench.max_over_ranks(w, float(10 + rank))
    out.put((rank, w, m))
    dist.destroy_process_group()


def test_two_rank_max_and_barrier():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2, 11.0), (1, 2, 11.0)]


def test_reference_arm_prints_on_rank_zero_only(capsys):
    import bench

    class A:
        workload = "sphere512"
        steps = 1
        warmup = 0
        gpus = 2

    bench.run_reference(A(), world=2, rank=1)
    assert capsys.readouterr().out == ""
