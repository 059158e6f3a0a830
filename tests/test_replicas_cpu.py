"""The bench's replica harness on CPU: world_size 2 over gloo on 127.0.0.1.
Each rank runs its own replica; the whole-job time is the slowest rank's,
and the reference arm runs on rank 0 alone (the other ranks exit at once)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, ws, port, out):
    import sys
    import time
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        got = bench.max_over_ranks(10.0 * (rank + 1))
        assert bench.dist_env() == (ws, rank, rank)
        # the reference arm: only rank 0 works
        args = type("A", (), {"steps": 1, "warmup": 0, "gpus": ws})()
        t0 = time.perf_counter()
        rc = bench.run_reference(args) if rank != 0 else 0
        out.put((rank, got, rc, time.perf_counter() - t0))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(100)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert [r[1] for r in res] == [20.0, 20.0]       # max over ranks
    assert res[1][2] == 0 and res[1][3] < 5.0         # rank 1 left the reference arm at once
