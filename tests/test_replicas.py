"""Replica plumbing of bench.py over gloo on CPU (world size 2): ranks draw different seeded
workloads, meet only at barriers, and the whole-job time is the max over ranks."""
import os
import socket

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), GS_DIST_BACKEND="gloo")
    import bench
    from gaussium_gb300.workloads import random_shell_quartets
    r, w = bench.dist_init()
    sb, q, _ = random_shell_quartets(16, seed=0 + r)
    bench.barrier(w)
    t = bench.max_over_ranks(1.0 + r, w)
    out.put((r, w, float(sb.centre[0, 0]), t))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_replicas():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [x[0] for x in res] == [0, 1] and all(x[1] == 2 for x in res)
    assert res[0][2] != res[1][2]                   # each replica draws its own workload
    assert all(x[3] == 2.0 for x in res)            # max over ranks
