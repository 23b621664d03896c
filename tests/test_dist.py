"""The N > 1 path on CPU: bench.py runs one independent sphere per rank
(replicas, no data-path collective) and reduces only the timing (max) and the
work done (sum).  Two gloo ranks on 127.0.0.1 check that aggregation."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, ws, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank)})
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    ws_, rank_, local_ = bench.dist_env()
    dist = bench.init_dist(ws_)
    bench.barrier(dist)
    mx = bench.max_over_ranks(dist, 10.0 + rank)        # per-rank timed ms
    sm = bench.sum_over_ranks(dist, 1000.0 * (rank + 1))  # per-rank cell-steps
    q.put((rank, mx, sm))
    dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    out = sorted(q.get(timeout=10) for _ in range(2))
    assert all(p.exitcode == 0 for p in procs)
    for rank, mx, sm in out:
        assert mx == 11.0 and sm == 3000.0
