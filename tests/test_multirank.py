"""The bench's multi-rank logic on CPU: two gloo ranks (127.0.0.1) run the
same barrier / max / sum and the replica throughput as the NCCL path does on
GPUs -- value = all ranks' tets / the slowest rank's time."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank)})
    import bench
    d = bench.Dist(ws, rank, backend="gloo")
    d.barrier()
    tets = 100.0 * (rank + 1)
    ms = 10.0 * (rank + 1)
    value, ms_max = bench.replica_value(d, tets, ms)
    q.put((rank, d.max(float(rank)), d.sum(1.0), value, ms_max))
    d.barrier()
    d.close()


def test_two_gloo_ranks_replica_value():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, sm, value, ms_max in res:
        assert mx == 1.0 and sm == 2.0
        assert ms_max == 20.0
        assert value == pytest.approx((100.0 + 200.0) / 0.020)
