"""The bench's multi-rank logic on CPU: two gloo ranks (127.0.0.1) run the
same barrier / max / sum and the replica throughput as the NCCL path does on
GPUs -- value = all ranks' tets / the slowest rank's time -- and the gate
before the timed region, where a rank whose host work raised, or that died,
stops every rank with an error instead of a hang."""
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


def _gated_rank(rank, ws, port, q, mode):
    """A rank of the bench's gate before the timed region.  mode: 'raise' --
    rank 1's untimed work raises; 'die' -- rank 1 exits without reaching the
    gate; 'ok' -- both get through."""
    sys.path.insert(0, ROOT)
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank)})
    import time

    import bench
    d = bench.Dist(ws, rank, backend="gloo", timeout_s=20)

    def work():
        if rank == 1 and mode == "raise":
            raise ValueError("rank 1: octree build failed")
        if rank == 1 and mode == "die":
            os._exit(3)
        return rank

    t0 = time.monotonic()
    try:
        r = bench.gated(d, work, "the warm-up")
        q.put((rank, "ok", r, time.monotonic() - t0))
    except bench.RankFailure as e:
        q.put((rank, "peer_failed", str(e), time.monotonic() - t0))
    except ValueError as e:
        q.put((rank, "own_error", str(e), time.monotonic() - t0))


def _run_gated(mode):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_gated_rank, args=(r, 2, port, q, mode)) for r in range(2)]
    for p in procs:
        p.start()
    n = 1 if mode == "die" else 2
    res = sorted(q.get(timeout=120) for _ in range(n))
    for p in procs:
        p.join(timeout=60)
    return res, [p.exitcode for p in procs]


def test_gate_passes_when_every_rank_gets_through():
    pytest.importorskip("torch")
    res, codes = _run_gated("ok")
    assert [(r, k, v) for r, k, v, _ in res] == [(0, "ok", 0), (1, "ok", 1)]
    assert codes == [0, 0]


def test_rank_that_raises_stops_every_rank_before_the_timed_region():
    pytest.importorskip("torch")
    res, _ = _run_gated("raise")
    assert res[0][:2] == (0, "peer_failed") and "no number is reported" in res[0][2]
    assert res[1][:2] == (1, "own_error") and "octree build failed" in res[1][2]


def test_rank_that_dies_is_detected_not_waited_for():
    """Rank 1 exits without reaching the gate: rank 0's collective fails
    (peer gone) or runs into the 20 s process-group timeout, and rank 0 stops
    with RankFailure instead of hanging."""
    pytest.importorskip("torch")
    res, codes = _run_gated("die")
    assert len(res) == 1
    rank, kind, msg, dt = res[0]
    assert (rank, kind) == (0, "peer_failed")
    assert dt < 60
    assert codes[1] == 3
