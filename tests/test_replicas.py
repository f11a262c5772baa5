"""The N > 1 path of bench.py on the CPU: N independent replicas (the single model does not
shard), joined only by host reductions over gloo: the whole-job value is the sum of the
replicas' simulated years over the slowest replica's time, and every rank waits at the
barriers that bracket the timed region."""
import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    r, n, dist = bench._dist()
    assert (r, n) == (rank, ws)
    bench._barrier(dist)
    years = 0.5 + rank            # simulated years of this replica
    secs = 2.0 + 3.0 * rank       # its device time
    tmax = bench._allreduce(dist, secs, bench._max_op())
    tot = bench._allreduce(dist, years, bench._sum_op())
    bench._barrier(dist)
    out.put((rank, tot / (tmax / 3600.0)))
    dist.destroy_process_group()


def test_replicas_reduce_to_the_whole_job_value():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    expect = (0.5 + 1.5) / (5.0 / 3600.0)     # sum of years over the slowest replica's hours
    assert res[0] == pytest.approx(expect) and res[1] == pytest.approx(expect)
