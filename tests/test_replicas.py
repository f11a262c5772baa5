"""The N > 1 paths of bench.py on the CPU.  The single model does not shard: N independent
replicas, joined only by host reductions over gloo (the whole-job value is the sum of the
replicas' simulated years over the slowest replica's time, and every rank waits at the
barriers that bracket the timed region).  The ensemble shards: its independent members split
across the ranks with no exchange, every member on exactly one rank, loads balanced."""
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


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_ensemble_shards_cover_every_member_once(world):
    from eqcycle_gb300.config import ensemble_members, shard_members
    cfgs = ensemble_members(64)
    nodes = [(4 * c.NelX + 1) * (4 * c.NelY + 1) for c in cfgs]
    shards = [shard_members(cfgs, r, world) for r in range(world)]
    flat = sorted(k for sh in shards for k in sh)
    assert flat == list(range(64))
    loads = [sum(nodes[k] for k in sh) for sh in shards]
    assert max(loads) - min(loads) <= max(nodes)
    assert shards == [shard_members(cfgs, r, world) for r in range(world)]   # deterministic
    with pytest.raises(ValueError):
        shard_members(cfgs, world, world)


def _shard_rank_main(rank, ws, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import torch
    import bench
    from eqcycle_gb300.config import ensemble_members, shard_members
    r, n, dist = bench._dist()
    cfgs = ensemble_members(64)
    mine = shard_members(cfgs, r, n)
    mask = torch.zeros(64, dtype=torch.float64)
    mask[mine] = 1.0
    dist.all_reduce(mask)                  # every member counted once over the ranks
    nodes = sum((4 * cfgs[k].NelX + 1) * (4 * cfgs[k].NelY + 1) for k in mine)
    tot = bench._allreduce(dist, nodes, bench._sum_op())
    bench._barrier(dist)
    out.put((r, mask.tolist(), tot, len(mine)))
    dist.destroy_process_group()


def test_ensemble_shards_over_gloo():
    mp = pytest.importorskip("torch.multiprocessing")
    from eqcycle_gb300.config import ensemble_members
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_shard_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    total = sum((4 * c.NelX + 1) * (4 * c.NelY + 1) for c in ensemble_members(64))
    for r, mask, tot, k in res:
        assert mask == [1.0] * 64 and tot == total and k > 0
    assert sum(k for _, _, _, k in res) == 64


def test_bench_refuses_a_gpu_count_without_ranks():
    """bench.py --gpus N needs one rank per GPU (torchrun sets WORLD_SIZE = N): a mismatch exits
    with a message instead of reporting fewer GPUs than asked for."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--gpus", "2", "--steps", "1"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode != 0
    assert "WORLD_SIZE=1" in r.stderr and "torch.distributed.run" in r.stderr
