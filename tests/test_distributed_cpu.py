"""CPU, world size 2 over gloo: the multi-rank host logic (sharding, gathering, timing reduction)."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from spectrax_gb300.distributed import gather_results, reduce_timing, shard_instances
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        costs = [5.0, 1.0, 3.0, 3.0, 2.0, 8.0, 1.0, 4.0]
        mine = shard_instances(costs, world, rank)
        local = {i: {"rank": rank, "cost": costs[i]} for i in mine}
        merged = gather_results(local)
        t, work = reduce_timing(10.0 + rank, float(len(mine)))
        q.put((rank, sorted(mine), sorted(merged), t, work))
    finally:
        dist.destroy_process_group()


def test_sharding_and_reductions_world2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    shards = [r[1] for r in res]
    assert sorted(shards[0] + shards[1]) == list(range(8))          # every instance exactly once
    assert not set(shards[0]) & set(shards[1])
    for r in res:
        assert r[2] == list(range(8))                              # everyone sees the merged results
        assert r[3] == 11.0                                        # max over ranks
        assert r[4] == 8.0                                         # work summed over ranks
    costs = [5.0, 1.0, 3.0, 3.0, 2.0, 8.0, 1.0, 4.0]
    loads = [sum(costs[i] for i in s) for s in shards]
    assert max(loads) - min(loads) <= max(costs)                   # LPT balance


def test_shard_single_rank_and_errors():
    from spectrax_gb300.distributed import reduce_timing, shard_instances
    assert shard_instances([1.0, 2.0, 3.0], 1, 0) == [0, 1, 2]
    with pytest.raises(ValueError):
        shard_instances([1.0], 2, 2)
    assert reduce_timing(3.0, 4.0) == (3.0, 4.0)                  # no process group


class _Pb:
    """Stand-in for spx_problem with the fields instance_cost reads."""

    def __init__(self, Nx, Nn):
        self.Nx, self.Nn, self.Ns, self.Lx, self.alpha_s = Nx, Nn, 2, 12.0, [1.4]


def _fake_solve(shard, t1, save_ts, rtol, atol, cluster, tile):
    # stands in for the GPU batch launch: y -> 2 y, with the instance's id
    return {k: dict(y=[2 * v for v in it["y0"]], id=it["id"]) for k, it in enumerate(shard)}


def _failing_solve(shard, t1, save_ts, rtol, atol, cluster, tile):
    import torch.distributed as dist
    if dist.get_rank() == 1:
        raise RuntimeError("device out of memory")
    return _fake_solve(shard, t1, save_ts, rtol, atol, cluster, tile)


def _batch_worker(rank, world, port, q, fail):
    import torch.distributed as dist
    from spectrax_gb300.distributed import RankFailure, run_sharded_batch
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        insts = [dict(problem=_Pb(Nx, Nn), y0=[float(i), float(i) + 0.5], id=i)
                 for i, (Nx, Nn) in enumerate([(17, 32), (65, 256), (33, 64), (17, 128), (65, 32), (33, 256)])]
        try:
            out = run_sharded_batch(insts, 1.0, solve_shard=_failing_solve if fail else _fake_solve)
            q.put((rank, "ok", {i: (r["id"], r["y"]) for i, r in out.items()}))
        except RankFailure as exc:
            q.put((rank, "failed", str(exc)))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("fail", [False, True])
def test_run_sharded_batch_world2(fail):
    # every instance solved exactly once and gathered on both ranks; a rank whose
    # shard raises is reported on every rank (no rank hangs in the exchange)
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_batch_worker, args=(r, 2, port, q, fail)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    if not fail:
        for rank, kind, out in res:
            assert kind == "ok"
            assert sorted(out) == list(range(6))
            for i, (ident, y) in out.items():
                assert ident == i and y == [2.0 * i, 2.0 * i + 1.0]
    else:
        for rank, kind, msg in res:
            assert kind == "failed" and "rank 1" in msg and "device out of memory" in msg
