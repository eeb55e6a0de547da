"""Multi-GPU host logic: one process per GPU, no collective on the data path.

* A single instance does not shard (no reference code splits one solve), so N
  ranks run N independent replicas.
* A batch of independent instances shards: ``shard_instances`` gives each rank
  a cost-balanced subset (longest-processing-time-first), each rank runs its own
  persistent batch launch, and only the small results are gathered at the end.
* ``reduce_timing`` is the max-over-ranks / sum-over-ranks reduction of the
  benchmark (the slowest rank sets the time, every rank's work counts).
"""
from __future__ import annotations

import heapq

import torch


def shard_instances(costs, world: int, rank: int):
    """Indices of the instances rank `rank` solves: greedy LPT over `world` ranks."""
    if world <= 0 or not (0 <= rank < world):
        raise ValueError("bad world/rank")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, r) for r in range(world)]
    heapq.heapify(heap)
    owner = [0] * len(costs)
    for i in order:
        load, r = heapq.heappop(heap)
        owner[i] = r
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [i for i in range(len(costs)) if owner[i] == rank]


def instance_cost(problem) -> float:
    """Relative cost of one 1D1V instance: FFT work per RHS x stability-limited steps."""
    import math
    kmax = (problem.Nx // 2) * 2 * math.pi / problem.Lx
    return (problem.Ns * problem.Nn * problem.Nx * math.log2(problem.Nx + 1)
            * (1.0 + kmax * abs(problem.alpha_s[0]) * math.sqrt(2.0 * problem.Nn)))


def reduce_timing(t_ms: float, work: float, group=None, device=None):
    """(max time over ranks, total work over ranks); identity without a process group."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return float(t_ms), float(work)
    dev = device if device is not None else torch.device("cpu")
    a = torch.tensor([float(t_ms)], dtype=torch.float64, device=dev)
    b = torch.tensor([float(work)], dtype=torch.float64, device=dev)
    dist.all_reduce(a, op=dist.ReduceOp.MAX, group=group)
    dist.all_reduce(b, op=dist.ReduceOp.SUM, group=group)
    return float(a.item()), float(b.item())


def gather_results(local: dict, group=None):
    """Merge per-rank {instance_index: result} dicts on every rank."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return dict(local)
    parts = [None] * dist.get_world_size(group)
    dist.all_gather_object(parts, local, group=group)
    out = {}
    for p in parts:
        out.update(p)
    return out


class RankFailure(RuntimeError):
    """Another rank's shard failed; raised on every rank after the result exchange."""


def solve_shard_on_gpu(shard, t1, save_ts=None, rtol=1e-8, atol=1e-8, cluster=4, tile=16):
    """One persistent batch launch over this rank's instances; {local index: result}."""
    from .batch import BatchSolver
    b = BatchSolver([it["problem"] for it in shard], t1, rtol=rtol, atol=atol, save_ts=save_ts,
                    cluster=cluster, tile=tile, masses=[it.get("masses") or [1.0] * 8 for it in shard])
    ys = b.unpack(b.run(b.pack([it["y0"] for it in shard])))
    stats, ens = b.results()
    return {k: dict(y=ys[k], stats=stats[k], energies=ens[k]) for k in range(len(shard))}


def run_sharded_batch(insts, t1, save_ts=None, rtol=1e-8, atol=1e-8, cluster=4, tile=16, group=None,
                      solve_shard=None):
    """Each rank solves its cost-balanced shard of `insts` (one persistent launch by
    default; `solve_shard(shard, t1, save_ts, rtol, atol, cluster, tile)` replaces
    it) and the per-instance results are gathered on every rank.  A rank whose
    shard raises still takes part in the exchange, so the others learn of the
    failure at once; every rank then raises RankFailure naming it."""
    import torch.distributed as dist
    solve_shard = solve_shard or solve_shard_on_gpu
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    mine = shard_instances([instance_cost(it["problem"]) for it in insts], world, rank)
    local, error = {}, None
    if mine:
        try:
            res = solve_shard([insts[i] for i in mine], t1, save_ts, rtol, atol, cluster, tile)
            local = {mine[k]: v for k, v in res.items()}
        except Exception as exc:            # reported to every rank below
            error = f"rank {rank}: {type(exc).__name__}: {exc}"
    merged = gather_results({("error", rank): error, **local}, group)
    errors = sorted(v for k, v in merged.items() if isinstance(k, tuple) and v is not None)
    if errors:
        raise RankFailure("; ".join(errors))
    return {k: v for k, v in merged.items() if not isinstance(k, tuple)}
