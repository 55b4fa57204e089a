"""Replicas over several GPUs, one process per GPU (the q-pool layer of the
reference, Phonon_Calculations/SRC/calculations.F90:42-59 with -D__QPOOL,
without its ScaLAPACK grid: every matrix stays on one GPU).

q-points are independent and the output has one group per q-point, so the
q list is dealt round-robin to the ranks (rank r solves q[r::world]), every
rank solves its share on its own GPU with its own context, and rank 0
collects the results round by round and writes them in global order.  No
collective touches the device data: results travel as host objects over a
gloo group, once per round of `batch` q-points per rank.

Launch: `python -m torch.distributed.run --nproc-per-node N --master-addr
127.0.0.1 ...`; RANK / WORLD_SIZE / LOCAL_RANK / MASTER_* come from the
environment.
"""
from __future__ import annotations

import math
import os
from typing import Callable, Sequence

import numpy as np


def world_info() -> tuple[int, int, int]:
    """(world, rank, local_rank) from the launcher's environment (1, 0, 0 alone)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(nq: int, rank: int, world: int) -> np.ndarray:
    """Global indices of the q-points of `rank`: rank, rank + world, ..."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    return np.arange(rank, nq, world, dtype=np.int64)


def rounds(nq: int, world: int, batch: int) -> int:
    """Rounds every rank takes part in (ranks with fewer q-points solve empty batches)."""
    if batch < 1:
        raise ValueError("batch must be >= 1")
    return math.ceil(math.ceil(nq / world) / batch) if nq > 0 else 0


def init_group(world: int, rank: int, timeout_s: float = 600.0):
    """The gloo process group used for the result gathering (created on the
    default group when torch.distributed is not initialised yet).  A rank that
    dies or never reaches a gathering makes the others' next collective fail
    with an error after at most timeout_s seconds instead of waiting forever."""
    import datetime
    import torch.distributed as dist
    if world == 1:
        return None
    timeout = datetime.timedelta(seconds=timeout_s)
    if not dist.is_initialized():
        dist.init_process_group("gloo", rank=rank, world_size=world, timeout=timeout)
    if dist.get_backend() == "gloo":
        return None  # the default group already is gloo
    return dist.new_group(backend="gloo", timeout=timeout)


def max_over_ranks(x: float, world: int, group=None) -> float:
    """Largest value of x over the ranks (the timing rule of a replicated run)."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def run_sharded(q: np.ndarray, batch: int, solve: Callable[[np.ndarray], Sequence[object]],
                write: Callable[[int, object], None] | None, world: int = 1, rank: int = 0, group=None) -> int:
    """Solve this rank's share of q in rounds of `batch` q-points.

    solve(q_batch) returns one result per row of q_batch; after every round
    rank 0 receives the round's results of all ranks and calls write(t, result)
    for each global index t in increasing order (write may be None on the other
    ranks).  Returns the number of q-points solved by this rank."""
    q = np.asarray(q, dtype=np.float64).reshape(-1, 3)
    mine = shard(len(q), rank, world)
    done = 0
    for r in range(rounds(len(q), world, batch)):
        idx = mine[r * batch:(r + 1) * batch]
        res = list(solve(q[idx])) if len(idx) else []
        if len(res) != len(idx):
            raise RuntimeError(f"solve returned {len(res)} results for {len(idx)} q-points")
        done += len(idx)
        items = list(zip(idx.tolist(), res))
        if world > 1:
            import torch.distributed as dist
            gathered = [None] * world if rank == 0 else None
            dist.gather_object(items, gathered, dst=0, group=group)
            if rank == 0:
                items = [it for part in gathered for it in part]
        if rank == 0:
            for t, rt in sorted(items, key=lambda it: it[0]):
                write(t, rt)
    return done


def split_result(res, count: int) -> list[dict]:
    """Per-q dictionaries of an api.Result (host arrays) for run_sharded."""
    out = []
    for b in range(count):
        m, nz = int(res.m[b]), int(res.nz[b])
        d = {"m": m, "nz": nz, "info": int(res.info[b]), "w": np.array(res.w[b, :m])}
        if res.vel is not None:
            d["vel"] = np.array(res.vel[b, :nz])
        if res.z is not None:
            d["z"] = np.array(res.z[b][:, :nz])
        out.append(d)
    return out
