"""Spreading the batched solves over several GPUs, one process per GPU.

Batched TEMPO instances are independent units (nothing flows between them),
so one batch is partitioned across ranks with no device collective:

* every rank predicts every instance's cost from a short probe of the batch
  on its own GPU (the engine is deterministic, so all ranks predict the same
  costs) -- cost ~ (dkmax + 1) * chi^3, the memory window times the cube of
  the probe's largest bond, the scaling of one TEMPO step;
* ``lpt_partition`` assigns instances to ranks longest-processing-time
  first (the most expensive instance to the least loaded rank), identically
  on every rank;
* each rank solves its part and the states are gathered to rank 0 on the
  host (``gather_rows``), in the batch's order.

``compute_dynamics`` for many systems against one process tensor splits the
systems into contiguous chunks (``split_range``); every rank holds its own
copy of the process tensor in its own GPU's memory (built there; the build
is deterministic) and the states are gathered the same way.

A single TEMPO or PT-TEMPO chain does not shard (its sites depend on one
another step after step): it runs on one GPU.
"""

from typing import Callable, List, Sequence

import numpy as np


def predicted_costs(dkmax: Sequence[int], bonds: Sequence[int]) -> np.ndarray:
    """Cost of one TEMPO step of each instance: memory window x bond^3."""
    return (np.asarray(dkmax, dtype=float) + 1.0) * np.asarray(bonds, dtype=float) ** 3


def probe_costs(instances: Sequence[dict], steps: int = 20, precision: str = "mixed",
                chi_cap: int = 64) -> np.ndarray:
    """Predicted costs from ``steps`` TEMPO steps of the whole batch on this
    GPU (the probe's largest bond per instance)."""
    from .tempo import TempoBatch
    b = TempoBatch(instances, precision=precision, chi_cap=chi_cap, out_cap=2)
    b.advance(steps)
    b.check_status()
    bonds = [b.info(i)["max_bond"] for i in range(b.n)]
    b.close()
    return predicted_costs([int(x["dkmax"]) for x in instances], bonds)


def lpt_partition(costs: Sequence[float], world: int) -> List[List[int]]:
    """Longest-processing-time-first assignment of instances to ``world``
    ranks: instances by decreasing cost (ties by index), each to the rank
    with the least load so far (ties by rank).  Each rank's list is
    returned in increasing instance order.  Deterministic."""
    costs = np.asarray(costs, dtype=float)
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    loads = [0.0] * world
    parts: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (loads[k], k))
        parts[r].append(i)
        loads[r] += float(costs[i])
    return [sorted(p) for p in parts]


def split_range(n: int, world: int) -> List[range]:
    """Contiguous, balanced chunks of ``range(n)`` (sizes differ by <= 1)."""
    base, extra = divmod(n, world)
    out, start = [], 0
    for r in range(world):
        size = base + (1 if r < extra else 0)
        out.append(range(start, start + size))
        start += size
    return out


def gather_rows(local: np.ndarray, parts: Sequence[Sequence[int]], n: int, rank: int,
                world: int, group=None):
    """Rows ``local[k]`` of this rank's instances ``parts[rank][k]`` to rank
    0 in the batch's order (host gather through the process group; rank 0
    returns an array ``[n, ...]``, the other ranks ``None``)."""
    if world == 1:
        return np.asarray(local)
    import torch.distributed as dist
    got = [None] * world if rank == 0 else None
    dist.gather_object(np.asarray(local), got, dst=0, group=group)
    if rank != 0:
        return None
    shape = next(g.shape[1:] for g in got if g.size)
    out = np.empty((n,) + tuple(shape), dtype=got[0].dtype)
    for r in range(world):
        for k, i in enumerate(parts[r]):
            out[i] = got[r][k]
    return out


def run_partitioned(instances: Sequence[dict], costs: Sequence[float],
                    solve: Callable[[List[dict]], np.ndarray], rank: int, world: int, group=None):
    """Solve this rank's cost-balanced part of the batch with ``solve``
    (instances -> states ``[len, ...]``) and gather all states to rank 0."""
    parts = lpt_partition(costs, world)
    mine = [instances[i] for i in parts[rank]]
    local = solve(mine) if mine else np.zeros((0,))
    return gather_rows(local, parts, len(instances), rank, world, group), parts
