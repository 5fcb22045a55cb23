"""Replicas over GPUs: independent solves per rank, host-side FP64 reductions.

The path shards by independent solves.  The reference distributes reference
stations over MATLAB ``parfor`` workers (code/calculate_data.m:189,
inversion/optlib_callback_fct/eval_objective_and_gradient.m:35) and its only
cross-solve step is the kernel sum ``grad_parameters = grad_parameters +
grad_i_1 + grad_i_2`` (eval_objective_and_gradient.m:110; the Hessian-vector
product likewise, eval_hessian_vector_product.m:181).  Here each rank owns one
GPU and a share of the stations; per-station results stay on their rank, and
the kernel sum is one FP64 all-reduce of an nx*nz*(n_basis_fct+1) vector on
host tensors (works with the gloo backend; no device collective).
"""
from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np


def station_shard(costs: Sequence[float], world: int, rank: int) -> List[int]:
    """Stations of ``rank``: longest-processing-time assignment by cost
    (grid-point updates), ties to the lower rank; deterministic on every rank."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world / rank")
    load = [0.0] * world
    owner = [0] * len(costs)
    for i in sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i)):
        r = min(range(world), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += float(costs[i])
    return [i for i in range(len(costs)) if owner[i] == rank]


def sum_kernels(local: np.ndarray, group=None) -> np.ndarray:
    """Sum of the ranks' FP64 kernel arrays (every rank gets the sum).

    ``local`` is this rank's sum over its stations.  Without an initialised
    process group the local array is returned unchanged (one replica)."""
    import torch
    import torch.distributed as dist
    a = np.ascontiguousarray(local, dtype=np.float64)
    if not (dist.is_available() and dist.is_initialized()):
        return a.copy()
    t = torch.from_numpy(a.copy())
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.numpy()


def gather_rows(local: dict, n_total: int, group=None) -> Optional[List[np.ndarray]]:
    """Collects {station index: array} from every rank; rank 0 receives the list
    ordered by station index (others get None)."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return [local[i] for i in range(n_total)]
    parts = [None] * dist.get_world_size(group)
    dist.all_gather_object(parts, local, group=group)
    if dist.get_rank(group) != 0:
        return None
    merged = {}
    for p in parts:
        merged.update(p)
    if sorted(merged) != list(range(n_total)):
        raise RuntimeError("stations missing from the gather")
    return [merged[i] for i in range(n_total)]
