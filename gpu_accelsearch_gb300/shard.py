"""Trial sharding across ranks (one process per GPU).

DM trials are independent, so N GPUs split the trials with no data-path
collective: each rank searches its own share and the candidate lists are
concatenated on the host at the end (all_gather of small host arrays).
"""
from __future__ import annotations

import numpy as np


def shard_trials(ntrials: int, rank: int, world: int, costs=None):
    """Indices of the trials rank `rank` searches.  With per-trial costs
    (e.g. sample counts) the trials are dealt greedily, largest first, to the
    least-loaded rank, so uneven lengths balance; otherwise round-robin."""
    if world <= 1:
        return list(range(ntrials))
    if costs is None:
        return list(range(rank, ntrials, world))
    order = sorted(range(ntrials), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    owner = [0] * ntrials
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        owner[i] = r
        load[r] += costs[i]
    return [i for i in range(ntrials) if owner[i] == rank]


def gather_candidates(local: np.ndarray, trial_ids, group=None) -> np.ndarray:
    """Concatenate every rank's candidates (their `trial` field mapped back
    to global trial indices) and sort them by (trial, step, numharm, z, r)."""
    import torch.distributed as dist
    loc = local.copy()
    if len(loc):
        loc["trial"] = np.asarray(trial_ids)[loc["trial"]]
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        parts = [None] * dist.get_world_size(group)
        dist.all_gather_object(parts, loc, group=group)
        loc = np.concatenate([p for p in parts if p is not None and len(p)] or [loc[:0]])
    return np.sort(loc, order=["trial", "step", "numharm", "z", "r"])
