"""Replicas on several GPUs: one process per GPU, distinct seeds, a host-side argmin.

Chains are independent, so the multi-GPU form of the fit is the reference's own practice of
running separate processes with different seeds (README.md:80-86) and keeping the best output
line (asteroid.c:741-759): no device collective, no peer memory.  Each rank fits on its GPU with
replica_seed(seed, rank); merge() (or gather_best() over torch.distributed) then picks the first
minimum of the per-group results in (rank, group) order, which is the host argmin over the
ranks' output lines concatenated in rank order.
"""
from __future__ import annotations

import numpy as np

_GOLDEN = 0x9E3779B97F4A7C15
_MASK = (1 << 64) - 1


def replica_seed(seed: int, rank: int) -> int:
    """The seed of rank's replica: distinct per rank, rank 0 keeps the caller's seed."""
    return (int(seed) + _GOLDEN * int(rank)) & _MASK


def best_of(result) -> dict:
    """The best group of one rank's result (the first minimum, asteroid.c:741-759)."""
    f = np.asarray(result["best_f"] if isinstance(result, dict) else result.best_f)
    p = np.asarray(result["best_params"] if isinstance(result, dict) else result.best_params)
    dv = np.asarray(result["best_dv"] if isinstance(result, dict) else result.best_dv)
    g = int(np.argmin(f))
    return {"chi2": float(f[g]), "group": g, "params": p[g].tolist(), "dv": dv[g].tolist()}


def merge(bests: list) -> dict:
    """Host argmin over per-rank bests in rank order; ties keep the lowest rank."""
    r = min(range(len(bests)), key=lambda k: (bests[k]["chi2"], k))
    out = dict(bests[r])
    out["rank"] = r
    return out


def gather_best(result, dist) -> dict:
    """All-gather every rank's best over the process group and merge (the same on every rank)."""
    mine = best_of(result)
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return merge([mine])
    got = [None] * dist.get_world_size()
    dist.all_gather_object(got, mine)
    return merge(got)
