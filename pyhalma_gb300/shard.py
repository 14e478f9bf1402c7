"""Multi-rank sharding of the unbinding work (one process per GPU).

Haloes are independent, so the data path needs no collective: haloes are dealt to ranks by
longest-processing-time on their cost N_h^2 (largest first, each to the least-loaded rank),
every rank unbinds its own haloes on its own GPU, and the per-halo results are gathered on
the host (``torch.distributed.all_gather_object``) only to assemble the catalogue.  FoF is
not split: a snapshot is processed by one rank, and ranks take different snapshots (the
driver's loop over snapshots, pyHALMA.py:455).
"""
from __future__ import annotations

import heapq

import numpy as np


def partition_haloes(sizes, world):
    """LPT assignment: returns a list (per rank) of ascending halo indices."""
    sizes = np.asarray(sizes, dtype=np.int64)
    order = np.argsort(-(sizes.astype(np.float64) ** 2), kind="stable")
    heap = [(0.0, r) for r in range(world)]
    heapq.heapify(heap)
    out = [[] for _ in range(world)]
    for h in order:
        load, r = heapq.heappop(heap)
        out[r].append(int(h))
        heapq.heappush(heap, (load + float(sizes[h]) ** 2, r))
    return [np.sort(np.asarray(o, dtype=np.int64)) for o in out]


def gather_rows(offsets, halo_ids):
    """Particle rows of the chosen haloes and the CSR offsets of the gathered sub-catalogue."""
    offsets = np.asarray(offsets, dtype=np.int64)
    counts = offsets[halo_ids + 1] - offsets[halo_ids]
    rows = np.concatenate([np.arange(offsets[h], offsets[h + 1]) for h in halo_ids]) if len(halo_ids) else \
        np.zeros(0, dtype=np.int64)
    sub = np.concatenate(([0], np.cumsum(counts))).astype(np.int64)
    return rows, sub


def unbind_sharded(offsets, x, y, z, vx, vy, vz, m, options=None, compute=None, group=None):
    """Every rank unbinds its LPT share; returns the full (bound, halo table) on every rank.

    ``compute`` defaults to :func:`pyhalma_gb300.unbinding.unbind_batched` (the GPU path); it
    receives host arrays of the rank's sub-catalogue and returns (bound, halo_table, _)."""
    import torch.distributed as dist
    if compute is None:
        from .unbinding import unbind_batched as compute
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    offsets = np.asarray(offsets, dtype=np.int64)
    nh = len(offsets) - 1
    parts = partition_haloes(np.diff(offsets), world)
    mine = parts[rank]
    rows, sub = gather_rows(offsets, mine)
    cols = [np.ascontiguousarray(np.asarray(a)[rows]) for a in (x, y, z, vx, vy, vz, m)]
    bound, table, _ = compute(sub, *cols, options) if options is not None else compute(sub, *cols)
    local = (mine, rows, np.asarray(bound), np.asarray(table))
    if world > 1:
        everyone = [None] * world
        dist.all_gather_object(everyone, local, group=group)
    else:
        everyone = [local]
    n = len(np.asarray(x))
    full_bound = np.zeros(n, dtype=np.uint8)
    full_table = None
    for ids, r, b, t in everyone:
        full_bound[r] = b
        if full_table is None:
            full_table = np.zeros((nh, t.shape[1] if t.ndim == 2 and t.shape[0] else 11))
        if len(ids):
            full_table[ids] = t
    if full_table is None:
        full_table = np.zeros((nh, 11))
    return full_bound, full_table
