"""Multi-rank sharding of the halo-finding path (one process per GPU).

Unbinding: haloes are independent, so the data path needs no collective: haloes are dealt to
ranks by longest-processing-time on their cost N_h^2 (largest first, each to the least-loaded
rank), every rank unbinds its own haloes on its own GPU, and the per-halo results are gathered
on the host (``torch.distributed.all_gather_object``) only to assemble the catalogue.

FoF (``fof_slabs``): the box is cut into x-slabs at least one linking length wide, one per
rank.  Each rank receives from its two neighbours their particles within one linking length
of the shared face (ghosts), runs the FoF of its own particles plus the ghosts on its own GPU,
and reports, for every particle that lives on two ranks, the smallest global id of the local
component it fell in.  One all-gather of those (id, component minimum) pairs, a union of them
and a relabel to the smallest global id give every rank the exact global partition for its
own particles.  The reference's decomposed FoF (fof.py:95-176) instead cuts the box into
sub-cubes with a fixed 0.1 Mpc buffer and deduplicates groups by centre of mass, which can
split groups longer than the buffer; this one is exact for any group size.
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


# ---------------------------------------------------------------------------------------
# FoF over x-slabs
# ---------------------------------------------------------------------------------------
def slab_edges(xmin, xmax, world, linking_length):
    """x edges of the slabs (len = slabs + 1): `world` slabs of equal width, fewer when the
    box is narrower than world linking lengths (every slab is at least one linking length
    wide, so a ghost layer only ever comes from the two neighbouring slabs).  The last edge is
    nudged above xmax so that every particle falls in [edges[r], edges[r + 1])."""
    width = float(xmax) - float(xmin)
    k = int(max(1, min(world, width // max(float(linking_length), 1e-300)))) if width > 0 else 1
    edges = float(xmin) + width * np.arange(k + 1) / k
    edges[-1] = np.nextafter(float(xmax), np.inf)
    return edges


def slab_of(x, edges):
    """Slab index of every particle."""
    return np.clip(np.searchsorted(edges, np.asarray(x), side="right") - 1, 0, len(edges) - 2)


def _merge_pairs(pairs):
    """Union of (id, id) pairs; returns (ids, root) with root[k] the smallest id connected to
    ids[k]."""
    if len(pairs) == 0:
        return np.zeros(0, dtype=np.int64), np.zeros(0, dtype=np.int64)
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components
    pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    ids, inv = np.unique(pairs, return_inverse=True)
    inv = inv.reshape(-1, 2)
    k = len(ids)
    g = coo_matrix((np.ones(len(inv)), (inv[:, 0], inv[:, 1])), shape=(k, k))
    _, comp = connected_components(g, directed=False)
    cmin = np.full(comp.max() + 1, np.iinfo(np.int64).max, dtype=np.int64)
    np.minimum.at(cmin, comp, ids)
    return ids, cmin[comp]


def fof_slabs(x, y, z, gid, linking_length, edges, local_fof=None, group=None):
    """FoF of the rank's slab particles (x in [edges[rank], edges[rank + 1])), exact across
    slab faces.  ``gid`` are the particles' global ids (their index in the whole snapshot).
    Returns int64 labels for the rank's particles: the smallest global id of the FoF
    component (all ranks' particles), -1 for particles without a friend — the labels of
    ``fof.fof_labels`` on the whole snapshot, restricted to this rank.

    ``local_fof(x, y, z, ll)`` is the per-rank FoF (default: the GPU's ``fof.fof_labels``);
    with one rank or one slab no exchange happens."""
    import torch.distributed as dist
    if local_fof is None:
        from .fof import fof_labels as local_fof
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
    gid = np.asarray(gid, dtype=np.int64)
    n = len(x)
    ll = float(linking_length)
    nslab = len(edges) - 1
    if world == 1 or nslab == 1:
        lab = np.asarray(local_fof(x, y, z, ll)).astype(np.int64)
        return np.where(lab >= 0, gid[np.maximum(lab, 0)], -1)
    if rank >= nslab:
        lo_face, hi_face = np.inf, -np.inf   # a rank without a slab holds no particles
    else:
        lo_face, hi_face = edges[rank], edges[rank + 1]
    # ghosts: own particles within ll of a face (plus a hair against the rounding of the
    # face +- ll), for the neighbour across it; sending a few too many changes nothing
    pad = 1e-9 * (ll + max(abs(lo_face), abs(hi_face))) if rank < nslab else 0.0
    down = np.nonzero(x <= lo_face + ll + pad)[0] if rank > 0 else np.zeros(0, dtype=np.int64)
    up = np.nonzero(x >= hi_face - ll - pad)[0] if rank + 1 < nslab else np.zeros(0, dtype=np.int64)
    pack = lambda idx: (x[idx], y[idx], z[idx], gid[idx])
    everyone = [None] * world
    dist.all_gather_object(everyone, (pack(down), pack(up)), group=group)
    recv = []
    if rank > 0:
        recv.append(everyone[rank - 1][1])          # the lower neighbour's upper ghosts
    if rank + 1 < world:
        recv.append(everyone[rank + 1][0])          # the upper neighbour's lower ghosts
    gx = np.concatenate([x] + [r[0] for r in recv])
    gy = np.concatenate([y] + [r[1] for r in recv])
    gz = np.concatenate([z] + [r[2] for r in recv])
    gg = np.concatenate([gid] + [r[3] for r in recv])
    lab = np.asarray(local_fof(gx, gy, gz, ll)).astype(np.int64)
    # smallest global id of every local component
    member = lab >= 0
    cmin = np.full(len(gx), np.iinfo(np.int64).max, dtype=np.int64)
    np.minimum.at(cmin, lab[member], gg[member])
    comp_min = np.where(member, cmin[np.maximum(lab, 0)], -1)
    # particles held by two ranks (ghosts received and own particles sent): (id, component min)
    shared = np.zeros(len(gx), dtype=bool)
    shared[n:] = True
    shared[down] = True
    shared[up] = True
    shared &= member
    pairs = np.stack([gg[shared], comp_min[shared]], 1)
    allpairs = [None] * world
    dist.all_gather_object(allpairs, pairs, group=group)
    ids, root = _merge_pairs(np.concatenate([p for p in allpairs if len(p)]) if any(len(p) for p in allpairs)
                             else np.zeros((0, 2), dtype=np.int64))
    out = comp_min[:n].copy()
    if len(ids):
        pos = np.searchsorted(ids, out)
        hit = (out >= 0) & (pos < len(ids))
        hit[hit] = ids[pos[hit]] == out[hit]
        out[hit] = root[pos[hit]]
    return out


# ---------------------------------------------------------------------------------------
# one snapshot over several ranks: slab FoF, groups, halo-sharded unbinding
# ---------------------------------------------------------------------------------------
def find_haloes_sharded(x, y, z, vx, vy, vz, m, gid, linking_length, minp, edges, options=None,
                        local_fof=None, compute=None, group=None):
    """FoF + groups of >= minp members + iterative unbinding of one snapshot spread over the
    ranks by x-slab.  Each rank passes its slab's particles and their global ids; returns
    (labels, bound) for those particles — the labels of the single-process FoF (smallest global
    id of the group, -1 alone) and 1 for members of kept groups that survive the unbinding —
    and (halo_ids, table): the groups this rank unbound (identified by their label) and their
    unbinding table rows.

    Groups are dealt to ranks by longest-processing-time on N_h^2; a group's members are sent
    to its rank (one all-gather of the members of groups that span or leave a slab), sorted by
    global id (the reference's member order), unbound there, and the bound flags go back to
    the ranks that hold the particles (one more all-gather).  ``local_fof`` and ``compute``
    default to the GPU's FoF and ``unbinding.unbind_batched``."""
    import torch.distributed as dist
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    if compute is None:
        from .unbinding import unbind_batched as compute
    cols = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z, vx, vy, vz, m)]
    gid = np.asarray(gid, dtype=np.int64)
    lab = fof_slabs(cols[0], cols[1], cols[2], gid, linking_length, edges, local_fof=local_fof, group=group)

    def allgather(obj):
        if world == 1:
            return [obj]
        out = [None] * world
        dist.all_gather_object(out, obj, group=group)
        return out
    # group sizes over all ranks
    inn = lab >= 0
    ul, cnt = np.unique(lab[inn], return_counts=True)
    parts = allgather((ul, cnt))
    allul = np.concatenate([p[0] for p in parts]) if parts else np.zeros(0, dtype=np.int64)
    allcnt = np.concatenate([p[1] for p in parts]) if parts else np.zeros(0, dtype=np.int64)
    labels_g, inv = np.unique(allul, return_inverse=True)
    sizes = np.zeros(len(labels_g), dtype=np.int64)
    np.add.at(sizes, inv, allcnt)
    keep = sizes >= max(int(minp), 1)
    kept, ksize = labels_g[keep], sizes[keep]          # ascending label = the reference's group order
    owner_of = np.full(len(kept), -1, dtype=np.int64)
    for r, hs in enumerate(partition_haloes(ksize, world)):
        owner_of[hs] = r
    # members to their group's rank
    pos = np.searchsorted(kept, lab)
    mine_in = inn & (pos < len(kept))
    mine_in[mine_in] = kept[pos[mine_in]] == lab[mine_in]
    rows = np.nonzero(mine_in)[0]
    send = (lab[rows], gid[rows], np.stack([c[rows] for c in cols], 1))
    got = allgather(send)
    mylab = np.concatenate([g[0] for g in got])
    mygid = np.concatenate([g[1] for g in got])
    mydat = np.concatenate([g[2] for g in got]) if mylab.size else np.zeros((0, 7))
    sel = owner_of[np.searchsorted(kept, mylab)] == rank if mylab.size else np.zeros(0, dtype=bool)
    mylab, mygid, mydat = mylab[sel], mygid[sel], mydat[sel]
    order = np.lexsort((mygid, mylab))                 # groups by label, members by global id
    mylab, mygid, mydat = mylab[order], mygid[order], mydat[order]
    halo_ids, starts = np.unique(mylab, return_index=True)
    off = np.append(starts, len(mylab)).astype(np.int64)
    if len(halo_ids):
        res = compute(off, *[np.ascontiguousarray(mydat[:, q]) for q in range(7)], options) \
            if options is not None else compute(off, *[np.ascontiguousarray(mydat[:, q]) for q in range(7)])
        b, table = np.asarray(res[0]).astype(np.uint8), np.asarray(res[1])
    else:
        b, table = np.zeros(0, dtype=np.uint8), np.zeros((0, 11))
    # bound flags back to the ranks holding the particles
    back = allgather((mygid, b))
    bgid = np.concatenate([g[0] for g in back])
    bval = np.concatenate([g[1] for g in back])
    bound = np.zeros(len(gid), dtype=np.uint8)
    if bgid.size:
        o = np.argsort(bgid, kind="stable")
        bgid, bval = bgid[o], bval[o]
        p2 = np.searchsorted(bgid, gid)
        hit = p2 < len(bgid)
        hit[hit] = bgid[p2[hit]] == gid[hit]
        bound[hit] = bval[p2[hit]]
    return lab, bound, halo_ids, table
