"""N>1 host path on the CPU: LPT halo sharding and the host-side gather over a world-size-2
gloo group.  The per-rank compute is the FP64 oracle (no GPU here); the assembled catalogue
must equal the single-process result."""
import os
import socket

import numpy as np
import pytest

from pyhalma_gb300 import shard, synth


def test_partition_is_complete_and_balanced():
    rng = np.random.default_rng(0)
    sizes = synth.powerlaw_counts(rng, 5000, alpha=1.0, n_min=50, n_max=200_000)
    parts = shard.partition_haloes(sizes, 4)
    allh = np.sort(np.concatenate(parts))
    assert np.array_equal(allh, np.arange(5000))
    loads = [float((sizes[p].astype(float) ** 2).sum()) for p in parts]
    biggest = float(sizes.max()) ** 2
    assert max(loads) - min(loads) <= biggest + 1.0


def _oracle_compute(offsets, x, y, z, vx, vy, vz, m):
    from oracle.unbind import unbind_halo
    n = len(x)
    bound = np.zeros(n, dtype=np.uint8)
    table = np.zeros((len(offsets) - 1, 11))
    for h in range(len(offsets) - 1):
        sl = slice(offsets[h], offsets[h + 1])
        b, it = unbind_halo(x[sl], y[sl], z[sl], vx[sl], vy[sl], vz[sl], m[sl], eps=1e-4, max_iter=20, ncores=1)
        bound[sl] = b
        table[h, 7] = b.sum()
        table[h, 8] = it
    return bound, table, None


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cat = synth.powerlaw_catalogue(12, seed=4, n_min=50, n_max=800)
    b, t = shard.unbind_sharded(cat.offsets, cat.x, cat.y, cat.z, cat.vx, cat.vy, cat.vz, cat.mass,
                                compute=_oracle_compute)
    q.put((rank, b, t))
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_rank_gloo_gather_equals_single_process():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    cat = synth.powerlaw_catalogue(12, seed=4, n_min=50, n_max=800)
    b1, t1, _ = _oracle_compute(cat.offsets, cat.x, cat.y, cat.z, cat.vx, cat.vy, cat.vz, cat.mass)
    for rank, b, t in res:
        assert np.array_equal(b, b1), rank
        assert np.array_equal(t, t1), rank


# ---------------------------------------------------------------------------------------
# FoF over x-slabs: two gloo ranks, the C oracle as each rank's local FoF
# ---------------------------------------------------------------------------------------
def _slab_snapshot():
    """Plummer clumps on both sides of the slab face, one clump sitting on it, and a chain of
    particles 0.9 LL apart crossing the face (a bridge that only the exchange can join)."""
    s = synth.plummer_snapshot(30_000, 12, seed=9, box_mpc=0.4, bg_frac=0.2)
    x0 = 0.5 * (s.x.min() + s.x.max())
    t = np.arange(-60, 61, dtype=np.float64)
    cx = x0 + 0.0009 * t
    cy = np.full(t.shape, 0.07) + 1e-6 * np.sin(t)
    cz = np.full(t.shape, -0.03)
    rng = np.random.default_rng(2)
    blob = rng.normal(0, 0.0007, (400, 3)) + np.array([x0, -0.05, 0.02])
    x = np.concatenate([s.x, cx, blob[:, 0]])
    y = np.concatenate([s.y, cy, blob[:, 1]])
    z = np.concatenate([s.z, cz, blob[:, 2]])
    return x, y, z


def _slab_worker(rank, world, port, q):
    import torch.distributed as dist
    import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    x, y, z = _slab_snapshot()
    ll = 0.0015
    edges = shard.slab_edges(x.min(), x.max(), world, ll)
    mine = np.nonzero(shard.slab_of(x, edges) == rank)[0]
    lab = shard.fof_slabs(x[mine], y[mine], z[mine], mine, ll, edges, local_fof=oracle.fof_labels)
    q.put((rank, mine, lab))
    dist.destroy_process_group()


def test_slab_fof_two_ranks_equals_single_process():
    import multiprocessing as mp
    import oracle
    oracle.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_slab_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    x, y, z = _slab_snapshot()
    ref = oracle.fof_labels(x, y, z, 0.0015)
    got = np.full(len(x), -2, dtype=np.int64)
    for rank, mine, lab in res:
        got[mine] = lab
    assert (got != -2).all()
    assert np.array_equal(got, ref)
    # the chain crosses the face: one group with members on both ranks
    edges = shard.slab_edges(x.min(), x.max(), 2, 0.0015)
    side = shard.slab_of(x, edges)
    chain = np.arange(len(x) - 400 - 121, len(x) - 400)
    assert len(set(got[chain])) == 1 and len(set(side[chain])) == 2


def test_slab_edges_and_single_rank():
    import oracle
    e = shard.slab_edges(0.0, 1.0, 4, 0.3)
    assert len(e) == 4 and e[0] == 0.0 and e[-1] > 1.0          # only 3 slabs fit 0.3 wide
    assert np.all(np.diff(e) >= 0.3)
    x, y, z = _slab_snapshot()
    lab = shard.fof_slabs(x, y, z, np.arange(len(x)), 0.0015, shard.slab_edges(x.min(), x.max(), 1, 0.0015),
                          local_fof=oracle.fof_labels)
    assert np.array_equal(lab, oracle.fof_labels(x, y, z, 0.0015))


def _slab_worker3(rank, world, port, q):
    """Three ranks over a box whose x-extent holds only two slabs: the third rank has no slab
    and no particles but takes part in the exchange."""
    import torch.distributed as dist
    import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    x, y, z = _narrow_snapshot()
    ll = 0.0015
    edges = shard.slab_edges(x.min(), x.max(), world, ll)
    mine = np.nonzero(shard.slab_of(x, edges) == rank)[0] if rank < len(edges) - 1 else np.zeros(0, dtype=np.int64)
    lab = shard.fof_slabs(x[mine], y[mine], z[mine], mine, ll, edges, local_fof=oracle.fof_labels)
    q.put((rank, mine, lab, len(edges) - 1))
    dist.destroy_process_group()


def _narrow_snapshot():
    """A 2.2 LL wide strip of particles (so only two slabs of >= LL fit) with chains along x
    that cross the face."""
    rng = np.random.default_rng(6)
    n = 3000
    x = rng.uniform(0.0, 0.0033, n)
    y = rng.uniform(-0.05, 0.05, n)
    z = rng.uniform(-0.05, 0.05, n)
    t = np.arange(0, 5, dtype=np.float64)
    cx, cy, cz = 0.0002 + 0.0007 * t, np.full(5, 0.01), np.full(5, 0.02)
    return np.concatenate([x, cx]), np.concatenate([y, cy]), np.concatenate([z, cz])


def test_slab_fof_three_ranks_two_slabs():
    import multiprocessing as mp
    import oracle
    oracle.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_slab_worker3, args=(r, 3, port, q)) for r in range(3)]
    for p in procs:
        p.start()
    res = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    x, y, z = _narrow_snapshot()
    ref = oracle.fof_labels(x, y, z, 0.0015)
    got = np.full(len(x), -2, dtype=np.int64)
    for rank, mine, lab, nslab in res:
        assert nslab == 2
        got[mine] = lab
    assert (got != -2).all()
    assert np.array_equal(got, ref)
    assert len(set(got[-5:])) == 1


def _pipeline_snapshot():
    """Contaminated Plummer spheres; the largest one is moved onto the middle of the x-range,
    where the two-slab face lies, so that its group spans both slabs."""
    s = synth.plummer_snapshot(20_000, 10, seed=12, box_mpc=0.3, bg_frac=0.1, contaminant_frac=0.15)
    big = int(np.argmax(np.bincount(s.sphere[s.sphere >= 0])))
    sel = s.sphere == big
    s.x[sel] += 0.5 * (s.x.min() + s.x.max()) - np.median(s.x[sel])
    return s


def _pipeline_worker(rank, world, port, q):
    import torch.distributed as dist
    import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    s = _pipeline_snapshot()
    edges = shard.slab_edges(s.x.min(), s.x.max(), world, 0.0015)
    mine = np.nonzero(shard.slab_of(s.x, edges) == rank)[0]
    cols = [a[mine] for a in (s.x, s.y, s.z, s.vx, s.vy, s.vz, s.mass)]
    lab, bound, ids, table = shard.find_haloes_sharded(*cols, mine, 0.0015, 50, edges, local_fof=oracle.fof_labels,
                                                       compute=_oracle_compute)
    q.put((rank, mine, lab, bound, ids, table))
    dist.destroy_process_group()


def test_sharded_pipeline_two_ranks_equals_single_process():
    """Slab FoF, groups of >= 50, LPT halo sharding and the bound flags sent back: the same
    labels, bound flags and per-halo pass counts as one process doing it all."""
    import multiprocessing as mp
    import oracle
    oracle.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_pipeline_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    s = _pipeline_snapshot()
    lab_ref = oracle.fof_labels(s.x, s.y, s.z, 0.0015)
    groups = [np.asarray(g) for g in oracle.labels_to_groups(lab_ref) if len(g) >= 50]
    off = np.concatenate([[0], np.cumsum([len(g) for g in groups])]).astype(np.int64)
    mem = np.concatenate(groups)
    b_ref, t_ref, _ = _oracle_compute(off, *[a[mem] for a in (s.x, s.y, s.z, s.vx, s.vy, s.vz, s.mass)])
    bound_ref = np.zeros(s.n, dtype=np.uint8)
    bound_ref[mem] = b_ref
    lab = np.full(s.n, -2, dtype=np.int64)
    bound = np.zeros(s.n, dtype=np.uint8)
    tables = {}
    for rank, mine, l, b, ids, table in res:
        lab[mine] = l
        bound[mine] = b
        for h, row in zip(ids, table):
            tables[int(h)] = row
    assert np.array_equal(lab, lab_ref)
    assert np.array_equal(bound, bound_ref)
    assert sorted(tables) == [int(g[0]) for g in groups]
    for k, g in enumerate(groups):
        assert tables[int(g[0])][7] == t_ref[k, 7] and tables[int(g[0])][8] == t_ref[k, 8]
    # some group spans both slabs, and both ranks unbind haloes
    edges = shard.slab_edges(s.x.min(), s.x.max(), 2, 0.0015)
    side = shard.slab_of(s.x, edges)
    assert any(len(set(side[g])) == 2 for g in groups)
    assert all(len(r[4]) > 0 for r in res)
