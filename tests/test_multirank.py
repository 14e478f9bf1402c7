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
