"""Tile-shape autotuner for the batched unbinding pair kernel.

The pair kernel processes a work item of 32*T target slots of one halo (T targets per lane,
T in {1, 2, 4, 8}).  Small T wastes fewer lanes on small haloes and gives more items for load
balance; large T reuses each shared-memory source read for more targets.  For each halo size
class the tuner times one unbinding pass (pair-kernel CUDA events, ``halma_set_profiling``)
over a synthetic catalogue of haloes drawn from that class with every candidate T, keeps the
fastest, and writes the table to ``tile_table.json`` beside this file; ``apply()`` loads a
saved table into the library (``halma_set_tile_table``).
"""
from __future__ import annotations

import json
import os

import numpy as np

from . import _lib

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE_PATH = os.path.join(HERE, "tile_table.json")
CLASS_UPPER = [32, 64, 128, 512, 2048, 8192, 2 ** 31 - 1]
CANDIDATES = [1, 2, 4, 8]


def set_table(upper, tvals):
    u = np.ascontiguousarray(upper, dtype=np.int32)
    t = np.ascontiguousarray(tvals, dtype=np.int32)
    _lib.check(_lib.lib().halma_set_tile_table(len(u), _lib.ptr(u), _lib.ptr(t)), "halma_set_tile_table")


def get_table():
    n = np.zeros(1, dtype=np.int32)
    u = np.zeros(8, dtype=np.int32)
    t = np.zeros(8, dtype=np.int32)
    _lib.check(_lib.lib().halma_get_tile_table(_lib.ptr(n), _lib.ptr(u), _lib.ptr(t)), "halma_get_tile_table")
    k = int(n[0])
    return u[:k].tolist(), t[:k].tolist()


def apply(path=TABLE_PATH):
    """Loads a saved table into the library; returns it (or None when there is none)."""
    if not os.path.exists(path):
        return None
    d = json.load(open(path))
    set_table(d["upper"], d["t"])
    return d


def _class_catalogue(lo, hi, target_pairs, seed):
    from .synth import powerlaw_catalogue
    mean_n2 = ((lo + hi) / 2.0) ** 2
    nh = int(np.clip(target_pairs / mean_n2, 8, 40_000))
    return powerlaw_catalogue(nh, seed=seed, alpha=0.0, n_min=lo, n_max=hi, contaminant_frac=0.0)


def tune(target_pairs=4e9, repeats=3, seed=0, save_path=TABLE_PATH, verbose=True):
    """Times every candidate T on every size class; returns and saves the table."""
    import torch
    from .unbinding import UnbindOptions, unbind_batched
    dev = torch.device("cuda", torch.cuda.current_device())
    best_t, report = [], []
    lo = 1
    for c, hi in enumerate(CLASS_UPPER):
        hi_eff = min(hi, 200_000)
        lo_eff = max(lo, 8)
        cat = _class_catalogue(lo_eff, hi_eff, target_pairs, seed + c)
        arrs = [torch.from_numpy(np.ascontiguousarray(a)).to(dev)
                for a in (cat.offsets, cat.x, cat.y, cat.z, cat.vx, cat.vy, cat.vz, cat.mass)]
        opt = UnbindOptions(eps=1e-4, max_iter=1)
        times = {}
        _lib.set_profiling(True)
        try:
            for t in CANDIDATES:
                set_table([2 ** 31 - 1], [t])
                unbind_batched(*arrs, opt)          # warm-up (graph capture for this shape)
                ms = []
                for _ in range(repeats):
                    unbind_batched(*arrs, opt)
                    st = _lib.profile_stats()
                    pairs, t_ms = st["passes"][0]
                    ms.append(t_ms)
                times[t] = (float(np.median(ms)), pairs)
        finally:
            _lib.set_profiling(False)
        tbest = min(times, key=lambda k: times[k][0])
        best_t.append(tbest)
        report.append({"class_upper": hi, "haloes": cat.n_haloes, "sizes": [lo_eff, hi_eff],
                       "ms": {str(k): v[0] for k, v in times.items()}, "pairs": times[tbest][1],
                       "gpairs_per_s": {str(k): v[1] / v[0] / 1e6 for k, v in times.items()}, "best": tbest})
        if verbose:
            print(f"class <= {hi}: " + ", ".join(f"T={k}: {v[0]:.3f} ms" for k, v in times.items())
                  + f" -> T={tbest}", flush=True)
        lo = hi + 1
    table = {"upper": CLASS_UPPER, "t": best_t, "device": torch.cuda.get_device_name(dev), "report": report}
    set_table(CLASS_UPPER, best_t)
    if save_path:
        with open(save_path, "w") as f:
            json.dump(table, f, indent=1)
    return table


if __name__ == "__main__":
    import sys
    out = sys.argv[1] if len(sys.argv) > 1 else TABLE_PATH
    tune(save_path=out)
