"""Tile-shape autotuner for the batched unbinding pair kernel.

A work item of the pair kernel is 32*T target slots of one halo (T targets per lane,
T in {1, 2, 4}) against one slice of ``slice`` source slots.  Small T wastes fewer lanes on
small haloes and gives more items for load balance; large T reuses each shared-memory source
read for more targets; shorter slices split the biggest haloes into more items so that no
single item outlasts a pass.  The tuner times one unbinding pass (pair-kernel CUDA events,
``halma_set_profiling``) per candidate: first T per halo size class on catalogues drawn from
that class, then the slice length on a power-law catalogue.  The table is written to
``tile_table.json`` beside this file; ``apply()`` loads a saved table into the library
(``halma_set_tile_table``).
"""
from __future__ import annotations

import json
import os

import numpy as np

from . import _lib

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE_PATH = os.path.join(HERE, "tile_table.json")
CLASS_UPPER = [32, 64, 128, 512, 2048, 8192, 2 ** 31 - 1]
CANDIDATES = [1, 2, 4]
SLICES = [1024, 2048, 4096, 8192, 16384, 1 << 20]


def set_table(upper, tvals, slice_len=4096):
    u = np.ascontiguousarray(upper, dtype=np.int32)
    t = np.ascontiguousarray(tvals, dtype=np.int32)
    _lib.check(_lib.lib().halma_set_tile_table(len(u), _lib.ptr(u), _lib.ptr(t), int(slice_len)),
               "halma_set_tile_table")


def get_table():
    """(upper bounds, tile shapes, slice length) currently used by the library."""
    n = np.zeros(1, dtype=np.int32)
    u = np.zeros(8, dtype=np.int32)
    t = np.zeros(8, dtype=np.int32)
    s = np.zeros(1, dtype=np.int32)
    _lib.check(_lib.lib().halma_get_tile_table(_lib.ptr(n), _lib.ptr(u), _lib.ptr(t), _lib.ptr(s)),
               "halma_get_tile_table")
    k = int(n[0])
    return u[:k].tolist(), t[:k].tolist(), int(s[0])


def apply(path=TABLE_PATH):
    """Loads a saved table into the library; returns it (or None when there is none)."""
    if not os.path.exists(path):
        return None
    d = json.load(open(path))
    set_table(d["upper"], d["t"], d.get("slice", 4096))
    return d


def _catalogue(lo, hi, target_pairs, seed, alpha=0.0):
    from .synth import powerlaw_catalogue
    mean_n2 = ((lo + hi) / 2.0) ** 2
    nh = int(np.clip(target_pairs / mean_n2, 8, 40_000))
    return powerlaw_catalogue(nh, seed=seed, alpha=alpha, n_min=lo, n_max=hi, contaminant_frac=0.0)


def _time_pass(arrs, repeats):
    from .unbinding import UnbindOptions, unbind_batched
    opt = UnbindOptions(eps=1e-4, max_iter=1)
    unbind_batched(*arrs, opt)          # warm-up (graph capture for this shape)
    ms = []
    pairs = 0.0
    for _ in range(repeats):
        unbind_batched(*arrs, opt)
        pairs, t_ms = _lib.profile_stats()["passes"][0]
        ms.append(t_ms)
    return float(np.median(ms)), pairs


def tune(target_pairs=4e9, repeats=3, seed=0, save_path=TABLE_PATH, verbose=True):
    """Times every candidate; returns and saves the table."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    to_dev = lambda cat: [torch.from_numpy(np.ascontiguousarray(a)).to(dev)
                          for a in (cat.offsets, cat.x, cat.y, cat.z, cat.vx, cat.vy, cat.vz, cat.mass)]
    from .synth import powerlaw_catalogue
    best_t, report = [], []
    _lib.set_profiling(True)
    try:
        # 1) slice length on the batched workload's size distribution (dN/dlogN ∝ N^-1 on
        #    [50, 2e5], 20 000 haloes) with the default shapes
        big = to_dev(powerlaw_catalogue(20_000, seed=seed + 99, alpha=1.0, contaminant_frac=0.0))
        stimes = {}
        for s in SLICES:
            set_table([32, 64, 2 ** 31 - 1], [1, 2, 4], s)
            stimes[s] = _time_pass(big, repeats)
        sbest = min(stimes, key=lambda k: stimes[k][0])
        if verbose:
            print("slices: " + ", ".join(f"{k}: {v[0]:.3f} ms" for k, v in stimes.items()) + f" -> {sbest}",
                  flush=True)
        # 2) tile shape per size class with that slice
        lo = 1
        for c, hi in enumerate(CLASS_UPPER):
            hi_eff, lo_eff = min(hi, 200_000), max(lo, 8)
            arrs = to_dev(_catalogue(lo_eff, hi_eff, target_pairs, seed + c))
            times = {}
            for t in CANDIDATES:
                set_table([2 ** 31 - 1], [t], sbest)
                times[t] = _time_pass(arrs, repeats)
            tbest = min(times, key=lambda k: times[k][0])
            best_t.append(tbest)
            report.append({"class_upper": hi, "sizes": [lo_eff, hi_eff],
                           "ms": {str(k): v[0] for k, v in times.items()},
                           "gpairs_per_s": {str(k): v[1] / v[0] / 1e6 for k, v in times.items()}, "best": tbest})
            if verbose:
                print(f"class <= {hi}: " + ", ".join(f"T={k}: {v[0]:.3f} ms" for k, v in times.items())
                      + f" -> T={tbest}", flush=True)
            lo = hi + 1
        # 3) the tuned table on the batched workload
        set_table(CLASS_UPPER, best_t, sbest)
        final_ms, final_pairs = _time_pass(big, repeats)
        if verbose:
            print(f"tuned table: {final_ms:.3f} ms per pass ({final_pairs / final_ms / 1e9:.3f} Tpairs/s)", flush=True)
    finally:
        _lib.set_profiling(False)
    table = {"upper": CLASS_UPPER, "t": best_t, "slice": sbest, "device": torch.cuda.get_device_name(dev),
             "report": report, "slice_ms": {str(k): v[0] for k, v in stimes.items()},
             "batched_pass_ms": final_ms, "batched_pass_pairs": final_pairs}
    set_table(CLASS_UPPER, best_t, sbest)
    if save_path:
        with open(save_path, "w") as f:
            json.dump(table, f, indent=1)
    return table


if __name__ == "__main__":
    import sys
    out = sys.argv[1] if len(sys.argv) > 1 else TABLE_PATH
    tune(save_path=out)
