#!/usr/bin/env python
"""FoF + batched unbinding throughput of one synthetic snapshot (single-GPU workload).

Default workload (one "step"): a 100 Mpc box with 20,000 Plummer haloes whose particle
counts follow dN/dlogN ∝ N^-alpha on [50, 2e5], alpha fitted so that the haloes hold
4.5e7 particles on average, 15 % contaminants per halo (uniform inside 3a at 3 v_esc) and a
uniform background filling the snapshot to 5e7 particles; FoF at LL = 1.5 kpc (exact
reference partition), groups >= 50 members, then iterative unbinding of every group (FP32
pair terms with compensated sums, FP64 reductions, softening 0.1 kpc) until no particle is
removed.  Inputs are seeded synthetic data (no public dataset is involved).  The same line
carries the 2e8-particle, 200,000-halo snapshot (one timed call, FoF stage broken out) under
``full_snapshot``.

Arms:
  default           the GB300 path; `value` = particles/s with inputs resident in HBM,
                    `e2e` = the same through the C ABI from pinned host buffers.
  --impl reference  the reference's CPU algorithm on this host (the oracle port: the KDTree
                    flood fill of fof.py step for step and the float32 potential loop of
                    particle_subroutines.f90 with OpenMP) on a size-stratified sample of the
                    same snapshot, measured per step; the full-snapshot time extrapolated from
                    it is reported under a separate key.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particles/sec FoF+unbinding and pair-interactions/sec, batched FP32 vs FP64 at ≤1e-6"
WORKLOADS = {
    # the default: 20k power-law haloes, 5e7 particles
    "northstar": dict(workload="powerlaw-20k-haloes-50M-particles", particles=50_000_000, haloes=20_000,
                      box_mpc=100.0, halo_sizes="dN/dlogN ~ N^-alpha on [50, 2e5], alpha fitted to a mean of 2250",
                      contaminant_frac=0.15, background_frac=0.10, linking_length_kpc=1.5, min_members=50,
                      softening_kpc=0.1, max_passes=30),
    # 2e6 particles in 500 Plummer spheres (the medium configuration)
    "plummer2m": dict(workload="plummer-2M-500sph-15pc-contaminants", particles=2_000_000, spheres=500,
                      box_mpc=10.0, contaminant_frac=0.15, background_frac=0.10, linking_length_kpc=1.5,
                      min_members=50, softening_kpc=0.1, max_passes=30),
    # 2e8 particles, 200k haloes, 5 % of them in bridged pairs, 20 % background
    "full": dict(workload="full-2e8-particles-200k-haloes", particles=200_000_000, haloes=200_000, box_mpc=100.0,
                 halo_sizes="dN/dlogN ~ N^-alpha on [50, 2e5], alpha fitted to a mean of 800", bridged_frac=0.05,
                 background_frac=0.20, contaminant_frac=0.0, linking_length_kpc=1.5, min_members=50,
                 softening_kpc=0.1, max_passes=30),
}
# FP32-pipe work of the pair kernels, counted from the instruction mix (an FMA is 2 flops):
#   a pair term evaluated for one particle (tiles, incremental passes): 3 sub + 3 fma for
#   r^2 + 1 fma to accumulate = 7 lane-operations, 11 flops, and one rsqrt;
#   a pair evaluated once for both particles (symmetric block kernel, full passes over the
#   haloes above 1024 particles): 3 sub + 3 fma + 2 fma = 8 lane-operations, 13 flops, one
#   rsqrt -- per pair term of the pass (each pair is two terms) 4 lane-operations, 6.5 flops
#   (the diagonal blocks, evaluated per particle, are counted the same way).
FLOPS_PER_TERM, OPS_PER_TERM = 11.0, 7.0
FLOPS_PER_SYM_TERM, OPS_PER_SYM_TERM = 6.5, 4.0
FOF_BYTES_PER_PARTICLE = 28  # FP64 xyz read once + int32 label written once
# CPU samples: every k-th halo by size rank + 1/k of the background; the reference arm runs
# one such sample per step (K + W steps), the GPU arm's cpu_baseline one larger sample
CPU_STRIDE_ARM, CPU_STRIDE_BASELINE = 600, 250


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), d.get("sm_max_mhz", 2070.0), "measured"
    return 6800.0, 2070.0, "fallback"


def make_snapshot(w, seed):
    from pyhalma_gb300 import synth
    if "spheres" in w:
        return synth.plummer_snapshot(w["particles"], w["spheres"], seed=seed, box_mpc=w["box_mpc"],
                                      bg_frac=w["background_frac"], contaminant_frac=w["contaminant_frac"])
    return synth.full_snapshot(w["particles"], w["haloes"], seed=seed, box_mpc=w["box_mpc"],
                               bg_frac=w["background_frac"], bridge_frac=w.get("bridged_frac", 0.0),
                               contaminant_frac=w["contaminant_frac"])


def snapshot(seed):
    """The 2e6-particle Plummer snapshot of the side workloads."""
    return make_snapshot(WORKLOADS["plummer2m"], seed)


# ---------------------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------------------
class ClockSampler:
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # nvidia-smi's start-up (NVML initialisation) stalls CUDA calls of this process for a
        # few hundred milliseconds: wait for its first sample so that it falls before the
        # timed region (on a 7 ms step it had made the wall clock 4x the event clock)
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.02)
        time.sleep(0.2)

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                try:
                    rows.append((float(parts[0]), float(parts[1]), parts[3:7]))
                except ValueError:
                    pass
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "samples": len(rows), "reasons": reasons}


# ---------------------------------------------------------------------------------------
# CPU leg: the reference algorithm on a size-stratified sample of the same snapshot
# ---------------------------------------------------------------------------------------
def cpu_sample(s, stride, seed=7):
    """Indices of the CPU sample: every `stride`-th generating halo in order of size (so the
    sample's halo sizes follow the snapshot's distribution) and 1/stride of the background."""
    hid = np.asarray(s.sphere)
    nh = int(hid.max()) + 1 if hid.size and hid.max() >= 0 else 0
    sizes = np.bincount(hid[hid >= 0], minlength=nh)
    order = np.argsort(sizes, kind="stable")
    picked = np.zeros(nh, dtype=bool)
    picked[order[stride // 2::stride]] = True
    rng = np.random.default_rng(seed)
    take = np.zeros(s.n, dtype=bool)
    take[hid >= 0] = picked[hid[hid >= 0]]
    bg = hid < 0
    take[bg] = rng.random(int(bg.sum())) < 1.0 / stride
    return np.nonzero(take)[0], int(picked.sum())


def cpu_step(s, idx, w, ncores):
    """One step of the reference's CPU path on the particles idx: the KDTree flood fill
    (fof.py:18-79 step for step, one thread, as the reference's serial FoF), groups of >=
    min_members, then per group the iterative escape cut (halo_properties.py:282-361 repeated)
    with the float32 potential loop of particle_subroutines.f90:466-514 (OpenMP over ncores):
    full potential in the first pass, then the potential of the particles removed by the
    previous pass subtracted, as the GPU path does."""
    import oracle
    from oracle import fof_kdtree
    ll = w["linking_length_kpc"] * 1e-3
    t0 = time.perf_counter()
    groups = fof_kdtree.friends_of_friends_serial(s.x[idx], s.y[idx], s.z[idx], ll)
    t_fof = time.perf_counter() - t0
    groups = [np.asarray(g) for g in groups if len(g) >= w["min_members"]]
    pairs = 0.0
    G = 4.3e-9
    t0 = time.perf_counter()
    for g in groups:
        gi = idx[g]
        m_all = s.mass[gi]
        c = [(m_all * a[gi]).sum() / m_all.sum() for a in (s.x, s.y, s.z)]
        px, py, pz = (np.float32(a[gi] - cc) for a, cc in zip((s.x, s.y, s.z), c))
        mf = m_all.astype(np.float32)
        phi = oracle.bf_potential_f32(mf, px, py, pz, px, py, pz, ncores=ncores).astype(np.float64)
        pairs += float(len(gi)) ** 2
        bound = np.ones(len(gi), dtype=bool)
        for _ in range(w["max_passes"]):
            sel = np.nonzero(bound)[0]
            b = gi[sel]
            m = s.mass[b]
            M = m.sum()
            v = [(m * a[b]).sum() / M for a in (s.vx, s.vy, s.vz)]
            e = 0.5 * ((s.vx[b] - v[0]) ** 2 + (s.vy[b] - v[1]) ** 2 + (s.vz[b] - v[2]) ** 2) - G * phi[sel]
            drop = e > 0
            if not drop.any():
                break
            bound[sel[drop]] = False
            gone, keep = sel[drop], np.nonzero(bound)[0]
            if keep.size:
                phi[keep] -= oracle.bf_potential_f32(mf[gone], px[gone], py[gone], pz[gone], px[keep], py[keep],
                                                     pz[keep], ncores=ncores)
                pairs += float(gone.size) * keep.size
    t_unb = time.perf_counter() - t0
    sum_n2 = float(sum(float(len(g)) ** 2 for g in groups))
    return dict(t_fof=t_fof, t_unbind=t_unb, n=len(idx), pairs=pairs, groups=len(groups), sum_n2=sum_n2,
                cores=ncores)


def cpu_extrapolation(d, n_full, sum_n2_full, source):
    """Full-snapshot CPU time from a sample step: FoF time scaled by particles, unbinding time
    by the sum of squared group sizes."""
    t_fof = d["t_fof"] * n_full / max(d["n"], 1)
    t_unb = d["t_unbind"] * sum_n2_full / max(d["sum_n2"], 1.0)
    return {"value": n_full / (t_fof + t_unb), "unit": "particles/s", "seconds": t_fof + t_unb,
            "fof_s": t_fof, "unbind_s": t_unb, "kind": "extrapolated",
            "rule": "FoF seconds x N / N_sample + unbinding seconds x sum N_h^2 / sum N_h^2 of the sample",
            "group_sizes": source}


def cpu_sample_text(d, n_haloes, stride):
    return (f"measured: every {stride}th halo by size rank ({n_haloes} haloes) + 1/{stride} of the background, "
            f"{d['n']} particles; FoF: KDTree flood fill of fof.py step for step, 1 thread ({d['t_fof']:.2f} s); "
            f"unbinding: float32 potential loop of the Fortran with OpenMP on {d['cores']} threads over the "
            f"sample's {d['groups']} groups, full first pass then incremental passes like the GPU "
            f"({d['pairs']:.3g} pair terms, {d['t_unbind']:.2f} s)")


# ---------------------------------------------------------------------------------------
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    world, rank, local = dist_env()
    if rank != 0:
        return 0
    import oracle
    oracle.build()
    w = WORKLOADS[args.workload]
    s = make_snapshot(w, seed=1)
    idx, nsh = cpu_sample(s, CPU_STRIDE_ARM)
    ncores = oracle.ncores_default()
    for _ in range(args.warmup):
        cpu_step(s, idx, w, ncores)
    secs, last = [], None
    t_all = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        last = cpu_step(s, idx, w, ncores)
        secs.append(time.perf_counter() - t0)
    timed = time.perf_counter() - t_all
    step_s = statistics.median(secs)
    value = last["n"] / step_s
    counts = s.meta.get("halo_counts")
    if counts is None:
        counts = s.meta.get("sphere_counts")
    counts = np.asarray(counts, dtype=np.float64)
    counts = counts[counts >= w["min_members"]]
    ext = cpu_extrapolation(last, s.n, float((counts ** 2).sum()), "generating halo sizes >= min_members")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "particles/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
            "timed_region_s": timed, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic", "config": dict(w, particles=s.n),
            "cpu_baseline": {"value": value, "unit": "particles/s", "cores": ncores, "kind": "port",
                             "sample": cpu_sample_text(last, nsh, CPU_STRIDE_ARM)},
            "e2e": {"value": value, "unit": "particles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "pair_interactions_per_s": last["pairs"] / max(last["t_unbind"], 1e-9),
            "extrapolated_full_snapshot": ext}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------------
# the plain FP64 per-halo path, on a size-stratified sample of the haloes
# ---------------------------------------------------------------------------------------
def fp64_sampled(off, members, dev_in, opt, per_class=3, n_classes=8):
    """Times the plain FP64 per-halo path (one pair launch per halo per pass, host-checked
    convergence) on `per_class` haloes of each logarithmic size class, spread evenly over the
    class in size order, and scales each class's time by the class's sum of N_h^2 over the
    sample's; the fixed cost of one call (measured on the smallest sampled halo alone) is taken
    off every class before scaling and counted once.  Also returns the per-halo relative
    potential error of one FP32C pass against one FP64 pass over the same sampled haloes."""
    import torch
    from pyhalma_gb300.unbinding import UnbindOptions, unbind_batched
    dev = dev_in[0].device
    sizes = np.diff(off)
    edges = np.geomspace(max(sizes.min(), 1), sizes.max() + 1, n_classes + 1)
    cls = np.clip(np.searchsorted(edges, sizes, side="right") - 1, 0, n_classes - 1)
    midx = members.long()

    def gather(hs):
        sel = np.concatenate([np.arange(off[h], off[h + 1]) for h in hs])
        soff = np.concatenate([[0], np.cumsum(sizes[hs])]).astype(np.int64)
        arr = [a[midx[torch.from_numpy(sel).to(dev)]].contiguous() for a in dev_in]
        return torch.from_numpy(soff).to(dev), arr

    def timed(doff, arr, o):
        unbind_batched(doff, *arr, o)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _, halo, _ = unbind_batched(doff, *arr, o)
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) * 1e-3, halo

    o64 = UnbindOptions(eps=opt.eps, max_iter=opt.max_iter, precision="fp64")
    picks, rows = [], []
    for c in range(n_classes):
        hs = np.nonzero(cls == c)[0]
        if hs.size == 0:
            continue
        hs = hs[np.argsort(sizes[hs], kind="stable")]
        k = min(per_class, hs.size)
        pick = hs[np.linspace(0, hs.size - 1, k).round().astype(int)]
        picks.append(pick)
        rows.append((c, hs, pick))
    smallest = min((p for p in np.concatenate(picks)), key=lambda h: sizes[h])
    t_fixed, _ = timed(*gather(np.array([smallest])), o64)
    total, classes = t_fixed, []
    for c, hs, pick in rows:
        t, halo = timed(*gather(pick), o64)
        n2c = float((sizes[hs].astype(np.float64) ** 2).sum())
        n2p = float((sizes[pick].astype(np.float64) ** 2).sum())
        est = max(t - t_fixed, 0.0) * n2c / n2p
        total += est
        classes.append({"sizes": [int(edges[c]), int(edges[c + 1])], "haloes": int(hs.size),
                        "sampled": [int(sizes[h]) for h in pick], "sample_s": t, "class_s": est,
                        "passes": [int(v) for v in halo[:, 8].cpu().numpy()]})
    # potential error of one FP32C pass against one FP64 pass on every sampled halo
    allp = np.sort(np.concatenate(picks))
    doff, arr = gather(allp)
    _, _, p32 = unbind_batched(doff, *arr, UnbindOptions(eps=opt.eps, max_iter=1, precision="fp32c"), want_phi=True)
    _, _, p64 = unbind_batched(doff, *arr, UnbindOptions(eps=opt.eps, max_iter=1, precision="fp64"), want_phi=True)
    p32, p64, so = p32.cpu().numpy(), p64.cpu().numpy(), doff.cpu().numpy()
    per_halo = []
    for h in range(len(so) - 1):
        a, b = p32[so[h]:so[h + 1]], p64[so[h]:so[h + 1]]
        both = (a != 0) & (b != 0)
        if both.any():
            per_halo.append(float(np.max(np.abs(a[both] / b[both] - 1.0))))
    err = {"per_halo_max": float(np.max(per_halo)), "per_halo_median": float(np.median(per_halo)),
           "haloes": len(per_halo), "bound": 1e-6, "sample": "the haloes sampled for the FP64 timing"}
    return total, classes, t_fixed, err


# ---------------------------------------------------------------------------------------
def _free_device_memory():
    import gc
    import torch
    from pyhalma_gb300 import _lib
    gc.collect()
    torch.cuda.synchronize()
    _lib.lib().halma_release_workspace()
    torch.cuda.empty_cache()


def full_snapshot_run(args, check_crop=True):
    """The 2e8-particle snapshot: FoF + groups + batched unbinding in one call (one warm-up,
    then args.full_steps timed calls), FoF stages broken out, FoF of a 1e7-particle crop
    checked bit-exact against the C oracle."""
    import torch
    import oracle
    from pyhalma_gb300 import _lib, fof
    from pyhalma_gb300.unbinding import UnbindOptions, find_haloes
    w = WORKLOADS["full"]
    dev = torch.device("cuda", 0)
    t0 = time.perf_counter()
    s = make_snapshot(w, seed=2)
    gen_s = time.perf_counter() - t0
    d = [torch.from_numpy(a).to(dev) for a in (s.x, s.y, s.z, s.vx, s.vy, s.vz, s.mass)]
    ll = w["linking_length_kpc"] * 1e-3
    opt = UnbindOptions(eps=w["softening_kpc"] * 1e-3, max_iter=w["max_passes"])
    _lib.set_profiling(True)
    find_haloes(*d, ll, w["min_members"], options=opt)
    torch.cuda.synchronize()
    ms, fof_ms, unb_ms, stages = [], [], [], []
    for _ in range(max(args.full_steps, 1)):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        cat = find_haloes(*d, ll, w["min_members"], options=opt)
        e1.record()
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
        st = _lib.profile_stats()
        fof_ms.append(st["fof_ms"])
        unb_ms.append(st["unbind_ms"])
        stages.append(_lib.profile_fof_stages())
    hbm, _, src = peaks()
    t_fof = statistics.mean(fof_ms)
    fof_gbs = FOF_BYTES_PER_PARTICLE * s.n / (t_fof * 1e-3) / 1e9
    out = {"workload": w["workload"], "particles": s.n, "haloes_generated": w["haloes"],
           "haloes_found": cat.n_haloes, "ms": statistics.mean(ms), "particles_per_s": s.n / (statistics.mean(ms) * 1e-3),
           "fof_ms": t_fof, "unbind_ms": statistics.mean(unb_ms),
           "fof_stages_ms": {k: statistics.mean(st[k] for st in stages) for k in stages[0]},
           "roofline_fof": {"bound": "hbm", "achieved": fof_gbs, "peak": hbm, "unit": "GB/s", "frac": fof_gbs / hbm,
                            "note": f"{FOF_BYTES_PER_PARTICLE} algorithmic B/particle over the FoF stage; hbm_gbs {src}"},
           "generate_s": gen_s, "alpha": s.meta["alpha"], "timed_calls": len(ms)}
    _lib.set_profiling(False)
    del d, cat
    _free_device_memory()
    if check_crop:
        k = min(args.crop, s.n)
        crop = np.sort(np.argpartition(s.x, k - 1)[:k])
        cx, cy, cz = (np.ascontiguousarray(a[crop]) for a in (s.x, s.y, s.z))
        lab_gpu = fof.fof_labels(cx, cy, cz, ll)
        lab_ref = oracle.fof_labels(cx, cy, cz, ll)
        out["crop_particles"] = int(k)
        out["crop_fof_bit_exact_vs_c_oracle"] = bool(np.array_equal(lab_gpu, lab_ref))
    return out


def run_gpu(args):
    import torch
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from pyhalma_gb300 import _lib
    from pyhalma_gb300.unbinding import UnbindOptions, find_haloes
    w = WORKLOADS[args.workload]
    t0 = time.perf_counter()
    s = make_snapshot(w, seed=1 + rank)
    gen_s = time.perf_counter() - t0
    n = s.n
    ll = w["linking_length_kpc"] * 1e-3
    opt = UnbindOptions(eps=w["softening_kpc"] * 1e-3, max_iter=w["max_passes"], precision="fp32c")
    host = [np.ascontiguousarray(a) for a in (s.x, s.y, s.z, s.vx, s.vy, s.vz, s.mass)]
    dev_in = [torch.from_numpy(a).to(dev) for a in host]
    pinned = [torch.from_numpy(a).pin_memory() for a in host]
    pinned_np = [t.numpy() for t in pinned]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)   # > 129 MB L2
    stream = torch.cuda.current_stream()
    # the FP32 pipe's peak on this GPU: packed and scalar FMA chains, the faster one
    fp32_peak = max(_lib.measure_fp32_fma_rate(packed=True)[0], _lib.measure_fp32_fma_rate(packed=False)[0])
    # the ceiling of the pair arithmetic itself (FP32 pipe and special-function unit together)
    pair_ceiling = _lib.measure_pair_rate()[0]
    term_ceiling = _lib.measure_term_rate()[0]   # the same for the tile kernel's per-particle terms

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    _lib.set_profiling(True)
    for _ in range(args.warmup):   # warm-up steps as the timed ones (the first L2 flush loads its kernel)
        flush.zero_()
        find_haloes(*dev_in, ll, w["min_members"], options=opt)
    torch.cuda.synchronize()

    # timed region: inputs resident in HBM, L2 flushed before every step
    ms, wall_ms, pairs, pair_ms, fof_ms, unbind_ms, passes = [], [], 0.0, 0.0, [], [], []
    sym_pairs, sym_ms, sym_launches, per_pass, stages = 0.0, 0.0, 0, [], []
    sampler = ClockSampler(local)
    sampler.start()
    launches0 = _lib.launch_count()
    barrier()
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        w0 = time.perf_counter()
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        cat = find_haloes(*dev_in, ll, w["min_members"], options=opt)
        e1.record(stream)
        e1.synchronize()
        wall_ms.append((time.perf_counter() - w0) * 1e3)
        ms.append(e0.elapsed_time(e1))
        st = _lib.profile_stats()
        stages.append(_lib.profile_fof_stages())
        fof_ms.append(st["fof_ms"])
        unbind_ms.append(st["unbind_ms"])
        for (p, t), sp, sm in zip(st["passes"], st["sym_pairs"], st["sym_ms"]):
            if p > 0:
                pairs += p
                pair_ms += t
                sym_pairs += sp
            if sp > 0:
                sym_ms += sm
                sym_launches += 1
        passes.append(sum(1 for p, _ in st["passes"] if p > 0))
        per_pass = [[int(p), round(t, 4), int(sp), round(sm, 4)]
                    for (p, t), sp, sm in zip(st["passes"], st["sym_pairs"], st["sym_ms"]) if p > 0]
    barrier()
    wall = time.perf_counter() - wall0
    launches = _lib.launch_count() - launches0
    clocks = sampler.stop()
    n_haloes = cat.n_haloes
    step_ms = statistics.mean(ms)
    if world > 1:
        t = torch.tensor([step_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        step_ms = float(t.item())
    value = n * world / (step_ms * 1e-3)

    # end to end through the C ABI from pinned host buffers (copies inside the timed region)
    _lib.set_profiling(False)

    def h2d_gbs():
        """The host-to-device copy rate of the positions (pinned -> HBM), for context: the
        positions' upload is the one copy on the end-to-end path that nothing overlaps."""
        dst = [torch.empty_like(t, device=dev) for t in pinned[:3]]
        torch.cuda.synchronize()
        c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        c0.record(stream)
        for d_, h_ in zip(dst, pinned[:3]):
            d_.copy_(h_, non_blocking=True)
        c1.record(stream)
        c1.synchronize()
        return 3 * 8 * n / (c0.elapsed_time(c1) * 1e-3) / 1e9

    h2d_before = h2d_gbs()
    e2e_ms, e2e_wall = [], []
    sampler_e2e = ClockSampler(local)
    sampler_e2e.start()
    for k in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        w0 = time.perf_counter()
        e0.record(stream)
        hc = find_haloes(*pinned_np, ll, w["min_members"], options=opt)
        e1.record(stream)
        e1.synchronize()
        if k >= args.warmup:
            e2e_ms.append(e0.elapsed_time(e1))
            e2e_wall.append((time.perf_counter() - w0) * 1e3)
    clocks_e2e = sampler_e2e.stop()
    h2d_after = h2d_gbs()
    ng = hc.n_haloes
    nm = int(hc.offsets[-1]) if ng else 0
    h2d = 7 * 8 * n
    d2h = 4 * n + n + 8 * (ng + 1) + 4 * nm + 8 * 11 * ng
    e2e_step = statistics.mean(e2e_ms)
    if world > 1:
        t = torch.tensor([e2e_step], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_step = float(t.item())

    # the plain FP64 per-halo path on a size-stratified sample, extrapolated to every halo
    fp64 = None
    if not args.skip_fp64 and rank == 0:
        off = cat.offsets.cpu().numpy()
        t_unb64, classes, t_fixed, err = fp64_sampled(off, cat.members, dev_in, opt)
        t_fof = statistics.mean(fof_ms) * 1e-3
        t64 = t_fof + t_unb64
        fp64 = {"value": n / t64, "unit": "particles/s", "ms_per_step": t64 * 1e3, "kind": "extrapolated",
                "speedup_fp32c_vs_fp64": t64 / (step_ms * 1e-3),
                "speedup_unbinding_only": t_unb64 / (statistics.mean(unbind_ms) * 1e-3),
                "rule": "FoF as measured + per size class: (FP64 time of the sampled haloes - one call's fixed "
                        "cost) x sum N_h^2 of the class / sum N_h^2 of the sample, + the fixed cost once",
                "fixed_call_s": t_fixed, "classes": classes, "potential_rel_err_vs_fp64": err}

    hbm, sm_max, src = peaks()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    n_pair_launches = sum(passes)
    flops = FLOPS_PER_TERM * (pairs - sym_pairs) + FLOPS_PER_SYM_TERM * sym_pairs
    lane_ops = OPS_PER_TERM * (pairs - sym_pairs) + OPS_PER_SYM_TERM * sym_pairs
    pipe_ops = fp32_peak * 1e12 / 2.0   # FP32 lane-operations per second at the measured peak
    achieved = flops / (pair_ms * 1e-3) / 1e12 if pair_ms > 0 else 0.0
    pipe = lane_ops / (pair_ms * 1e-3) / pipe_ops if pair_ms > 0 else 0.0
    traffic = {}
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        traffic = json.load(open(tp))
    # the dominant kernel: the symmetric block kernel of the first (full) pass, timed alone
    sym_achieved = FLOPS_PER_SYM_TERM * sym_pairs / (sym_ms * 1e-3) / 1e12 if sym_ms > 0 else 0.0
    sym_pipe = OPS_PER_SYM_TERM * sym_pairs / (sym_ms * 1e-3) / pipe_ops if sym_ms > 0 else 0.0
    peak_note = (f"FP32 peak measured on this GPU by the library's FMA-chain kernel "
                 f"(halma_measure_fp32_fma_rate, packed and scalar, the faster); {sms} SMs, SM clock during the "
                 f"timed region in `clocks`; flops from the instruction mix: 6.5 per pair term on the symmetric "
                 f"block kernel (a pair evaluated once for both particles: 3 sub + 3 fma + 2 fma = 13 flops), "
                 f"11 per term on the per-particle tile kernel (3 sub + 3 fma + 1 fma); 3 of every 8 (7) "
                 f"lane-operations are 1-flop subtractions, so frac <= 0.81 (0.79) at a full FP32 pipe; "
                 f"fp32_pipe_frac = lane-operations / (peak / 2)")
    roofline = {"bound": "fp32", "kernel": "ub_pair_sym_kernel", "achieved": sym_achieved, "peak": fp32_peak,
                "unit": "TFLOP/s", "frac": sym_achieved / fp32_peak if fp32_peak else None,
                "traffic": traffic.get("ub_pair_sym_kernel_bytes_per_launch"),
                "peak_source": peak_note, "fp32_pipe_frac": sym_pipe,
                "pair_terms_per_launch": sym_pairs / max(sym_launches, 1),
                "ms_per_launch": sym_ms / max(sym_launches, 1), "launches_timed": sym_launches,
                "pair_terms_per_s": sym_pairs / (sym_ms * 1e-3) if sym_ms > 0 else 0.0,
                "pair_arithmetic_ceiling": {
                    "pairs_per_s": pair_ceiling,
                    "kernel_pairs_per_s": sym_pairs / 2 / (sym_ms * 1e-3) if sym_ms > 0 else 0.0,
                    "frac": (sym_pairs / 2 / (sym_ms * 1e-3)) / pair_ceiling if sym_ms > 0 and pair_ceiling else None,
                    "note": "measured in the same run by the library's pair-arithmetic kernel "
                            "(halma_measure_pair_rate: the block kernel's per-pair f32x2 sub/fma and rsqrt from "
                            "shared memory, no reductions or bookkeeping, full occupancy); the mix needs the FP32 "
                            "pipe (8 lane-ops per pair) and the special-function unit (1 rsqrt per pair) each at "
                            "its throughput, so this, not the FP32 peak, is the kernel's practical ceiling"}}
    roofline_pairs = {"bound": "fp32", "kernel": "ub_pair_sym_kernel + ub_pair_kernel (every pass)",
                      "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                      "frac": achieved / fp32_peak if fp32_peak else None,
                      "traffic_ub_pair_kernel": traffic.get("ub_pair_kernel_bytes_per_launch"),
                      "fp32_pipe_frac": pipe, "sym_pair_terms": sym_pairs,
                      "tile_kernel_ceiling": {
                          "terms_per_s": term_ceiling,
                          "kernel_terms_per_s": (pairs - sym_pairs) / ((pair_ms - sym_ms) * 1e-3)
                          if pair_ms > sym_ms else 0.0,
                          "frac": ((pairs - sym_pairs) / ((pair_ms - sym_ms) * 1e-3)) / term_ceiling
                          if pair_ms > sym_ms and term_ceiling else None,
                          "note": "ub_pair_kernel (incremental passes and the small haloes' tiles) against the "
                                  "library's term-arithmetic kernel (halma_measure_term_rate: 3 sub + 3 fma + 1 fma "
                                  "as f32x2 and one rsqrt per term, 4 targets per lane, full occupancy)"},
                      "pairs_per_launch": pairs / max(n_pair_launches, 1),
                      "ms_per_launch": pair_ms / max(n_pair_launches, 1), "launches_timed": n_pair_launches,
                      "last_step_passes_pairs_ms_sympairs_symms": per_pass}
    fof_gbs = FOF_BYTES_PER_PARTICLE * n / (statistics.mean(fof_ms) * 1e-3) / 1e9
    roofline_fof = {"bound": "hbm", "achieved": fof_gbs, "peak": hbm, "unit": "GB/s", "frac": fof_gbs / hbm,
                    "traffic": None, "ms": statistics.mean(fof_ms),
                    "stages_ms": {k: statistics.mean(st[k] for st in stages) for k in stages[0]},
                    "note": f"{FOF_BYTES_PER_PARTICLE} algorithmic B/particle over the whole FoF stage "
                            f"(bbox, keys, sort, cells, links, labels, groups); hbm_gbs {src}"}

    line = {"metric": METRIC, "value": value, "unit": "particles/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "wall_ms_per_step": statistics.mean(wall_ms),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator of the configuration; no public dataset)",
            "config": dict(w, particles=n, haloes_found=n_haloes, generate_s=gen_s,
                           l2=f"inputs ({7 * 8 * n / 1e9:.1f} GB) larger than L2, and L2 flushed before every step "
                              f"(256 MB device write)", passes_mean=statistics.mean(passes),
                           fof_ms=statistics.mean(fof_ms), unbind_ms=statistics.mean(unbind_ms), reductions="FP64",
                           parallelism=f"snapshot-per-rank x{world}"),
            "pair_interactions_per_s": pairs / (sum(ms) * 1e-3) * world,
            "roofline": roofline, "roofline_pair_kernels": roofline_pairs, "roofline_fof": roofline_fof,
            "e2e": {"value": n * world / (e2e_step * 1e-3), "unit": "particles/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_step,
                    "steps_ms": [round(v, 2) for v in e2e_ms], "wall_ms_per_step": statistics.mean(e2e_wall),
                    "clocks": clocks_e2e,
                    "h2d_positions_gbs_before_after": [round(h2d_before, 1), round(h2d_after, 1)]},
            "gpu_launches": launches, "clocks": clocks, "fp64_path": fp64, "wall_s_timed": wall}
    if rank == 0 and world == 1 and not args.skip_cpu:
        import oracle
        idx, nsh = cpu_sample(s, CPU_STRIDE_BASELINE)
        d = cpu_step(s, idx, w, oracle.ncores_default())
        v = d["n"] / (d["t_fof"] + d["t_unbind"])
        sizes = np.diff(cat.offsets.cpu().numpy()).astype(np.float64)
        line["cpu_baseline"] = {"value": v, "unit": "particles/s", "cores": d["cores"], "kind": "port",
                                "sample": cpu_sample_text(d, nsh, CPU_STRIDE_BASELINE),
                                "extrapolated_full_snapshot": cpu_extrapolation(d, n, float((sizes ** 2).sum()),
                                                                                "the GPU's FoF groups")}
    del dev_in, pinned, pinned_np, flush, cat, hc
    if rank == 0 and world == 1 and args.workload == "northstar" and not args.skip_full:
        _free_device_memory()
        line["full_snapshot"] = full_snapshot_run(args)
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------------
# other workloads (informative lines, not the contract line)
# ---------------------------------------------------------------------------------------
def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def run_batched(args):
    """20 000 Plummer haloes, dN/dlogN ∝ N^-1 on [50, 2e5] (15 % contaminants): batched FP32C
    unbinding (one persistent launch per pass, graph-replayed) against the plain FP64
    per-halo path, per pass and to convergence."""
    import torch
    from pyhalma_gb300 import _lib, synth
    from pyhalma_gb300.unbinding import UnbindOptions, unbind_batched
    dev = torch.device("cuda", 0)
    cat = synth.powerlaw_catalogue(20_000, seed=1, alpha=args.alpha)
    arrs = [torch.from_numpy(np.ascontiguousarray(a)).to(dev)
            for a in (cat.offsets, cat.x, cat.y, cat.z, cat.vx, cat.vy, cat.vz, cat.mass)]
    out = {"workload": f"batched-20k-haloes-alpha{args.alpha}", "particles": cat.n, "haloes": cat.n_haloes,
           "sum_n2": cat.meta["sum_n2"]}
    _lib.set_profiling(True)
    for name, prec, iters in (("fp32c_pass", "fp32c", 1), ("fp32c_converged", "fp32c", 30),
                              ("fp64_pass", "fp64", 1)):
        opt = UnbindOptions(eps=1e-4, max_iter=iters, precision=prec)
        for _ in range(1 if prec == "fp64" else args.warmup):
            unbind_batched(*arrs, opt)
        reps = 1 if prec == "fp64" else max(args.steps, 1)
        ms = []
        for _ in range(reps):
            e0, e1 = _events()
            e0.record()
            _, halo, _ = unbind_batched(*arrs, opt)
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        t = statistics.mean(ms)
        st = _lib.profile_stats() if prec != "fp64" else None
        pairs = sum(p for p, _ in st["passes"]) if st else cat.meta["sum_n2"]
        out[name] = {"ms": t, "particles_per_s": cat.n / (t * 1e-3), "pairs_per_s": pairs / (t * 1e-3),
                     "passes": int(halo[:, 8].max().item())}
    out["speedup_fp32c_vs_fp64_per_pass"] = out["fp64_pass"]["ms"] / out["fp32c_pass"]["ms"]
    print(json.dumps(out), flush=True)
    return 0


def run_gas(args):
    """One gas halo: 2e6 NFW gas cells (float32 positions) and 5e5 stars; softened FP32C
    potential of all 2.5e6 sources on the gas (the gas cells are the first sources, so the
    gas-gas pairs run once for both cells on the symmetric block kernel and the star terms on
    the tile kernel), then the adjoint (accelerations, dE/dm); relative error against FP64 on
    512 gas targets."""
    import torch
    import oracle
    from pyhalma_gb300 import synth
    from pyhalma_gb300.autograd import potential_f32, softened_potential
    dev = torch.device("cuda", 0)
    g = synth.nfw_gas_halo(2_000_000, 500_000, seed=3)
    sx = np.concatenate([g.gas_x, g.st_x]).astype(np.float32)
    sy = np.concatenate([g.gas_y, g.st_y]).astype(np.float32)
    sz = np.concatenate([g.gas_z, g.st_z]).astype(np.float32)
    sm = np.concatenate([g.gas_mass, g.st_mass]).astype(np.float32)
    T = lambda a, rg=False: torch.tensor(a, device=dev, requires_grad=rg)
    eps = 1e-4
    S = [T(sx, True), T(sy, True), T(sz, True), T(sm, True)]
    ng = len(g.gas_x)
    tx, ty, tz = S[0][:ng], S[1][:ng], S[2][:ng]   # the gas cells, as views of the sources
    potential_f32(*(a.detach() for a in S), *(a.detach() for a in (tx, ty, tz)), eps)
    torch.cuda.synchronize()
    e0, e1 = _events()
    e0.record()
    phi = softened_potential(*S, tx, ty, tz, eps)
    e1.record()
    e1.synchronize()
    fwd = e0.elapsed_time(e1)
    e0, e1 = _events()
    e0.record()
    phi.sum().backward()
    e1.record()
    e1.synchronize()
    bwd = e0.elapsed_time(e1)
    pairs = float(len(sx)) * len(g.gas_x)
    idx = np.random.default_rng(0).choice(len(g.gas_x), 512, replace=False)
    ref = oracle.potential_f64(sm.astype(np.float64), sx.astype(np.float64), sy.astype(np.float64),
                               sz.astype(np.float64), g.gas_x[idx].astype(np.float64),
                               g.gas_y[idx].astype(np.float64), g.gas_z[idx].astype(np.float64),
                               eps2=eps * eps, mask=oracle.MASK_NONE)
    rel = np.abs(phi.detach().cpu().numpy()[idx] / ref - 1)
    print(json.dumps({"workload": "gas-2M-cells-500k-stars", "pairs": pairs,
                      "route": "gas-gas pairs on the symmetric block kernel, star terms on the tile kernel",
                      "forward_ms": fwd,
                      "forward_pairs_per_s": pairs / (fwd * 1e-3), "backward_ms": bwd,
                      "backward": "dL/dm and dL/d(source position) in one sweep over the pairs, dL/d(target "
                                  "position) (the accelerations) in a second",
                      "backward_pair_sweeps_per_s": 2 * pairs / (bwd * 1e-3), "max_rel_err_vs_fp64": float(rel.max()),
                      "median_rel_err_vs_fp64": float(np.median(rel))}), flush=True)
    return 0


def run_full(args):
    """The 2e8-particle snapshot alone (see full_snapshot_run)."""
    print(json.dumps(full_snapshot_run(args)), flush=True)
    return 0


def _timed(fn, reps=3, warmup=1):
    """Mean CUDA-event milliseconds of fn() on the current stream (after warm-up)."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ms = []
    for _ in range(reps):
        e0, e1 = _events()
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    return statistics.mean(ms)


def _groups_csr(groups):
    off = np.zeros(len(groups) + 1, dtype=np.int64)
    np.cumsum([len(g) for g in groups], out=off[1:])
    mem = np.concatenate([np.asarray(g, dtype=np.int32) for g in groups]) if off[-1] else np.zeros(0, np.int32)
    return off, mem


def _cpu_sample(groups, every, fn):
    """Runs fn(group) on every `every`-th group; returns (seconds, particles of the sample)."""
    t0 = time.perf_counter()
    npart = 0
    for g in groups[::every]:
        fn(g)
        npart += len(g)
    return time.perf_counter() - t0, npart


def run_substructure(args):
    """Substructure identification (pyHALMA.py:703-766) of the FoF groups of a bridged
    snapshot: 1000 sphere pairs joined by streams + 1000 lone spheres in a 20 Mpc box."""
    import ctypes
    import torch
    import oracle
    from oracle import fof_kdtree
    from oracle.reductions import center_of_mass, half_mass_radius
    from pyhalma_gb300 import _lib, fof, substructure, synth
    dev = torch.device("cuda", 0)
    s = synth.bridged_snapshot(1000, 1000, seed=5, box_mpc=20.0)
    off, mem = fof.fof_groups(fof.fof_labels(s.x, s.y, s.z, 0.0015), 50)
    groups = [mem[off[g]:off[g + 1]] for g in range(len(off) - 1)]
    prm = (0.0015, 25, 2.0, 0.0005, 0.75, 50)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    dx, dy, dz, dm, doff, dmem = T(s.x), T(s.y), T(s.z), T(s.mass), T(off), T(mem)
    cap = len(groups) + len(mem) // 25 + 1
    oo, om = torch.zeros(cap + 1, dtype=torch.int64, device=dev), torch.zeros(max(len(mem), 1), dtype=torch.int32,
                                                                                  device=dev)
    P = _lib.SubstructureParams(*prm[:1], prm[2], prm[3], prm[4], prm[1], prm[5])
    n_out, n_cut = ctypes.c_int64(0), ctypes.c_int64(0)

    def gpu():
        st = _lib.lib().halma_split_bridges(s.n, *[_lib.ptr(a) for a in (dx, dy, dz, dm)], len(groups),
                                            _lib.ptr(doff), _lib.ptr(dmem), ctypes.byref(P), ctypes.byref(n_out),
                                            cap, _lib.ptr(oo), _lib.ptr(om), ctypes.byref(n_cut),
                                            _lib.stream_of(dx))
        _lib.check(st, "halma_split_bridges")
    ms = _timed(gpu, reps=max(args.steps, 3), warmup=args.warmup)
    t0 = time.perf_counter()
    out, cut = substructure.identify_substructure(groups, s.x, s.y, s.z, s.mass, *prm)
    e2e = time.perf_counter() - t0
    # CPU: the reference's per-group loop with its KD-tree FoF on a sample of the groups

    def one(pl):
        pl = np.asarray(pl)
        cx, cy, cz, M = center_of_mass(pl, s.x, s.y, s.z, s.mass)
        half_mass_radius(cx, cy, cz, M, pl, s.x, s.y, s.z, s.mass)
        fof_kdtree.friends_of_friends_serial(s.x[pl], s.y[pl], s.z[pl], 0.00075)
    every = max(1, len(groups) // 40)
    t_cpu, n_cpu = _cpu_sample(groups, every, one)
    nm = len(mem)
    print(json.dumps({"workload": "substructure-bridged-1000pairs-1000single", "particles_in_groups": nm,
                      "groups_in": len(groups), "groups_out": int(n_out.value), "cut": int(n_cut.value),
                      "gpu_ms": ms, "gpu_particles_per_s": nm / (ms * 1e-3),
                      "e2e_s_host_arrays": e2e, "e2e_particles_per_s": nm / e2e,
                      "cpu_baseline": {"value": n_cpu / t_cpu, "unit": "particles/s", "cores": 1, "kind": "port",
                                       "sample": f"every {every}th group ({n_cpu} particles): centre of mass, "
                                                 f"half-mass radius and the KD-tree FoF at LL/2 per group"},
                      "speedup_vs_cpu": (nm / (ms * 1e-3)) / (n_cpu / t_cpu)}), flush=True)
    return 0


def run_gather(args):
    """Ball gather of the gas / potential set-up (halo_gas.py:223-277) on the 2e6-particle
    snapshot: spheres of 2 r_half (FACTOR_R12_POT) around every FoF group's centre."""
    import ctypes
    import torch
    from scipy.spatial import KDTree
    from pyhalma_gb300 import _lib, fof, halo_gas, halo_properties
    dev = torch.device("cuda", 0)
    s = snapshot(1)
    off, mem = fof.fof_groups(fof.fof_labels(s.x, s.y, s.z, 0.0015), 50)
    red = halo_properties.halo_reductions(off, *(np.ascontiguousarray(a[mem]) for a in
                                                 (s.x, s.y, s.z, s.vx, s.vy, s.vz, s.mass)))
    F = {k: i for i, k in enumerate(_lib.RED_FIELDS)}
    cx, cy, cz = (np.ascontiguousarray(red[:, F[k]]) for k in ("cx", "cy", "cz"))
    R = np.ascontiguousarray(2.0 * red[:, F["r05"]])
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d = [T(a) for a in (s.x, s.y, s.z, cx, cy, cz, R)]
    k = len(R)
    doff = torch.zeros(k + 1, dtype=torch.int64, device=dev)
    found = ctypes.c_int64(0)
    pts, balls = [_lib.ptr(a) for a in d[:3]], [_lib.ptr(a) for a in d[3:]]
    st = _lib.lib().halma_ball_gather(s.n, *pts, k, *balls, 0, _lib.ptr(doff), None, 0, ctypes.byref(found),
                                      _lib.stream_of(d[0]))
    _lib.check(st, "halma_ball_gather")
    total = int(found.value)
    didx = torch.zeros(max(total, 1), dtype=torch.int32, device=dev)

    def gpu():
        st = _lib.lib().halma_ball_gather(s.n, *pts, k, *balls, 0, _lib.ptr(doff), _lib.ptr(didx), total,
                                          ctypes.byref(found), _lib.stream_of(d[0]))
        _lib.check(st, "halma_ball_gather")
    ms = _timed(gpu, reps=max(args.steps, 3), warmup=args.warmup)
    t0 = time.perf_counter()
    halo_gas.balls_inside(s.x, s.y, s.z, cx, cy, cz, R)
    e2e = time.perf_counter() - t0
    # CPU: the reference's calls, a KD-tree over the stars and one query_ball_point per halo
    t0 = time.perf_counter()
    tree = KDTree(np.array((s.x, s.y, s.z)).T)
    t_build = time.perf_counter() - t0
    t0 = time.perf_counter()
    nq = 0
    for h in range(k):
        nq += len(tree.query_ball_point([cx[h], cy[h], cz[h]], R[h], workers=1))
    t_query = time.perf_counter() - t0
    print(json.dumps({"workload": "ball-gather-2M-snapshot-2r05", "particles": s.n, "spheres": k,
                      "particles_found": total, "gpu_ms": ms, "gpu_spheres_per_s": k / (ms * 1e-3),
                      "gpu_found_per_s": total / (ms * 1e-3), "e2e_s_host_arrays": e2e,
                      "cpu_baseline": {"value": nq / (t_build + t_query), "unit": "particles found/s", "cores": 1,
                                       "kind": "reference",
                                       "sample": f"scipy KDTree build ({t_build:.2f} s) + query_ball_point per halo "
                                                 f"({t_query:.2f} s) over all {k} spheres, 1 worker"},
                      "speedup_vs_cpu": (total / (ms * 1e-3)) / (nq / (t_build + t_query))}), flush=True)
    return 0


def run_psc(args):
    """Phase-space cleaning (pyHALMA.py:774-877) of the 2e6-particle snapshot's FoF groups."""
    import ctypes
    import torch
    import oracle.phase_space as ops
    from pyhalma_gb300 import _lib, fof, phase_space
    dev = torch.device("cuda", 0)
    s = snapshot(1)
    off, mem = fof.fof_groups(fof.fof_labels(s.x, s.y, s.z, 0.0015), 50)
    groups = [mem[off[g]:off[g + 1]] for g in range(len(off) - 1)]
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d = [T(a) for a in (s.x, s.y, s.z, s.vx, s.vy, s.vz, s.mass)]
    doff, dmem = T(off), T(mem)
    G, nm = len(groups), len(mem)
    ctl = torch.zeros(nm, dtype=torch.uint8, device=dev)
    which = torch.zeros(3 * nm, dtype=torch.int32, device=dev)
    nw = torch.zeros(G, dtype=torch.int64, device=dev)
    table = torch.zeros(G * len(_lib.PSC_FIELDS), dtype=torch.float64, device=dev)
    P = _lib.PscParams(0.0015, 1.0, 3.0, 1, 50, 50, 100_000)

    def gpu():
        st = _lib.lib().halma_phase_space_clean(s.n, *[_lib.ptr(a) for a in d], G, _lib.ptr(doff), _lib.ptr(dmem),
                                                ctypes.byref(P), _lib.ptr(ctl), _lib.ptr(which), _lib.ptr(nw),
                                                _lib.ptr(table), _lib.stream_of(d[0]))
        _lib.check(st, "halma_phase_space_clean")
    ms = _timed(gpu, reps=max(args.steps, 3), warmup=args.warmup)
    t0 = time.perf_counter()
    phase_space.phase_space_cleaning(groups, s.x, s.y, s.z, s.vx, s.vy, s.vz, s.mass, 0.0015, 1.0, 3.0, True, 50)
    e2e = time.perf_counter() - t0
    every = max(1, G // 30)
    t0 = time.perf_counter()
    sample = groups[::every]
    ops.phase_space_cleaning(sample, s.x, s.y, s.z, s.vx, s.vy, s.vz, s.mass, 0.0015, 1.0, 3.0, True, 50)
    t_cpu = time.perf_counter() - t0
    n_cpu = sum(len(g) for g in sample)
    passes = table.view(G, -1)[:, _lib.PSC_FIELDS.index("passes")].cpu().numpy()
    print(json.dumps({"workload": "phase-space-cleaning-2M-snapshot", "particles_in_groups": nm, "groups": G,
                      "max_sweeps": int(passes.max()), "gpu_ms": ms, "gpu_particles_per_s": nm / (ms * 1e-3),
                      "e2e_s_host_arrays": e2e,
                      "cpu_baseline": {"value": n_cpu / t_cpu, "unit": "particles/s", "cores": 1, "kind": "port",
                                       "sample": f"every {every}th group ({n_cpu} particles), NumPy restatement of "
                                                 f"calc_cell / clean_cell"},
                      "speedup_vs_cpu": (nm / (ms * 1e-3)) / (n_cpu / t_cpu)}), flush=True)
    return 0


def run_props(args):
    """The O(N) per-halo properties (pyHALMA.py:930-1016) of the 2e6-particle snapshot's groups
    after phase-space cleaning."""
    import ctypes
    import torch
    import oracle.properties as op
    from oracle.reductions import CM_velocity, half_mass_radius, sigma_effective
    from pyhalma_gb300 import _lib, fof, phase_space
    dev = torch.device("cuda", 0)
    s = snapshot(1)
    arrays = (s.x, s.y, s.z, s.vx, s.vy, s.vz, s.mass)
    off, mem = fof.fof_groups(fof.fof_labels(s.x, s.y, s.z, 0.0015), 50)
    groups = [mem[off[g]:off[g + 1]] for g in range(len(off) - 1)]
    cl = phase_space.phase_space_cleaning(groups, *arrays, 0.0015, 1.0, 3.0, True, 50)
    ng = cl["new_groups"]
    coff, cmem = _groups_csr(ng)
    cen = np.stack([np.asarray(cl[k], dtype=np.float64) for k in ("center_x", "center_y", "center_z", "masses",
                                                                    "rmax")], 1)
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d = [T(a) for a in arrays]
    doff, dmem, dcen = T(coff), T(cmem), T(cen)
    G, nm = len(ng), len(cmem)
    out = torch.zeros(G * len(_lib.PROP_FIELDS), dtype=torch.float64, device=dev)

    def gpu():
        st = _lib.lib().halma_halo_properties(s.n, *[_lib.ptr(a) for a in d], G, _lib.ptr(doff), _lib.ptr(dmem),
                                              _lib.ptr(dcen), 0.0015, _lib.ptr(out), _lib.stream_of(d[0]))
        _lib.check(st, "halma_halo_properties")
    ms = _timed(gpu, reps=max(args.steps, 3), warmup=args.warmup)
    every = max(1, G // 30)

    def one(h):
        pl = ng[h]
        cx, cy, cz, M, rmax = cen[h]
        r05 = half_mass_radius(cx, cy, cz, M, pl, s.x, s.y, s.z, s.mass)
        rp = op.half_mass_radius_proj(cx, cy, cz, M, pl, s.x, s.y, s.z, s.mass)
        ux, uy, uz = CM_velocity(M, pl, s.vx, s.vy, s.vz, s.mass)
        jx, jy, jz = op.angular_momentum(M, pl, *arrays[:6], s.mass, cx, cy, cz, ux, uy, uz)
        op.tully_fisher_velocity(pl, cx, cy, cz, s.x, s.y, s.z, ux, uy, uz, jx, jy, jz, s.vx, s.vy, s.vz, s.mass, r05)
        op.kinematic_morphology(pl, *arrays[:6], s.mass, cx, cy, cz, ux, uy, uz, jx, jy, jz)
        op.halo_shape_fortran(pl, s.x, s.y, s.z, s.mass, cx, cy, cz, r05)
        sigma_effective(pl, r05, s.x, s.y, s.z, s.vx, s.vy, s.vz, cx, cy, cz, ux, uy, uz)
        grid = np.arange(-(rmax + 0.0015), rmax + 0.0015, 2 * 0.0015)
        op.sigma_projections_fortran(grid, len(grid), pl, *arrays[:6], ux, uy, uz, s.mass, cx, cy, cz, *rp, 0.0015)
    t0 = time.perf_counter()
    n_cpu = 0
    for h in range(0, G, every):
        one(h)
        n_cpu += len(ng[h])
    t_cpu = time.perf_counter() - t0
    print(json.dumps({"workload": "halo-properties-2M-snapshot", "particles_in_groups": nm, "groups": G,
                      "gpu_ms": ms, "gpu_particles_per_s": nm / (ms * 1e-3),
                      "cpu_baseline": {"value": n_cpu / t_cpu, "unit": "particles/s", "cores": 1, "kind": "port",
                                       "sample": f"every {every}th group ({n_cpu} particles): NumPy restatements of "
                                                 f"the numba functions, C restatement of the Fortran ones"},
                      "speedup_vs_cpu": (nm / (ms * 1e-3)) / (n_cpu / t_cpu)}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["northstar", "plummer2m", "batched", "gas", "full", "substructure",
                                           "gather", "psc", "props"], default="northstar")
    ap.add_argument("--alpha", type=float, default=1.0)
    ap.add_argument("--full-steps", type=int, default=2)
    ap.add_argument("--crop", type=int, default=10_000_000)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-full", action="store_true")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="multiply the particle and halo counts of the workload (small cases for profiling)")
    args = ap.parse_args()
    if args.scale != 1.0:
        for w in WORKLOADS.values():
            w["particles"] = int(round(w["particles"] * args.scale))
            if "haloes" in w:
                w["haloes"] = int(round(w["haloes"] * args.scale))
            if "spheres" in w:
                w["spheres"] = max(1, int(round(w["spheres"] * args.scale)))
            w["workload"] += f"-scaled-{args.scale:g}"
    if args.impl == "reference":
        if args.workload not in ("northstar", "plummer2m"):
            args.workload = "northstar"
        return run_reference(args)
    from pyhalma_gb300 import build
    build.build()
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "gas":
        return run_gas(args)
    if args.workload == "full":
        return run_full(args)
    if args.workload == "substructure":
        return run_substructure(args)
    if args.workload == "gather":
        return run_gather(args)
    if args.workload == "psc":
        return run_psc(args)
    if args.workload == "props":
        return run_props(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
