"""The oracle against the reference's own outputs (golden fixtures) and known answers.

CPU only.  Pins: (1) scipy's pair predicate, (2) the FoF partition of the reference's
fof.friends_of_friends_serial on adversarial and Plummer inputs, (3) the reference's
reductions, (4) the reference's RPS / most_bound_particle host logic, (5) closed-form
potentials for the float32 restatement of particle_subroutines.f90:466-514.
"""
import hashlib
from fractions import Fraction

import numpy as np
import pytest

import oracle
from oracle import fof_kdtree, reductions
from pyhalma_gb300 import synth


def test_predicate_pairs_pin_sequential_sum(golden):
    d = golden("predicate.npz")
    a, b, r, hit = d["a"], d["b"], d["r"], d["hit"]
    dx, dy, dz = (a - b).T
    seq = (dx * dx + dy * dy) + dz * dz <= r * r
    assert len(hit) == 1200
    assert np.array_equal(seq, hit)
    # the pairs were chosen where other plausible predicates disagree
    alt = np.sqrt(dx * dx + dy * dy + dz * dz) <= r
    assert (alt != hit).sum() > 100


def _cases(d):
    return sorted(set(k.split("__")[0] for k in d.files))


def test_fof_oracle_matches_reference_cases(golden):
    d = golden("fof_cases.npz")
    for name in _cases(d):
        xyz = d[name + "__xyz"]
        ll = float(d[name + "__ll"])
        lab = oracle.fof_labels(xyz[:, 0], xyz[:, 1], xyz[:, 2], ll)
        assert np.array_equal(lab, d[name + "__labels"]), name
        assert len(oracle.labels_to_groups(lab)) == int(d[name + "__ngroups"]), name


def test_fof_kdtree_restatement_matches_reference_cases(golden):
    d = golden("fof_cases.npz")
    for name in _cases(d):
        xyz = d[name + "__xyz"]
        groups = fof_kdtree.friends_of_friends_serial(xyz[:, 0], xyz[:, 1], xyz[:, 2], float(d[name + "__ll"]))
        assert np.array_equal(oracle.groups_to_labels(groups, len(xyz)), d[name + "__labels"]), name


def _config1(golden):
    c = golden("fof_config1.npz")
    s = synth.plummer_snapshot(int(c["n"]), int(c["n_spheres"]), seed=int(c["seed"]), box_mpc=float(c["box_mpc"]))
    h = hashlib.sha256()
    for a in (s.x, s.y, s.z):
        h.update(np.ascontiguousarray(a).tobytes())
    if h.hexdigest() != str(c["sha256"]):
        pytest.skip("this NumPy regenerates a different 1e5-particle snapshot from the seed")
    return s, c


def test_fof_oracle_matches_reference_config1(golden):
    c = golden("fof_config1.npz")
    lab = oracle.fof_labels(c["x"], c["y"], c["z"], float(c["ll"]))
    assert np.array_equal(lab, c["labels"])
    assert len(oracle.labels_to_groups(lab)) == int(c["ngroups"])


def test_config1_generator_reproduces_stored_positions(golden):
    s, c = _config1(golden)     # skips where NumPy's transcendental kernels differ
    assert np.array_equal(s.x, c["x"]) and np.array_equal(s.z, c["z"])


def test_potential_oracle_known_answers():
    # two particles: phi = m / r exactly representable
    phi = oracle.bf_potential_f32([2.0], [0.0], [0.0], [0.0], [3.0], [4.0], [12.0])
    assert phi[0] == np.float32(2.0 / 13.0)
    # the reference mask drops any source sharing one coordinate with the target
    phi = oracle.bf_potential_f32([1.0, 1.0, 1.0], [1.0, 0.0, 2.0], [0.0, 5.0, 2.0], [3.0, 1.0, 2.0],
                                  [0.0], [0.0], [0.0])
    # source 0 shares y=0, source 1 shares x=0, source 2 differs in all three -> 1/sqrt(12)
    assert phi[0] == np.float32(np.float32(1.0) / np.sqrt(np.float32(12.0)))
    # empty sources give zero
    assert oracle.bf_potential_f32([], [], [], [], [1.0], [1.0], [1.0])[0] == 0.0


def test_potential_oracle_f32_is_sequential_float32():
    rng = np.random.default_rng(5)
    src = rng.normal(size=(300, 4)).astype(np.float32)
    src[:, 3] = np.abs(src[:, 3])
    tgt = rng.normal(size=(7, 3)).astype(np.float32)
    got = oracle.bf_potential_f32(src[:, 3], src[:, 0], src[:, 1], src[:, 2], tgt[:, 0], tgt[:, 1], tgt[:, 2])
    for i in range(7):
        acc = np.float32(0)
        for j in range(300):
            d = src[j, :3] - tgt[i]
            if np.all(src[j, :3] != tgt[i]):
                s = np.float32(d[0] * d[0])
                s = np.float32(s + np.float32(d[1] * d[1]))
                s = np.float32(s + np.float32(d[2] * d[2]))
                acc = np.float32(acc + np.float32(src[j, 3] / np.sqrt(s)))
        assert got[i] == acc


def test_potential_oracle_f64_lattice_exact():
    # 3x3x3 lattice of unit masses at integer points; target off-lattice at (0.5, 0.5, 0.5):
    # every source differs in all coordinates; compare with exact sums of 1/sqrt(k)
    g = np.arange(3.0)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    phi = oracle.potential_f64(np.ones(27), X.ravel(), Y.ravel(), Z.ravel(), [0.5], [0.5], [0.5])
    exact = sum(1.0 / np.sqrt(float((Fraction(int(2 * a) - 1, 2)) ** 2 + Fraction(int(2 * b) - 1, 2) ** 2
                                 + Fraction(int(2 * c) - 1, 2) ** 2))
                for a in g for b in g for c in g)
    assert abs(phi[0] - exact) < 1e-13 * exact
    # self mask excludes exactly the diagonal pair, softening enters as r^2 + eps^2
    p = oracle.potential_f64([1.0, 1.0], [0.0, 1.0], [0.0, 0.0], [0.0, 0.0], [0.0, 1.0], [0.0, 0.0], [0.0, 0.0],
                             eps2=0.25, mask=oracle.MASK_SELF)
    assert np.allclose(p, [1.0 / np.sqrt(1.25)] * 2, rtol=0, atol=1e-15)


def test_potential_grad_oracle_matches_finite_differences():
    rng = np.random.default_rng(2)
    n = 40
    x, y, z = rng.normal(size=(3, n))
    m = rng.uniform(0.5, 2.0, n)
    g = rng.normal(size=n)
    eps2 = 0.01
    gm, gs, gt = oracle.potential_grad_f64(m, x, y, z, x, y, z, g, eps2=eps2, mask=oracle.MASK_SELF)
    L = lambda mm, xx: float(g @ oracle.potential_f64(mm, xx, y, z, xx, y, z, eps2=eps2, mask=oracle.MASK_SELF))
    h = 1e-6
    for j in (0, 7, 33):
        e = np.zeros(n)
        e[j] = h
        fd_m = (L(m + e, x) - L(m - e, x)) / (2 * h)
        fd_x = (L(m, x + e) - L(m, x - e)) / (2 * h)
        assert abs(fd_m - gm[j]) < 1e-6 * max(1, abs(fd_m))
        assert abs(fd_x - (gs[j, 0] + gt[j, 0])) < 1e-5 * max(1, abs(fd_x))


def test_reductions_oracle_matches_reference(golden):
    d = golden("halo_props.npz")
    x, y, z, vx, vy, vz, m = (d[k] for k in ("x", "y", "z", "vx", "vy", "vz", "m"))
    for h, row in enumerate(d["results"]):
        pl = d[f"pl{h}"]
        tm, cx, cy, cz, M, ux, uy, uz, rmax, r05, sig = row
        assert np.isclose(reductions.total_mass(pl, m), tm, rtol=1e-12)
        got = reductions.center_of_mass(pl, x, y, z, m)
        assert np.allclose(got, (cx, cy, cz, M), rtol=1e-12, atol=0)
        assert np.allclose(reductions.CM_velocity(M, pl, vx, vy, vz, m), (ux, uy, uz), rtol=1e-11, atol=1e-9)
        assert np.isclose(reductions.furthest_particle(cx, cy, cz, pl, x, y, z), rmax, rtol=1e-12)
        assert np.isclose(reductions.half_mass_radius(cx, cy, cz, M, pl, x, y, z, m), r05, rtol=1e-12)
        assert np.isclose(reductions.sigma_effective(pl, r05, x, y, z, vx, vy, vz, cx, cy, cz, ux, uy, uz), sig,
                          rtol=1e-11)


def test_unbind_oracle_removes_contaminants():
    cat = synth.powerlaw_catalogue(3, seed=1, n_min=300, n_max=600, contaminant_frac=0.15)
    for h in range(3):
        sl = slice(cat.offsets[h], cat.offsets[h + 1])
        bound, it = __import__("oracle.unbind", fromlist=["unbind_halo"]).unbind_halo(
            cat.x[sl], cat.y[sl], cat.z[sl], cat.vx[sl], cat.vy[sl], cat.vz[sl], cat.mass[sl])
        cont = cat.contaminant[sl]
        assert not bound[cont].any()          # 3 v_esc contaminants are all removed
        # sigma = sqrt(GM/6a) at every radius over-heats the outskirts: most members stay bound
        assert bound[~cont].mean() > 0.7
        assert 2 <= it <= 8
