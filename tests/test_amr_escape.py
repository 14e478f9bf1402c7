"""AMR gas conversion (halo_gas.py:9-141) and the single-pass escape cut
(halo_properties.py:282-361) against golden vectors recorded from the reference's own
functions (tests/golden/make_golden.py: amr.npz, escape.npz).

Tolerances: the GPU conversion and the drop-in escape cut are bit-exact (the potential in
its default reference mode is the Fortran loop's float32 arithmetic).  The FP64 oracle pass
(no softening, coordinate mask) may disagree with the reference's float32 cut only for stars
whose FP64 energy lies within 1e-5 of (E_kin + G phi) of zero.
"""
import numpy as np
import pytest

from oracle import amr as oamr
from oracle.unbind import escape_pass

G_CONST = 4.3e-3 * 1e-6


def load_grid(d, key):
    """Rebuilds the reference's grid_data / gas_data tuples from the flat fixture arrays."""
    pn, pr = d[key + "_patchn"], d[key + "_patchr"]
    cells = pn.astype(np.int64).prod(axis=1)
    off = np.concatenate([[0], np.cumsum(cells)])
    fields = []
    for j in range(7):
        flat = d[key + f"_f{j}"]
        flat = flat.astype(np.float64) if j < 5 else flat.astype(bool)
        fields.append([flat[off[p]:off[p + 1]].reshape(tuple(pn[p])) for p in range(len(pn))])
    grid = [None] * 15
    npatch = d[key + "_npatch"]
    grid[2], grid[5] = len(npatch) - 1, npatch
    grid[6], grid[7], grid[8] = pn[:, 0], pn[:, 1], pn[:, 2]
    grid[12], grid[13], grid[14] = pr[:, 0], pr[:, 1], pr[:, 2]
    L, ncoarse, rho_B = d[key + "_scalars"]
    return grid, fields, float(L), int(ncoarse), float(rho_B)


def _levels(npatch):
    return np.concatenate([[0]] + [[lev] * int(c) for lev, c in enumerate(npatch[1:], start=1)]).astype(int)


def _cases(d):
    for k in range(int(d["ngrid"])):
        grid, fields, L, nc, rho_B = load_grid(d, f"g{k}")
        for j in range(int(d["nbox"])):
            R, cx, cy, cz = d[f"g{k}b{j}_box"]
            ref = [d[f"g{k}b{j}_out{q}"] for q in range(8)]
            yield grid, fields, L, nc, rho_B, (float(R), float(cx), float(cy), float(cz)), ref


def test_amr_oracle_matches_reference(golden):
    d = golden("amr.npz")
    for grid, fields, L, nc, rho_B, (R, cx, cy, cz), ref in _cases(d):
        box = np.array([cx - R, cx + R, cy - R, cy + R, cz - R, cz + R])
        got = oamr.amr_to_particles(L, nc, _levels(grid[5]), np.stack(grid[6:9], 1), np.stack(grid[12:15], 1),
                                    fields, box, rho_B)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)


def test_escape_oracle_pass_agrees_with_reference(golden):
    """One FP64 escape pass of the oracle (the formula the iterative unbinding repeats), no
    softening, coordinate mask, on the reference's own sources, against the reference's cut."""
    da, de = golden("amr.npz"), golden("escape.npz")
    for k in range(int(de["ngrid"])):
        grid, fields, L, nc, rho_B = load_grid(da, f"g{k}")
        c = da[f"g{k}_centre"]
        dm = [de[f"g{k}_dm{q}"] for q in range(4)]
        st = {n: de[f"g{k}_{n}"] for n in ("st_x", "st_y", "st_z", "st_vx", "st_vy", "st_vz", "st_mass",
                                           "part_list")}
        pl = st["part_list"]
        for j in range(int(de["ncase"])):
            rete, Rmax, fv, bx, by, bz = de[f"g{k}e{j}_params"]
            R = Rmax
            box = np.array([c[0] - R, c[0] + R, c[1] - R, c[1] + R, c[2] - R, c[2] + R])
            gx, gy, gz, _, _, _, gm, _ = oamr.amr_to_particles(L, nc, _levels(grid[5]), np.stack(grid[6:9], 1),
                                                                np.stack(grid[12:15], 1), fields, box, rho_B)
            gin = np.sqrt((gx - c[0]) ** 2 + (gy - c[1]) ** 2 + (gz - c[2]) ** 2) < Rmax
            din = np.sqrt((dm[0] - c[0]) ** 2 + (dm[1] - c[1]) ** 2 + (dm[2] - c[2]) ** 2) < Rmax
            sx, sy, sz = (np.concatenate([ga[gin], st[n][pl], dm[q][din]])
                          for q, (ga, n) in enumerate(((gx, "st_x"), (gy, "st_y"), (gz, "st_z"))))
            sm = np.concatenate([gm[gin] * rete ** 3, st["st_mass"][pl], dm[3][din]])
            # the f2py wrapper casts to float32 before the loop (halo_gas.py:176-180)
            f = lambda a: a.astype(np.float32).astype(np.float64)
            phi, ek, e = escape_pass(f(sm), f(sx), f(sy), f(sz), f(st["st_x"][pl]), f(st["st_y"][pl]),
                                     f(st["st_z"][pl]), st["st_vx"][pl], st["st_vy"][pl], st["st_vz"][pl],
                                     (bx, by, bz), factor_v=fv, G=G_CONST)
            ref = de[f"g{k}e{j}_bound"]
            diff = (e <= 0) != ref
            scale = np.abs(e) / (ek + G_CONST * fv * fv * phi)
            assert np.all(scale[diff] <= 1e-5), (k, j, scale[diff])
            assert diff.sum() <= 2


@pytest.mark.gpu
def test_gpu_amr_conversion_is_bit_exact(golden, cuda):
    from pyhalma_gb300 import halo_gas
    d = golden("amr.npz")
    for grid, fields, L, nc, rho_B, (R, cx, cy, cz), ref in _cases(d):
        got = halo_gas.AMRgrid_to_particles(L, nc, grid, fields, R, cx, cy, cz, rho_B)
        assert len(got) == 8
        for a, b in zip(got, ref):
            assert a.dtype == np.float64 and np.array_equal(a, b)


@pytest.mark.gpu
def test_gpu_amr_conversion_edge_cases(cuda):
    from pyhalma_gb300 import halo_gas, synth
    g = synth.amr_grid(seed=3)
    # a box far from every patch: no particles, float64 empties
    out = halo_gas.AMRgrid_to_particles(g.L, g.ncoarse, g.grid_data, g.gas_data, 0.01, 30.0, 30.0, 30.0, g.rho_B)
    assert all(a.shape == (0,) and a.dtype == np.float64 for a in out)
    # only the base grid: nothing converted
    grid = list(g.grid_data)
    grid[5] = np.zeros_like(grid[5])
    for q in (6, 7, 8, 12, 13, 14):
        grid[q] = grid[q][:1]
    out = halo_gas.AMRgrid_to_particles(g.L, g.ncoarse, grid, [f[:1] for f in g.gas_data], 1.0, *g.centre, g.rho_B)
    assert all(a.shape == (0,) for a in out)


@pytest.mark.gpu
def test_gpu_escape_cut_is_bit_exact(golden, cuda):
    from pyhalma_gb300 import halo_properties
    da, de = golden("amr.npz"), golden("escape.npz")
    for k in range(int(de["ngrid"])):
        grid, fields, L, nc, rho_B = load_grid(da, f"g{k}")
        c = da[f"g{k}_centre"]
        dm = [de[f"g{k}_dm{q}"] for q in range(4)]
        st = [de[f"g{k}_{n}"] for n in ("st_x", "st_y", "st_z", "st_vx", "st_vy", "st_vz", "st_mass")]
        pl = de[f"g{k}_part_list"]
        for j in range(int(de["ncase"])):
            rete, Rmax, fv, bx, by, bz = de[f"g{k}e{j}_params"]
            bound = halo_properties.escape_velocity_unbinding_fortran(rete, L, nc, grid, fields, dm, c[0], c[1],
                                                                      c[2], bx, by, bz, Rmax, pl, *st, fv, rho_B)
            ref = de[f"g{k}e{j}_bound"]
            assert bound.dtype == ref.dtype and np.array_equal(bound, ref), (k, j)
