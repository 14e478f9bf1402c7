"""ORACLE (test infrastructure only): pyHALMA's substructure block restated on the CPU.

Restates pyHALMA.py:703-766 group by group, exactly as the main script runs it: for sub_LL =
LL/DEC_FACTOR, LL/DEC_FACTOR^2, ... while sub_LL > MIN_LL, centre of mass
(halo_properties.py:26-43) and half-mass radius (halo_properties.py:365-392) of the current
particle list, FoF of the list at sub_LL (fof.py:87-89, here the C oracle's exact partition),
sub-groups with >= MINP_SUB members (pyHALMA.py:148-149), the share cut 0.6 > len/len(list)
> 0.01 and the distance cut |c - c_sub| > DIST_FACTOR * r12 (pyHALMA.py:733-740), removal of
the accepted sub-groups (np.setdiff1d, pyHALMA.py:744-745), emptying below 30 % of the
starting size (pyHALMA.py:751-753), appending the new groups (pyHALMA.py:758-759) and the
final good_groups(MINP) filter (pyHALMA.py:763).
"""
from __future__ import annotations

import numpy as np

from . import fof_labels, labels_to_groups
from .reductions import center_of_mass, half_mass_radius


def identify_substructure(groups, st_x, st_y, st_z, st_mass, LL, MINP_SUB, DEC_FACTOR, MIN_LL, DIST_FACTOR, MINP):
    st_x, st_y, st_z, st_mass = (np.asarray(a, dtype=np.float64) for a in (st_x, st_y, st_z, st_mass))
    counter_sub = 0
    out = [list(g) for g in groups]
    appended = []
    for ihal in range(len(groups)):
        part_list = np.array(groups[ihal], dtype=np.int64)
        starting_npart = len(part_list)
        new_groups = []
        sub_LL = LL / DEC_FACTOR
        while sub_LL > MIN_LL:
            if len(part_list) == 0:
                sub_LL = sub_LL / DEC_FACTOR
                continue
            cx, cy, cz, mass = center_of_mass(part_list, st_x, st_y, st_z, st_mass)
            r12 = half_mass_radius(cx, cy, cz, mass, part_list, st_x, st_y, st_z, st_mass)
            lab = fof_labels(st_x[part_list], st_y[part_list], st_z[part_list], sub_LL)
            sub_groups = [g for g in labels_to_groups(lab) if len(g) >= MINP_SUB]
            for group in sub_groups:
                part_fraction = len(group) / len(part_list)
                if 0.6 > part_fraction > 0.01:
                    cx_sub, cy_sub, cz_sub, _ = center_of_mass(part_list[group], st_x, st_y, st_z, st_mass)
                    dist_sub = np.sqrt((cx - cx_sub) ** 2 + (cy - cy_sub) ** 2 + (cz - cz_sub) ** 2)
                    if dist_sub > DIST_FACTOR * r12:
                        new_groups.append(part_list[group].tolist())
                        counter_sub += 1
            for new_group in new_groups:
                part_list = np.setdiff1d(part_list, new_group)
            sub_LL = sub_LL / DEC_FACTOR
        if starting_npart == 0 or len(part_list) / starting_npart < 0.3:
            out[ihal] = []
        else:
            out[ihal] = part_list.tolist()
        appended.extend(new_groups)
    out.extend(appended)
    return [g for g in out if len(g) >= MINP], counter_sub
