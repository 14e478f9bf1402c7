"""ORACLE (test infrastructure / CPU baseline only): the reference's KDTree flood fill.

Restates python_scripts/fof.py:18-79 (``friends_of_friends``): a breadth-first flood fill
that calls ``scipy.spatial.KDTree.query_ball_point(point, linking_length)`` once per
particle it visits.  Seeds are taken in index order (fof.py:34), a seed whose ball holds
only itself is skipped (fof.py:43-44), and each finished group is returned as a sorted
list of ints (fof.py:76).  The reference's periodic ``already_friend`` bookkeeping
(fof.py:48, 62-72) only prunes duplicate queue entries; here a single ``queued`` mask does
that job, which leaves the set of visited particles, and so the output, unchanged.

``friends_of_friends_serial`` restates fof.py:87-89 (pack three 1-D arrays into (N,3)).
This is the algorithm the CPU baseline times: one Python-level KDTree query per particle.
"""
from __future__ import annotations

import numpy as np
from scipy.spatial import KDTree


def friends_of_friends(data, linking_length):
    data = np.asarray(data)
    tree = KDTree(data)
    n = data.shape[0]
    queued = np.zeros(n, dtype=bool)
    out = []
    for seed in range(n):
        if queued[seed]:
            continue
        first = tree.query_ball_point(data[seed], linking_length)
        if len(first) <= 1:
            continue
        members = list(first)
        queued[first] = True
        head = 0
        while head < len(members):
            p = members[head]
            head += 1
            if p == seed:
                continue
            nb = tree.query_ball_point(data[p], linking_length)
            fresh = [q for q in nb if not queued[q]]
            if fresh:
                queued[fresh] = True
                members.extend(fresh)
        out.append(sorted(set(int(i) for i in members)))
    return out


def friends_of_friends_serial(st_x, st_y, st_z, linking_length):
    data = np.array((st_x, st_y, st_z)).T
    return friends_of_friends(data, linking_length)
