"""ORACLE (test infrastructure / CPU baseline only): the reference's KDTree flood fill.

Restates python_scripts/fof.py:18-79 (``friends_of_friends``) operation for operation, so that
its CPU time stands for the reference's own where the reference cannot be imported (the GPU
host has no copy of it):

* one ``scipy.spatial.KDTree`` over the (N, 3) positions (fof.py:20);
* seeds in index order, skipping particles already looked at (fof.py:34-37);
* a seed whose ball holds only itself is skipped (fof.py:40-44);
* the queue is a Python list consumed with ``pop(0)`` (fof.py:53-55); every visited particle
  queries its ball, drops entries already looked at and entries already marked as friends by
  two list comprehensions, and appends the rest to the queue and to the group
  (fof.py:58-67);
* every 64 visits the queue's entries are marked as friends (fof.py:70-72);
* each finished group is ``np.unique`` of everything appended, as a list (fof.py:76).

``friends_of_friends_serial`` restates fof.py:87-89 (pack three 1-D arrays into (N,3)).
The output equals the reference's on every golden case (tests/test_oracle.py).
"""
from __future__ import annotations

import numpy as np
from scipy.spatial import KDTree

CLEAN_EVERY = 64   # fof.py:33 iterations_to_clean


def friends_of_friends(data, linking_length, boxsize=None):
    """fof.py:18-79; ``boxsize`` (None in the reference) gives the tree a periodic box."""
    data = np.asarray(data)
    tree = KDTree(data) if boxsize is None else KDTree(data, boxsize=boxsize)
    n = data.shape[0]
    looked = np.zeros(n, dtype=bool)
    marked = np.zeros(n, dtype=bool)
    groups = []
    for seed in range(n):
        if looked[seed]:
            continue
        queue = tree.query_ball_point(data[seed], linking_length)
        if len(queue) <= 1:
            continue
        found = queue.copy()
        looked[seed] = True
        marked[queue] = True
        visits = 0
        while len(queue) > 0:
            p = queue.pop(0)
            if looked[p]:
                continue
            fresh = tree.query_ball_point(data[p], linking_length)
            fresh = [q for q in fresh if not looked[q]]
            fresh = [q for q in fresh if not marked[q]]
            queue += fresh
            found += fresh
            looked[p] = True
            if visits % CLEAN_EVERY == 0 and visits != 0:
                marked[queue] = True
            visits += 1
        groups.append(np.unique(np.array(found)).tolist())
    return groups


def friends_of_friends_serial(st_x, st_y, st_z, linking_length, boxsize=None):
    data = np.array((st_x, st_y, st_z)).T
    return friends_of_friends(data, linking_length, boxsize)
