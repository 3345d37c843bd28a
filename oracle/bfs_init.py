"""CPU restatement of the breadth-first greedy start (numpy, FP64).

TEST INFRASTRUCTURE ONLY: imported by tests/.  The start has no reference
counterpart (it applies initDFS's placement rule, sample/algorithms.cpp:29-97,
on a breadth-first tree); this file is its oracle and follows
batchlayoutcode_gb300/csrc/bfsinit.cu step by step:

* a level-synchronous BFS from vertex 0; a vertex's parent is the smallest-id
  vertex of the previous level adjacent to it;
* a child's rank k among its parent's children by first occurrence in the
  parent's CSR row; offset (0.1 cos a + r, 0.1 sin a + r), a = pi (k * 360 /
  deg(parent)) / 180, r = splitmix64(id) >> 40 over 2^24; the root at (1, 1);
* positions: offsets summed from the root, level by level;
* scale 2 * 3 / max(x range, y range) over the reached vertices; unreached
  vertices at the origin.
"""
from __future__ import annotations

import numpy as np

MASK = (1 << 64) - 1


def hash_unit(ids: np.ndarray) -> np.ndarray:
    x = ids.astype(np.uint64)
    with np.errstate(over="ignore"):
        x = x + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        x = x ^ (x >> np.uint64(31))
    return (x >> np.uint64(40)).astype(np.float64) / 16777216.0


def bfs_tree(rowptr, colids):
    """-> (level (-1 unreached), parent (-1 for the root and unreached))."""
    rowptr = np.asarray(rowptr, np.int64)
    colids = np.asarray(colids, np.int64)
    n = rowptr.shape[0] - 1
    level = np.full(n, -1, np.int64)
    parent = np.full(n, -1, np.int64)
    level[0] = 0
    frontier = np.array([0], np.int64)
    L = 0
    while frontier.size:
        L += 1
        deg = rowptr[frontier + 1] - rowptr[frontier]
        src = np.repeat(frontier, deg)
        starts = np.repeat(rowptr[frontier], deg)
        idx = starts + (np.arange(src.size) - np.repeat(np.cumsum(deg) - deg, deg))
        dst = colids[idx]
        new = level[dst] == -1
        src, dst = src[new], dst[new]
        if dst.size == 0:
            break
        best = np.full(n, np.iinfo(np.int64).max, np.int64)
        np.minimum.at(best, dst, src)
        nxt = np.unique(dst)
        level[nxt] = L
        parent[nxt] = best[nxt]
        frontier = nxt
    return level, parent


def bfs_init(rowptr, colids) -> np.ndarray:
    rowptr = np.asarray(rowptr, np.int64)
    colids = np.asarray(colids, np.int64)
    n = rowptr.shape[0] - 1
    level, parent = bfs_tree(rowptr, colids)
    # first occurrence of each child in its parent's row
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    e = np.arange(colids.size)
    is_child = parent[colids] == rows
    firstpos = np.full(n, np.iinfo(np.int64).max, np.int64)
    np.minimum.at(firstpos, colids[is_child], e[is_child])
    kids = np.nonzero(parent >= 0)[0]
    order = np.lexsort((firstpos[kids], parent[kids]))
    kids = kids[order]
    par = parent[kids]
    group_start = np.r_[0, np.nonzero(np.diff(par))[0] + 1]
    rank = np.arange(kids.size) - np.repeat(group_start, np.diff(np.r_[group_start, kids.size]))
    off = np.zeros((n, 2))
    off[0] = (1.0, 1.0)
    deg = np.maximum(np.diff(rowptr), 1).astype(np.float64)
    step = 360.0 / deg[par]
    ang = np.pi * (rank * step) / 180.0
    r = hash_unit(kids)
    off[kids, 0] = 0.1 * np.cos(ang) + r
    off[kids, 1] = 0.1 * np.sin(ang) + r
    xy = off.copy()
    maxl = level.max()
    for L in range(1, maxl + 1):
        at = np.nonzero(level == L)[0]
        xy[at] = off[at] + xy[parent[at]]
    reached = level >= 0
    span = max(np.ptp(xy[reached, 0]), np.ptp(xy[reached, 1]))
    scale = 2.0 * 3.0 / span if span > 0 else 1.0
    return xy * scale
