"""The FP64 oracle against golden vectors produced by the reference itself
(tests/golden/make_golden.py: the reference's own routines, strict FP64 build).

Every comparison is exact: the oracle follows the reference's operation order.
"""
import numpy as np
import pytest

import oracle
from conftest import GOLDEN_GRAPHS, load_golden


@pytest.fixture(scope="module", params=GOLDEN_GRAPHS)
def gold(request):
    return request.param, load_golden(request.param)


@pytest.mark.parametrize("algo,iters", [(a, i) for a in (2, 3, 4, 5, 6, 7, 8) for i in (1, 4)] + [(5, 6)])
def test_layout_bit_exact(gold, algo, iters):
    _, z = gold
    out, e, loops, f = oracle.layout(algo, z["csr_rowptr"], z["csr_colids"], z["init_xy"], iters, 32,
                                     want_forces=True, nthreads=1)
    assert np.array_equal(out, z[f"L{algo}_i{iters}_xy"])
    assert np.array_equal(f, z[f"L{algo}_i{iters}_f"])
    assert e == float(z[f"L{algo}_i{iters}_e"])


def test_layout_threads_do_not_change_result(gold):
    _, z = gold
    a = oracle.layout(2, z["csr_rowptr"], z["csr_colids"], z["init_xy"], 4, 32, nthreads=1)
    b = oracle.layout(2, z["csr_rowptr"], z["csr_colids"], z["init_xy"], 4, 32, nthreads=4)
    assert np.array_equal(a[0], b[0]) and a[1] == b[1]


def test_converged_bit_exact(gold):
    _, z = gold
    out, e, loops = oracle.layout(2, z["csr_rowptr"], z["csr_colids"], z["init_xy"], 600, 32, engt=0.05,
                                  nthreads=1)
    assert loops == int(z["conv_loops"])
    assert e == float(z["conv_e"])
    assert np.array_equal(out, z["conv_xy"])


def test_morton_sort_matches_reference(gold):
    _, z = gold
    xy = z["init_xy"]
    _, keys, perm = oracle.morton_sort(xy)
    assert np.array_equal(xy[perm], z["bh_sorted"])
    assert np.all(np.diff(keys.astype(np.float64)) >= 0)


def test_tree_matches_reference(gold):
    _, z = gold
    t = oracle.bh_tree(z["init_xy"])
    for k in ("lo", "hi", "depth", "nchild"):
        assert np.array_equal(t[k], z["tree_" + k]), k
    assert np.array_equal(t["centroid"], z["tree_centroid"])


@pytest.mark.parametrize("theta", [1.2, 0.5])
def test_bh_repulsion_matches_reference(gold, theta):
    _, z = gold
    xy = z["init_xy"]
    r = oracle.bh_repulsion(xy, xy, theta, nthreads=2)
    assert np.array_equal(r, z[f"bh_rep_t{theta}"])


def test_greedy_walks_follow_the_reference_rules(gold):
    """Algo 5's walk sources (algorithms.cpp:1126-1170): never i or a
    neighbour of i, at least 200 pushes unless the stack ran dry, and the
    overshoot past 200 is bounded by one row."""
    _, z = gold
    rp, ci = z["csr_rowptr"], z["csr_colids"]
    off, src = oracle.greedy_walks(rp, ci)
    deg = np.diff(rp)
    n = rp.shape[0] - 1
    for i in range(n):
        w = src[off[i]:off[i + 1]]
        excl = set(ci[rp[i]:rp[i + 1]].tolist()) | {i}
        assert not (set(w.tolist()) & excl)
        assert len(w) < 200 + deg.max()
        if len(w) < 200:  # only when the walk ran out of vertices
            reach = set()
            for v in w:
                reach |= set(ci[rp[v]:rp[v + 1]].tolist())
            assert reach - excl <= set(w.tolist())


def test_grid64_600_iterations_energy_bit_exact():
    """The 4,096-vertex triangulated grid workload (algo 2, batch 256, 600
    iterations from the seeded disc start): the oracle's final energy equals
    the reference's own (strict build) bit for bit, and the reader's CSR
    checksum matches the generator's graph."""
    import os
    from batchlayoutcode_gb300 import graphs as G
    from conftest import GOLDEN
    z = np.load(os.path.join(GOLDEN, "ref_grid64_cfg1.npz"))
    g, xy = G.workload("grid64")
    assert np.array_equal(np.asarray(xy, np.float64), z["init_xy"])
    assert z["csr_sum"].tolist() == [g.n, g.nnz, int(np.sum(g.colids, dtype=np.int64))]
    _, e, _ = oracle.layout(2, g.rowptr, g.colids, z["init_xy"], int(z["iterations"]), int(z["batch"]))
    assert e == float(z["energy"])


def _canonical_walk_visits(xy, theta):
    """Records read by a pre-order walk of the canonical tree (oracle.bh_tree:
    nodes with two or more children, and the leaf points) that opens a node
    when D / dist >= theta, D = MAXMIN 2^-depth (BarnesHut.h:71-72): what the
    device's stackless walk reads for the same decisions."""
    import math
    import sys
    sys.setrecursionlimit(10000)
    frame, _, perm = oracle.morton_sort(xy)
    t = oracle.bh_tree(xy)
    lo, hi, dep, cen = t["lo"], t["hi"], t["depth"], t["centroid"]
    kids = [[] for _ in range(len(lo))]
    stack = []
    for k in range(len(lo)):
        while stack and not (lo[k] >= lo[stack[-1]] and hi[k] <= hi[stack[-1]]):
            stack.pop()
        if stack:
            kids[stack[-1]].append(k)
        stack.append(k)
    total = 0
    for q in xy:
        count = [0]

        def visit(k):
            count[0] += 1
            dx, dy = cen[k][0] - q[0], cen[k][1] - q[1]
            dist = math.sqrt(dx * dx + dy * dy)
            if dist > 0 and math.ldexp(frame[2], -int(dep[k])) / dist < theta:
                return
            p, c = lo[k], 0
            while p < hi[k]:
                if c < len(kids[k]) and lo[kids[k][c]] == p:
                    visit(kids[k][c])
                    p = hi[kids[k][c]]
                    c += 1
                else:
                    count[0] += 1
                    p += 1
        visit(0)
        total += count[0]
    return total


@pytest.mark.parametrize("theta", [1.2, 0.5])
def test_bh_visit_count_is_the_canonical_walk(gold, theta):
    """The oracle's per-query visit counts (its recursion over the reference
    quadtree, a single-child chain counted once) add up to the records a walk
    of the canonical tree reads: the figure the device's walk is held to."""
    _, z = gold
    xy = z["init_xy"]
    _, vis = oracle.bh_repulsion(xy, xy, theta, visits=True)
    assert int(vis.sum()) == _canonical_walk_visits(xy, theta)
