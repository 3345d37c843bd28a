"""GPU breadth-first greedy start (bl_bfs_init) against its FP64 oracle
(oracle/bfs_init.py): positions within 1e-5 (FP32 output of FP64 sums that
the device adds by pointer jumping and the oracle level by level), and its
properties on the 1M-vertex benchmark graph."""
import time

import numpy as np
import pytest

from oracle import bfs_init as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def B():
    import batchlayoutcode_gb300 as B
    B.build()
    return B


def _graphs():
    from batchlayoutcode_gb300 import graphs as G
    return [G.grid_triangulated(40, 50), G.random_geometric(20000, 6.0, seed=2), G.chung_lu(8000, 2.5, 8.0, seed=3)]


@pytest.mark.parametrize("k", [0, 1, 2])
def test_bfs_init_matches_oracle(B, k):
    g = _graphs()[k]
    with B.Algorithms(g.rowptr, g.colids) as a:
        a.bfsInit()
        xy = a.nCoordinates
    exp = O.bfs_init(g.rowptr, g.colids)
    assert np.abs(xy - exp).max() <= 1e-5
    level, _ = O.bfs_tree(g.rowptr, g.colids)
    assert np.all(xy[level < 0] == 0.0)


def test_bfs_init_disconnected_and_repeatable(B):
    from batchlayoutcode_gb300 import graphs as G
    g = G.grid_triangulated(10, 10)
    # a second component (ids 100..103) that vertex 0 does not reach
    rp = list(g.rowptr)
    ci = list(g.colids)
    extra = {100: [101], 101: [100, 102], 102: [101, 103], 103: [102]}
    for v in range(100, 104):
        ci += extra[v]
        rp.append(len(ci))
    rp, ci = np.array(rp, np.int32), np.array(ci, np.int32)
    with B.Algorithms(rp, ci) as a:
        a.bfsInit()
        x1 = a.nCoordinates
        a.bfsInit()
        x2 = a.nCoordinates
    assert np.array_equal(x1, x2)
    assert np.all(x1[100:] == 0.0)
    assert np.abs(x1 - O.bfs_init(rp, ci)).max() <= 1e-5


def test_bfs_init_rgg1m(B):
    from batchlayoutcode_gb300 import graphs as G
    g, _ = G.cached_workload("rgg1m")
    with B.Algorithms(g.rowptr, g.colids) as a:
        a.bfsInit()  # first call: allocation and warm-up
        t0 = time.perf_counter()
        a.bfsInit()
        dt = time.perf_counter() - t0
        xy = a.nCoordinates
    span = max(np.ptp(xy[:, 0]), np.ptp(xy[:, 1]))
    assert abs(span - 6.0) <= 1e-4
    assert np.all(np.isfinite(xy))
    print(f"bfs init 1M: {dt * 1e3:.1f} ms")
    assert dt < 0.25  # the host initDFS takes ~0.25 s on this graph
