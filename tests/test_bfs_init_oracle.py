"""The breadth-first start's CPU oracle (oracle/bfs_init.py) against scipy's
BFS and its own definition (CPU only)."""
import numpy as np


def test_bfs_init_oracle_tree():
    """The breadth-first start's oracle: levels are BFS distances from vertex
    0 (scipy), every parent is the smallest-id neighbour one level up, and
    the layout spans 2 * MAXMIN."""
    from scipy.sparse import csr_matrix
    from scipy.sparse.csgraph import shortest_path
    from batchlayoutcode_gb300 import graphs as G
    from oracle import bfs_init as O
    g = G.chung_lu(3000, 2.5, 8.0, seed=7)
    level, parent = O.bfs_tree(g.rowptr, g.colids)
    A = csr_matrix((np.ones(g.colids.size), g.colids, g.rowptr), shape=(g.n, g.n))
    d = shortest_path(A, unweighted=True, indices=[0])[0]
    assert np.array_equal(np.where(np.isinf(d), -1, d).astype(np.int64), level)
    for v in range(1, g.n):
        if level[v] < 0:
            continue
        nb = g.colids[g.rowptr[v]:g.rowptr[v + 1]]
        assert parent[v] == nb[level[nb] == level[v] - 1].min()
    xy = O.bfs_init(g.rowptr, g.colids)
    reached = level >= 0
    assert abs(max(np.ptp(xy[reached, 0]), np.ptp(xy[reached, 1])) - 6.0) < 1e-12
