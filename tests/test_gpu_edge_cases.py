"""Edge cases of the single-graph paths against the FP64 oracle: one, two and
three vertices, isolated vertices (degree 0) among connected ones, coincident
points (neighbours and non-neighbours at the same position), batch 1 (pure
Gauss-Seidel), a batch larger than the graph (one Jacobi batch), zero
iterations, and arguments the library rejects.

Each case runs one iteration of a method on the device and compares its
forces and energy with the oracle re-seeded from the device trajectory
(oracle.forces_on_trajectory), within the tolerances of the other parity
tests (forces relative L2 1e-5, energy 2e-5; absolute where they are zero).
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5


def csr(n, edges):
    adj = [set() for _ in range(n)]
    for u, v in edges:
        if u != v:
            adj[u].add(v)
            adj[v].add(u)
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum([len(a) for a in adj])
    ci = np.array([v for a in adj for v in sorted(a)], np.int32)
    return rp, ci


def case_graphs():
    from batchlayoutcode_gb300 import graphs as G
    rng = np.random.default_rng(21)
    cases = {}
    cases["single"] = (*csr(1, []), np.array([[0.5, -0.25]]))
    cases["pair"] = (*csr(2, [(0, 1)]), rng.uniform(-3, 3, (2, 2)))
    cases["path3"] = (*csr(3, [(0, 1), (1, 2)]), rng.uniform(-3, 3, (3, 2)))
    # a random geometric graph with 20 isolated vertices spread among its ids
    g = G.random_geometric(300, 6.0, seed=3)
    n = g.n + 20
    iso = np.sort(rng.choice(n, 20, replace=False))
    keep = np.setdiff1d(np.arange(n), iso)  # new id of old vertex k: keep[k]
    rows = np.repeat(np.arange(g.n), np.diff(g.rowptr))
    cases["isolated"] = (*csr(n, zip(keep[rows], keep[g.colids])), rng.uniform(-3, 3, (n, 2)))
    # an 8 x 8 grid with coincident vertices: 5 and 17 (not adjacent), 9 and 10 (adjacent)
    edges = [(r * 8 + c, r * 8 + c + 1) for r in range(8) for c in range(7)]
    edges += [(r * 8 + c, (r + 1) * 8 + c) for r in range(7) for c in range(8)]
    xy = rng.uniform(-3, 3, (64, 2))
    xy[17] = xy[5]
    xy[10] = xy[9]
    cases["coincident"] = (*csr(64, edges), xy)
    return cases


CASES = case_graphs()


@pytest.fixture(scope="module")
def B():
    import batchlayoutcode_gb300 as B
    B.build()
    return B


def check(f, e, tf, te):
    nf = np.linalg.norm(tf)
    if nf > 0:
        assert np.linalg.norm(f - tf) <= FORCE_TOL * nf
    else:
        assert np.abs(f).max() == 0.0
    if te > 0:
        assert abs(e - te) <= 2 * FORCE_TOL * te
    else:
        assert e == 0.0


def run_one(B, name, algo, batch):
    rp, ci, xy0 = CASES[name]
    with B.Algorithms(rp, ci) as a:
        a.nCoordinates = xy0
        xy = a.nCoordinates  # the FP32 start the device works from
        if algo == 4:
            e = a.barnes_hut_iteration(batch, 1.2, 1.0)
        elif algo == 5:  # greedy approximation, first phase
            e = a.greedy_iteration(batch, 1.0)
        elif algo == 50:  # greedy approximation, second phase
            e = a.minibatch_iteration(5, batch, 1.0)
        else:
            e = a.minibatch_iteration(algo, batch, 1.0)
        f = a.prevCoordinates
        out = a.nCoordinates
    tf, te = oracle.forces_on_trajectory(algo, rp, ci, xy, out, batch)
    check(f, e, tf, te)
    return xy, out, f


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("algo", [2, 3, 8])
@pytest.mark.parametrize("batch", [1, 7, 4096])
def test_minibatch_edge_cases(B, name, algo, batch):
    run_one(B, name, algo, batch)


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("batch", [1, 256])
def test_barnes_hut_edge_cases(B, name, batch):
    run_one(B, name, 4, batch)


@pytest.mark.parametrize("name", [k for k in CASES if k != "single"])
@pytest.mark.parametrize("algo", [7, 5, 50])
def test_sd_and_greedy_edge_cases(B, name, algo):
    run_one(B, name, algo, 7)


@pytest.mark.parametrize("algo", [2, 4])
def test_single_vertex_stays(B, algo):
    """A lone vertex has no force: the update is skipped (the reference's unit
    vector of a zero force is NaN) and the vertex stays where it is."""
    xy, out, f = run_one(B, "single", algo, 1)
    assert np.array_equal(out, xy)
    assert np.all(f == 0.0)


def test_isolated_vertices_move_by_repulsion_only(B):
    """Degree-0 vertices get repulsion and no attraction; they move by STEP
    along it like the others."""
    rp, ci, _ = CASES["isolated"]
    xy, out, f = run_one(B, "isolated", 2, 7)
    iso = np.nonzero(np.diff(rp) == 0)[0]
    assert len(iso) == 20
    step = np.linalg.norm(out[iso] - xy[iso], axis=1)
    assert np.allclose(step, 1.0, atol=1e-5)


@pytest.mark.parametrize("algo", [2, 4])
def test_zero_iterations_change_nothing(B, algo):
    rp, ci, xy0 = CASES["isolated"]
    with B.Algorithms(rp, ci) as a:
        a.nCoordinates = xy0
        xy = a.nCoordinates
        e = a.run_resident(algo, 0, 32, 1.2, 1.0)
        assert np.array_equal(a.nCoordinates, xy)
    assert e == 0.0


def test_rejected_arguments(B):
    rp, ci, xy0 = CASES["path3"]
    with B.Algorithms(rp, ci) as a:
        a.nCoordinates = xy0
        with pytest.raises(RuntimeError):
            a.minibatch_iteration(2, 0, 1.0)  # batch must be >= 1
        with pytest.raises(RuntimeError):
            a.barnes_hut_iteration(0, 1.2, 1.0)
        with pytest.raises(RuntimeError):
            a.minibatch_iteration(1, 32, 1.0)  # algo 1 is not on this path
        # the context is still usable after the rejected calls
        assert np.isfinite(a.minibatch_iteration(2, 2, 1.0))
