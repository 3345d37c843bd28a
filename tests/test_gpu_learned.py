"""The learned initializer end to end on the GPU: training lowers the loss,
the shipped model's start reaches the plain run's final energy within a few
Barnes-Hut iterations (the plain run needs all 600), the network beats the
same pipeline without it (zero network output: the pivot-MDS shape) both in
its first iteration and in the iterations it needs to reach that pipeline's
best energy, the plain run is the fallback, and the CLI accepts -learned."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def B():
    import batchlayoutcode_gb300 as B
    B.build()
    return B


def test_training_lowers_loss(B):
    from batchlayoutcode_gb300 import learned as LR
    gs = LR.training_graphs(6, 500, 3000, seed=77)
    lays = LR.target_layouts(gs, 100)
    params, sm, hist = LR.train(gs, lays, 300, 3e-3)
    assert np.all(np.isfinite(hist)) and np.all(np.isfinite(params))
    assert hist[-1] < 0.3 * hist[0], (hist[0], hist[-1])


@pytest.fixture(scope="module")
def rgg():
    from batchlayoutcode_gb300 import graphs as G
    return G.random_geometric(100_000, 6.0, seed=99)


def test_learned_start_reaches_plain_energy(B, rgg):
    from batchlayoutcode_gb300 import learned as LR
    params, sm = LR.load_model()
    with B.Algorithms(rgg.rowptr, rgg.colids, init=0) as a:
        e_plain, _ = a.BarnesHutApproximation(600, 0, 256, 1.2, 0)
    with B.Algorithms(rgg.rowptr, rgg.colids, init=0) as a:
        r = a.learnedLayout(params, sm, 600, e_plain * 1.005)
    assert not r["fell_back"]
    assert r["iterations"] <= 10 and r["energy"] <= e_plain * 1.005


def test_network_gains_over_mds_shape(B, rgg):
    from batchlayoutcode_gb300 import learned as LR
    params, sm = LR.load_model()
    e = {}
    for name, p in (("learned", params), ("mds", np.zeros_like(params))):
        with B.Algorithms(rgg.rowptr, rgg.colids, init=0) as a:
            a.learnedInit(p, sm)
            e[name] = a.barnes_hut_iteration(256, 1.2, LR.STEP0)
    assert e["learned"] < 0.95 * e["mds"], e


@pytest.mark.parametrize("name", ["rgg1m", "grid300"])
def test_network_reaches_the_zero_networks_best_energy_in_fewer_iterations(B, name):
    """On held-out graphs -- the 1M-vertex benchmark graph and a 300 x 300
    triangulated grid -- the lowest energy the pipeline without the network
    (the pivot-MDS shape) reaches in its first 100 refinement iterations is
    reached from the network's start in at most a quarter as many iterations
    (measured: 1 against 42 and 1 against 56).  The energy, sum |f|^2 of an
    iteration, is not monotone in the iterations (it settles at a level the
    step size sets), so the target is the zero network's best, not its last.
    On 100k-vertex random geometric graphs the gain depends on the graph (6
    against 43 iterations on one seed, the target missed within 100 on
    another) and on Chung-Lu graphs there is none."""
    from batchlayoutcode_gb300 import graphs as G
    from batchlayoutcode_gb300 import learned as LR
    g = G.cached_workload("rgg1m")[0] if name == "rgg1m" else G.grid_triangulated(300, 300)
    params, sm = LR.load_model()
    with B.Algorithms(g.rowptr, g.colids, init=0) as a:
        a.learnedInit(np.zeros_like(params), sm)
        es, step = [], LR.STEP0
        for _ in range(100):
            es.append(a.barnes_hut_iteration(256, 1.2, step))
            step *= 0.999
    floor = min(es) * 1.005
    zero_its = int(np.argmax(np.array(es) <= floor)) + 1
    with B.Algorithms(g.rowptr, g.colids, init=0) as a:
        r = a.learnedLayout(params, sm, 100, floor)
    assert not r["fell_back"] and r["energy"] <= floor
    assert 4 * r["iterations"] <= zero_its, (r["iterations"], zero_its, es)


def test_fallback_is_the_plain_run(B):
    from batchlayoutcode_gb300 import graphs as G
    from batchlayoutcode_gb300 import learned as LR
    g = G.grid_triangulated(30, 30)
    params, sm = LR.load_model()
    with B.Algorithms(g.rowptr, g.colids, init=0) as a:
        e_plain, _ = a.BarnesHutApproximation(20, 0, 256, 1.2, 0)
        xy_plain = a.nCoordinates
    with B.Algorithms(g.rowptr, g.colids, init=0) as a:
        r = a.learnedLayout(params, sm, 20, 0.0)
        xy = a.nCoordinates
    assert r["fell_back"]
    assert r["energy"] == e_plain
    assert np.array_equal(xy, xy_plain)


def test_cli_learned_init(B, tmp_path):
    from batchlayoutcode_gb300 import graphs as G
    from batchlayoutcode_gb300 import learned as LR
    from batchlayoutcode_gb300.build import CLI
    g = G.grid_triangulated(20, 25)
    mtx = str(tmp_path / "g.mtx")
    G.write_mtx(g, mtx)
    out = subprocess.run([CLI, "-input", mtx, "-output", str(tmp_path) + "/", "-algo", "4", "-iter", "5",
                          "-learned", LR.DEFAULT_MODEL], capture_output=True, text=True, cwd=tmp_path, timeout=300)
    assert out.returncode == 0, out.stderr
    assert os.path.exists(str(tmp_path / "g.mtxBHMINB256PARAOUT5.txt")) or \
        any(f.endswith("PARAOUT5.txt") for f in os.listdir(tmp_path))
    assert "LEARNED" in open(tmp_path / "Results.txt").read()
