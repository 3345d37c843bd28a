"""GPU parity of the batched many-graph launch (bl_batched_*).

* minibatch graphs (algo 2/3/8): one iteration of every graph against the FP64
  oracle on the same minibatch schedule, re-seeded from the device trajectory:
  its energy within 2e-5 (the force tolerance of the single-graph tests) and
  every vertex's move (a unit step, STEP = 1) along the oracle's force
  direction, relative L2 1e-4 over the graph; the free-running oracle's
  coordinates within 1e-3 (float32 rounding of moved coordinates shifts the
  repulsion of close pairs in later batches);
* Barnes-Hut graphs (algo 4): bit-identical coordinates to the single-graph
  device path (bl_barnes_hut_iteration) after several iterations, and the
  first iteration's energy against the oracle re-seeded from the trajectory;
* a graph's layout does not depend on the other graphs of the launch, a run
  repeats bit for bit, and invalid input is rejected with its error code.
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL = 2e-5


@pytest.fixture(scope="module")
def B():
    import batchlayoutcode_gb300 as B
    B.build()
    return B


def _mix(sizes, seed=3):
    from batchlayoutcode_gb300 import graphs as G
    out = []
    for k, n in enumerate(sizes):
        if k % 3 == 0:
            r = max(2, int(round(np.sqrt(n))))
            g = G.grid_triangulated(r, max(1, int(round(n / r))))
        elif k % 3 == 1:
            g = G.random_geometric(n, 6.0, seed=seed + k)
        else:
            g = G.chung_lu(n, 2.5, 8.0, seed=seed + k)
        xy = G.init_disc(g.n, seed=seed + 17 * k).astype(np.float64)
        out.append((g, xy))
    return out


@pytest.mark.parametrize("algo", [2, 3, 8])
def test_batched_minibatch_one_iteration_matches_oracle(B, algo):
    mix = _mix([150, 333, 700, 1500, 2600, 4100])
    with B.BatchedLayout([(g.rowptr, g.colids) for g, _ in mix], algo, [xy for _, xy in mix]) as bl:
        bl.run(1, 256)
        xs, es = bl.result()
        assert set(bl.parts().tolist()) <= {1, 2, 4}
    for (g, xy0), x, e in zip(mix, xs, es):
        tf, te = oracle.forces_on_trajectory(algo, g.rowptr, g.colids, xy0, x, 256)
        assert abs(e - te) / te <= TOL, (g.name, e, te)
        unit = tf / np.linalg.norm(tf, axis=1, keepdims=True)
        move = x - xy0
        assert np.linalg.norm(move - unit) / np.linalg.norm(unit) <= 1e-4, g.name
        oxy, _, oe = oracle.smu_iteration(algo, g.rowptr, g.colids, xy0, 256, 1.0, 1.0)
        assert np.abs(x - oxy).max() <= 1e-3, g.name


@pytest.mark.parametrize("parts", [1, 2, 4])
def test_batched_every_source_split_matches_oracle(B, parts):
    mix = _mix([300, 1200, 3000], seed=11)
    with B.BatchedLayout([(g.rowptr, g.colids) for g, _ in mix], 2, [xy for _, xy in mix]) as bl:
        bl.set_parts([parts] * 3)
        bl.run(1, 256)
        xs, es = bl.result()
        assert bl.parts().tolist() == [parts] * 3
    for (g, xy0), x, e in zip(mix, xs, es):
        _, te = oracle.forces_on_trajectory(2, g.rowptr, g.colids, xy0, x, 256)
        assert abs(e - te) / te <= TOL, (g.name, parts)


def test_batched_bh_bit_identical_to_single_graph_path(B):
    mix = _mix([5200, 6100, 7000], seed=5)
    iters = 3
    with B.BatchedLayout([(g.rowptr, g.colids) for g, _ in mix], 4, [xy for _, xy in mix]) as bl:
        bl.run(iters, 256, 1.2)
        xs, es = bl.result()
    for (g, xy0), x, e in zip(mix, xs, es):
        with B.Algorithms(g.rowptr, g.colids) as a:
            a.nCoordinates = xy0
            step = 1.0
            for _ in range(iters):
                e1 = a.barnes_hut_iteration(256, 1.2, step)
                step *= 0.999
            xy1 = a.nCoordinates
        assert np.array_equal(x, xy1), g.name
        assert abs(e - e1) <= 1e-12 * e1, (g.name, e, e1)


def test_batched_bh_first_iteration_against_oracle(B):
    mix = _mix([5100, 5600], seed=9)
    with B.BatchedLayout([(g.rowptr, g.colids) for g, _ in mix], 4, [xy for _, xy in mix]) as bl:
        bl.run(1, 256, 1.2)
        xs, es = bl.result()
    for (g, xy0), x, e in zip(mix, xs, es):
        _, te = oracle.forces_on_trajectory(4, g.rowptr, g.colids, xy0, x, 256, theta=1.2)
        assert abs(e - te) / te <= TOL, (g.name, e, te)


def test_batched_mixed_independent_and_repeatable(B):
    mix = _mix([180, 5300, 900, 2100, 5050, 400, 3300], seed=21)
    algo = [2 if g.n < 5000 else 4 for g, _ in mix]
    graphs = [(g.rowptr, g.colids) for g, _ in mix]
    xys = [xy for _, xy in mix]
    with B.BatchedLayout(graphs, algo, xys) as bl:
        bl.set_parts([2, 2, 2])
        bl.run(4, 256, 1.2)
        xs1, es1 = bl.result()
        bl.run(4, 256, 1.2)  # replay of the captured launch
        xs2, es2 = bl.result()
    for a, b in zip(xs1, xs2):
        assert np.array_equal(a, b)
    assert np.array_equal(es1, es2)
    sub = [5, 1, 3]  # other neighbours, other queue positions
    with B.BatchedLayout([graphs[k] for k in sub], [algo[k] for k in sub], [xys[k] for k in sub]) as bl:
        bl.set_parts([2, 2, 2])
        bl.run(4, 256, 1.2)
        xs3, es3 = bl.result()
    for j, k in enumerate(sub):
        assert np.array_equal(xs3[j], xs1[k])
        assert es3[j] == es1[k]


def test_batched_input_errors(B):
    from batchlayoutcode_gb300._lib import BatchLayoutError
    g, xy = _mix([200])[0]
    with pytest.raises(BatchLayoutError) as ei:
        B.BatchedLayout([(g.rowptr, g.colids)], 5, [xy])
    assert ei.value.code == -4
    bad = g.colids.copy()
    bad[0] = g.n
    with pytest.raises(BatchLayoutError) as ei:
        B.BatchedLayout([(g.rowptr, bad)], 2, [xy])
    assert ei.value.code == -1
    with B.BatchedLayout([(g.rowptr, g.colids)], 2, [xy]) as bl:
        with pytest.raises(BatchLayoutError) as ei:
            bl.run(0, 256)
        assert ei.value.code == -1
