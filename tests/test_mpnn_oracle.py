"""The network's CPU oracle (oracle/mpnn.py) against finite differences, and
its BF16 rounding against the definition (CPU only)."""
import numpy as np

from oracle import mpnn as M


def _graph(n=30, seed=0):
    rng = np.random.default_rng(seed)
    edges = set()
    for v in range(n):
        for _ in range(3):
            u = int(rng.integers(0, n))
            if u != v:
                edges.add((min(u, v), max(u, v)))
    rows = [[] for _ in range(n)]
    for a, b in edges:
        rows[a].append(b)
        rows[b].append(a)
    rowptr = np.zeros(n + 1, np.int64)
    rowptr[1:] = np.cumsum([len(r) for r in rows])
    colids = np.array([c for r in rows for c in sorted(r)], np.int64)
    return rowptr, colids


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -2.5, 3.0e38, 1e-40], np.float32)
    r = M.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: ties go to the even mantissa (1.0)
    assert r[1] == np.float32(1.0)
    assert r[2] == np.float32(1.0078125)
    assert r[0] == 1.0 and r[3] == np.float32(1.0078125) and r[4] == -2.5
    bits = r.view(np.uint32)
    assert np.all(bits & 0xFFFF == 0)


def test_backward_matches_finite_differences():
    rowptr, colids = _graph()
    n = rowptr.shape[0] - 1
    rng = np.random.default_rng(1)
    feats = rng.normal(size=(n, M.FEATURES))
    target = rng.normal(size=(n, 2))
    w = np.full(n, 1.0 / n)
    p = M.init_params(3).astype(np.float64)
    p[M.NPARAMS - 130:] += rng.normal(0, 0.1, 130)
    loss, g, _ = M.loss_and_grad(p, rowptr, colids, feats, target, w, mimic=False)
    idx = rng.choice(M.NPARAMS, 60, replace=False)
    eps = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        lp = M.loss_and_grad(pp, rowptr, colids, feats, target, w, mimic=False)[0]
        lm = M.loss_and_grad(pm, rowptr, colids, feats, target, w, mimic=False)[0]
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-8, (i, fd, g[i])


def test_mimic_forward_close_to_fp64():
    rowptr, colids = _graph(50, 2)
    n = rowptr.shape[0] - 1
    rng = np.random.default_rng(4)
    feats = rng.normal(size=(n, M.FEATURES))
    p = M.init_params(5)
    a = M.forward(p, rowptr, colids, feats, mimic=True)["xy"]
    b = M.forward(p, rowptr, colids, feats, mimic=False)["xy"]
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < 3e-2

