"""CPU restatement of the learned initializer's network (FP64 numpy).

TEST INFRASTRUCTURE ONLY: imported by tests/ (and nothing in the package).
The network has no counterpart in the reference; this file is its oracle.

forward()/backward() follow batchlayoutcode_gb300/csrc/mpnn.cu operation by
operation.  With ``mimic=True`` every value the device rounds to BF16 (the
features, the weights, each layer's activations and neighbour means, the
backward operands dz) is rounded the same way, and the neighbour sums run in
FP32 in CSR order like the device; the matrix products themselves are FP64,
so the device differs only by its FP32 accumulation order.  With
``mimic=False`` everything is plain FP64, which is what the finite-difference
check of backward() uses.

Parameter vector layout: W1 (64 x 32), b1 (64), W2 (64 x 128), b2, W3
(64 x 128), b3, Wo (2 x 64), bo (2).
"""
from __future__ import annotations

import numpy as np

FEATURES = 16
HIDDEN = 64
DIMS = (16, 64, 64)
NPARAMS = 64 * 32 + 64 + 2 * (64 * 128 + 64) + 2 * 64 + 2


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to BF16 (round to nearest, ties to even), returned
    as float32 holding the rounded values."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    out = (r << 16).astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out).astype(np.float32)


def unpack(params: np.ndarray):
    p = np.asarray(params, np.float64)
    out, o = [], 0
    for din in DIMS:
        W = p[o:o + 64 * 2 * din].reshape(64, 2 * din)
        o += 64 * 2 * din
        b = p[o:o + 64]
        o += 64
        out.append((W, b))
    Wo = p[o:o + 128].reshape(2, 64)
    bo = p[o + 128:o + 130]
    return out, Wo, bo


def _nbr_mean(h: np.ndarray, rowptr, colids, mimic: bool) -> np.ndarray:
    n = rowptr.shape[0] - 1
    deg = np.diff(rowptr)
    if mimic:
        acc = np.zeros(h.shape, np.float32)
        hf = h.astype(np.float32)
        for s in range(int(deg.max()) if n else 0):
            has = deg > s
            idx = rowptr[:-1][has] + s
            acc[has] += hf[colids[idx]]
        inv = np.where(deg > 0, np.float32(1.0) / np.maximum(deg, 1).astype(np.float32), np.float32(0.0))
        return bf16(acc * inv.astype(np.float32)[:, None])
    acc = np.zeros(h.shape, np.float64)
    np.add.at(acc, np.repeat(np.arange(n), deg), h[colids[:rowptr[-1]]])
    return acc / np.maximum(deg, 1)[:, None] * (deg > 0)[:, None]


def forward(params, rowptr, colids, features, mimic: bool = True):
    """-> dict(xy, h: [h1, h2, h3], A: [A1, A2, A3] (the [h | agg] inputs))."""
    rowptr = np.asarray(rowptr, np.int64)
    colids = np.asarray(colids, np.int64)
    layers, Wo, bo = unpack(params)
    rnd = bf16 if mimic else (lambda x: np.asarray(x, np.float64))
    h = rnd(np.asarray(features, np.float32)).astype(np.float64)
    hs, As = [], []
    for W, b in layers:
        agg = _nbr_mean(h, rowptr, colids, mimic).astype(np.float64)
        A = np.concatenate([h, agg], axis=1)
        Wr = rnd(W.astype(np.float32)).astype(np.float64) if mimic else W
        z = A @ Wr.T
        if mimic:
            z = (z.astype(np.float32) + b.astype(np.float32)).astype(np.float64)
        else:
            z = z + b
        h = np.maximum(z, 0.0)
        h = rnd(h.astype(np.float32)).astype(np.float64) if mimic else h
        hs.append(h)
        As.append(A)
    xy = h @ Wo.T + bo
    return dict(xy=xy, h=hs, A=As)


def loss_and_grad(params, rowptr, colids, features, target, vweight, mimic: bool = True):
    """Loss sum_v w_v |xy_v - t_v|^2 and its gradient (flat, FP64)."""
    rowptr = np.asarray(rowptr, np.int64)
    colids = np.asarray(colids, np.int64)
    f = forward(params, rowptr, colids, features, mimic)
    layers, Wo, bo = unpack(params)
    rnd = (lambda x: bf16(np.asarray(x, np.float32)).astype(np.float64)) if mimic else (lambda x: x)
    w = np.asarray(vweight, np.float64)[:, None]
    d = f["xy"] - np.asarray(target, np.float64)
    loss = float(np.sum(w * d * d))
    dxy = 2.0 * w * d
    if mimic:
        dxy = dxy.astype(np.float32).astype(np.float64)
    grads = [None] * 3
    h3 = f["h"][2]
    gWo = dxy.T @ h3
    gbo = dxy.sum(0)
    dz = (dxy @ Wo) * (h3 > 0)
    deg = np.diff(rowptr)
    n = rowptr.shape[0] - 1
    for l in (2, 1, 0):
        W, b = layers[l]
        din = DIMS[l]
        A = f["A"][l]
        dzr = rnd(dz)
        gW = dzr.T @ A
        gb = dz.sum(0)
        grads[l] = (gW, gb)
        if l > 0:
            Wr = rnd(W) if mimic else W
            q = dzr @ Wr
            P = q[:, :din]
            inv = np.where(deg > 0, 1.0 / np.maximum(deg, 1), 0.0)
            if mimic:
                inv = (np.float32(1.0) / np.maximum(deg, 1).astype(np.float32)).astype(np.float64) * (deg > 0)
            G = q[:, din:] * inv[:, None]
            s = P.copy()
            np.add.at(s, np.repeat(np.arange(n), deg), G[colids[:rowptr[-1]]])
            dz = s * (f["h"][l - 1] > 0)
    flat = []
    for gW, gb in grads:
        flat += [gW.ravel(), gb]
    flat += [gWo.ravel(), gbo]
    return loss, np.concatenate(flat), f


def init_params(seed: int = 0) -> np.ndarray:
    """He-style random initialisation (FP32)."""
    rng = np.random.default_rng(seed)
    out = []
    for din in DIMS:
        out.append(rng.normal(0.0, np.sqrt(2.0 / (2 * din)), size=64 * 2 * din))
        out.append(np.zeros(64))
    out.append(rng.normal(0.0, np.sqrt(1.0 / 64), size=128))
    out.append(np.zeros(2))
    return np.concatenate(out).astype(np.float32)


# ---- input features (batchlayoutcode_gb300/csrc/features.cu) ----------------

def splitmix64_pivots(n: int, seed: int, k: int = 16) -> np.ndarray:
    """The device's pivot choice: splitmix64 draws modulo n, duplicates skipped."""
    if n <= k:
        return np.arange(k) % n
    mask = (1 << 64) - 1
    x = seed & mask
    out = []
    while len(out) < k:
        x = (x + 0x9E3779B97F4A7C15) & mask
        z = x
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & mask
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & mask
        z ^= z >> 31
        p = z % n
        if p not in out:
            out.append(p)
    return np.array(out, np.int64)


def hop_distances(rowptr, colids, pivots) -> np.ndarray:
    """(n, 16) hop distances, -1 where unreachable (FP64 BFS by scipy)."""
    from scipy.sparse import csr_matrix
    from scipy.sparse.csgraph import shortest_path
    rowptr = np.asarray(rowptr, np.int64)
    n = rowptr.shape[0] - 1
    A = csr_matrix((np.ones(rowptr[-1]), np.asarray(colids, np.int64)[:rowptr[-1]], rowptr), shape=(n, n))
    D = shortest_path(A, unweighted=True, directed=False, indices=np.asarray(pivots)).T
    return np.where(np.isinf(D), -1, D).astype(np.int64)


def features(rowptr, colids, pivots):
    """-> (features (n, 16) FP64, eigenvalues (16,), hop distances)."""
    rowptr = np.asarray(rowptr, np.int64)
    colids = np.asarray(colids, np.int64)
    n = rowptr.shape[0] - 1
    d = hop_distances(rowptr, colids, pivots).astype(np.float64)
    for s in range(d.shape[1]):
        col = d[:, s]
        m = col[col >= 0].max() if np.any(col >= 0) else 0.0
        col[col < 0] = m + 1
    D2 = d * d
    r = D2.mean(1)
    c = D2.mean(0)
    g = c.mean()
    C = -0.5 * (D2 - r[:, None] - c[None, :] + g)
    S = C.T @ C
    lam, V = np.linalg.eigh(S)
    order = np.argsort(-lam, kind="stable")
    lam, V = lam[order], V[:, order]
    for j in range(V.shape[1]):
        arg = int(np.argmax(np.abs(V[:, j])))
        if V[arg, j] < 0:
            V[:, j] = -V[:, j]
    Y = C @ V[:, :12]
    Y = Y / np.sqrt(lam[0] / n) if lam[0] > 0 else Y * 0.0
    deg = np.diff(rowptr).astype(np.float64)
    ld = np.log2(1.0 + deg)
    nb = np.zeros(n)
    np.add.at(nb, np.repeat(np.arange(n), np.diff(rowptr)), ld[colids[:rowptr[-1]]])
    nb = np.where(deg > 0, nb / np.maximum(deg, 1), 0.0)
    F = np.concatenate([Y, ld[:, None], (1.0 / (1.0 + deg))[:, None], nb[:, None],
                        np.full((n, 1), np.log2(n) / 20.0)], axis=1)
    return F, lam, d
