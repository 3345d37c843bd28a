"""Seeded synthetic graphs and initial layouts for BatchLayout workloads.

The reference ships no benchmark inputs; its layouts are computed from
MatrixMarket files read by ``ReadASCII`` (IO.h:60-155) into a symmetric CSR
with self-loops dropped and column ids ascending per row (CSR.h:155-186).
These generators produce such graphs directly:

* ``grid_triangulated``  -- an R x C lattice with right, down and down-right
  diagonal edges (64x64 -> 4,096 vertices, 12,033 edges).
* ``random_geometric``   -- n points uniform in the unit square, edges within
  radius sqrt(d / (pi n)) so the mean degree is about d, largest connected
  component kept (vertex ids keep generation order, i.e. spatially random).
* ``chung_lu``           -- expected-degree power-law graph, weights
  w_i ~ (i + i0)^(-1/(gamma-1)), m = n d / 2 endpoint pairs drawn with
  probability proportional to w, self loops and duplicates removed, largest
  component kept; edge values uniform in [0.5, 2] (written to .mtx files but
  ignored by the layout, as in the reference, whose reader truncates values
  with atoi and whose algorithms never read them).

All coordinates produced here are exactly representable in float32, so a
float32 device layout and an FP64 CPU run start from identical values.
"""
from __future__ import annotations

import dataclasses
import math
import os

import numpy as np


@dataclasses.dataclass
class Graph:
    """Symmetric CSR graph, int32 arrays, colids ascending per row."""

    n: int
    rowptr: np.ndarray
    colids: np.ndarray
    values: np.ndarray | None = None  # per-edge values of the upper triangle (unused by layout)
    name: str = "graph"

    @property
    def nnz(self) -> int:
        return int(self.rowptr[-1])


def csr_from_edges(n: int, u: np.ndarray, v: np.ndarray, name: str = "graph") -> Graph:
    """Build the symmetric CSR that ReadASCII + CSC + CSR yield for an undirected
    edge list without self loops or duplicates (IO.h:122-137, CSR.h:176-183)."""
    u = np.asarray(u, dtype=np.int64)
    v = np.asarray(v, dtype=np.int64)
    keep = u != v
    u, v = u[keep], v[keep]
    a = np.minimum(u, v)
    b = np.maximum(u, v)
    key = np.unique(a * n + b)
    a, b = key // n, key % n
    rows = np.concatenate([a, b])
    cols = np.concatenate([b, a])
    order = np.lexsort((cols, rows))
    rows, cols = rows[order], cols[order]
    counts = np.bincount(rows, minlength=n)
    rowptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=rowptr[1:])
    return Graph(n=n, rowptr=rowptr.astype(np.int32), colids=cols.astype(np.int32), name=name)


def largest_component(g: Graph) -> Graph:
    """Keep the largest connected component, relabelling vertices in id order."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import connected_components

    adj = sp.csr_matrix((np.ones(g.nnz, dtype=np.int8), g.colids, g.rowptr), shape=(g.n, g.n))
    ncomp, labels = connected_components(adj, directed=False)
    if ncomp == 1:
        return g
    big = np.bincount(labels).argmax()
    keep = labels == big
    newid = -np.ones(g.n, dtype=np.int64)
    newid[keep] = np.arange(int(keep.sum()))
    rows = np.repeat(np.arange(g.n), np.diff(g.rowptr))
    m = keep[rows] & keep[g.colids]
    r2, c2 = newid[rows[m]], newid[g.colids[m]]
    sel = r2 < c2
    return csr_from_edges(int(keep.sum()), r2[sel], c2[sel], name=g.name)


def grid_triangulated(rows: int = 64, cols: int = 64) -> Graph:
    idx = np.arange(rows * cols).reshape(rows, cols)
    e = [
        (idx[:, :-1].ravel(), idx[:, 1:].ravel()),
        (idx[:-1, :].ravel(), idx[1:, :].ravel()),
        (idx[:-1, :-1].ravel(), idx[1:, 1:].ravel()),
    ]
    u = np.concatenate([a for a, _ in e])
    v = np.concatenate([b for _, b in e])
    return csr_from_edges(rows * cols, u, v, name=f"grid{rows}x{cols}")


def random_geometric(n: int, mean_degree: float = 6.0, seed: int = 1, lcc: bool = True) -> Graph:
    from scipy.spatial import cKDTree

    rng = np.random.default_rng(seed)
    pts = rng.random((n, 2))
    r = math.sqrt(mean_degree / (math.pi * n))
    pairs = cKDTree(pts).query_pairs(r, output_type="ndarray")
    g = csr_from_edges(n, pairs[:, 0], pairs[:, 1], name=f"rgg{n}")
    return largest_component(g) if lcc else g


def chung_lu(n: int, gamma: float = 2.5, mean_degree: float = 10.0, seed: int = 1,
             lcc: bool = True) -> Graph:
    rng = np.random.default_rng(seed)
    i0 = max(1.0, n ** (1.0 / (gamma - 1.0)) / 50.0)
    w = (np.arange(n) + i0) ** (-1.0 / (gamma - 1.0))
    p = w / w.sum()
    m = int(round(n * mean_degree / 2.0))
    u = rng.choice(n, size=m, p=p)
    v = rng.choice(n, size=m, p=p)
    g = csr_from_edges(n, u, v, name=f"chunglu{n}")
    g = largest_component(g) if lcc else g
    nupper = g.nnz // 2
    g.values = rng.uniform(0.5, 2.0, size=nupper)
    return g


def init_disc(n: int, seed: int = 1, radius: float = 3.0) -> np.ndarray:
    """Uniform points in the disc of radius 3: the distribution of randInit
    (sample/algorithms.cpp:16-28), drawn from a seeded generator."""
    rng = np.random.default_rng(seed)
    out = np.empty((0, 2))
    while out.shape[0] < n:
        c = rng.uniform(-1.0, 1.0, size=(2 * (n - out.shape[0]) + 16, 2))
        c = c[(c * c).sum(1) <= 1.0]
        out = np.concatenate([out, c])
    return (out[:n] * radius).astype(np.float32)


def init_square(n: int, seed: int = 1, half: float = 3.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.uniform(-half, half, size=(n, 2)).astype(np.float32)


def write_mtx(g: Graph, path: str) -> None:
    """Write the lower triangle as a symmetric MatrixMarket file (1-based)."""
    rows = np.repeat(np.arange(g.n), np.diff(g.rowptr))
    sel = rows > g.colids
    r = rows[sel] + 1
    c = g.colids[sel] + 1
    with open(path, "w") as f:
        if g.values is not None:
            f.write("%%MatrixMarket matrix coordinate real symmetric\n")
            f.write(f"{g.n} {g.n} {r.size}\n")
            vals = g.values[: r.size]
            f.write("".join(f"{a} {b} {x:.6f}\n" for a, b, x in zip(r.tolist(), c.tolist(), vals.tolist())))
        else:
            f.write("%%MatrixMarket matrix coordinate pattern symmetric\n")
            f.write(f"{g.n} {g.n} {r.size}\n")
            f.write("".join(f"{a} {b}\n" for a, b in zip(r.tolist(), c.tolist())))


def write_initf(xy: np.ndarray, path: str) -> None:
    """`-initf` file: one `x y id` line per vertex (read with sscanf "%lf %lf %d",
    sample/algorithms.cpp:112-116).  Each float32 value is written with the
    shortest decimal that parses back (as a double) to exactly that value, so a
    reader in FP64 and the float32 device layout start from the same numbers."""
    xy = np.asarray(xy, dtype=np.float32).astype(np.float64)
    with open(path, "w") as f:
        f.write("".join(f"{x!r} {y!r} {i + 1}\n" for i, (x, y) in enumerate(xy.tolist())))


def batched_mix(num_graphs: int = 2048, lo: int = 200, hi: int = 20000, seed: int = 1,
                bh_min_vertices: int = 5000):
    """Many small graphs for the batched launch: sizes log-uniform in [lo, hi],
    a third each of triangulated grids, random geometric graphs (mean degree 6)
    and Chung-Lu graphs (exponent 2.5, mean degree 8), each with its own
    seeded disc initialisation; algo 2 below `bh_min_vertices` vertices and 4
    from there.  The largest-component step can shrink a graph below its
    drawn size.  -> (list of Graph, list of float32 (n, 2) arrays, algo array)"""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(math.log(lo), math.log(hi), size=num_graphs))
    graphs, xys = [], []
    for g in range(num_graphs):
        n = max(2, int(round(sizes[g])))
        kind = g % 3
        if kind == 0:
            r = max(2, int(round(math.sqrt(n))))
            c = max(1, int(round(n / r)))
            gr = grid_triangulated(r, c)
        elif kind == 1:
            gr = random_geometric(n, 6.0, seed=seed * 100003 + g)
        else:
            gr = chung_lu(n, 2.5, 8.0, seed=seed * 100003 + g)
            gr.values = None
        graphs.append(gr)
        xys.append(init_disc(gr.n, seed=seed * 100003 + g))
    algo = np.array([2 if gr.n < bh_min_vertices else 4 for gr in graphs], np.int32)
    return graphs, xys, algo


def workload(name: str, seed: int = 1):
    """Named workloads with their sizes: returns (graph, initial float32 xy)."""
    if name == "grid64":
        g = grid_triangulated(64, 64)
        return g, init_disc(g.n, seed)
    if name == "rgg1m":
        g = random_geometric(1_000_000, 6.0, seed)
        return g, init_square(g.n, seed)
    if name == "chunglu100k":
        g = chung_lu(100_000, 2.5, 10.0, seed)
        return g, init_disc(g.n, seed)
    raise KeyError(name)


def cached_workload(name: str, seed: int = 1, cache_dir: str | None = None):
    """workload() with an .npz cache (generation of the 1M-vertex graph takes seconds)."""
    cache_dir = cache_dir or os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "workloads")
    os.makedirs(cache_dir, exist_ok=True)
    path = os.path.join(cache_dir, f"{name}_s{seed}.npz")
    if os.path.exists(path):
        z = np.load(path)
        g = Graph(n=int(z["n"]), rowptr=z["rowptr"], colids=z["colids"], name=name)
        return g, z["xy"]
    g, xy = workload(name, seed)
    np.savez(path, n=g.n, rowptr=g.rowptr, colids=g.colids, xy=xy)
    return g, xy
