"""Learned initializer: training set, training and model files.

No counterpart in the reference, whose starting layouts are random, greedy
DFS or read from a file (sample/algorithms.cpp:16-119).  The network and its
training run on the GPU (bl_learned_* in the library); this module generates
the training set and reads and writes model files:

* training graphs: the same generator mix as the benchmark workloads
  (triangulated grids, random geometric graphs of mean degree 6, Chung-Lu
  graphs of exponent 2.5 and mean degree 8), sizes log-uniform in [lo, hi];
* target layouts: what algo 4 produces for each graph on the device (600
  iterations, batch 256, bht 1.2, STEP from 0.3) from the graph's pivot-MDS
  shape scaled to a mean edge length of 1.  (From the greedy DFS start, 600
  iterations leave graphs beyond a few thousand vertices as partly unfolded
  tangles whose RMS radius is capped near 320 by the step schedule, a shape
  no per-vertex function of the graph can predict; from the MDS shape the
  method settles into its balanced layout, which is what the network learns.)
* model file: b"BLMPNN01", uint32 parameter count, the FP32 parameters, then
  the three FP64 coefficients of the edge-length model.

    python -m batchlayoutcode_gb300.learned --train --out <file>
"""
from __future__ import annotations

import argparse
import math
import os
import struct
import time

import numpy as np

from . import graphs as G
from ._lib import MPNN_PARAMS, Algorithms, Mpnn

MAGIC = b"BLMPNN01"
STEP0 = 0.3          # STEP at the start of a refinement from a learned or MDS start
EDGE_LENGTH = 1.0    # mean edge length of the MDS start of the training targets
DEFAULT_MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "mpnn_bh.blw")


def save_model(path: str, params, scale_model) -> None:
    p = np.ascontiguousarray(params, np.float32)
    sm = np.ascontiguousarray(scale_model, np.float64)
    assert p.shape == (MPNN_PARAMS,) and sm.shape == (3,)
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(struct.pack("<I", MPNN_PARAMS))
        f.write(p.astype("<f4").tobytes())
        f.write(sm.astype("<f8").tobytes())


def load_model(path: str | None = None):
    """-> (params float32 [MPNN_PARAMS], scale_model float64 [3])."""
    path = path or DEFAULT_MODEL
    with open(path, "rb") as f:
        if f.read(8) != MAGIC:
            raise ValueError(f"{path}: not a model file")
        (count,) = struct.unpack("<I", f.read(4))
        if count != MPNN_PARAMS:
            raise ValueError(f"{path}: {count} parameters, expected {MPNN_PARAMS}")
        params = np.frombuffer(f.read(4 * count), "<f4").astype(np.float32)
        sm = np.frombuffer(f.read(24), "<f8").astype(np.float64)
    return params, sm


def _training_graph(k: int, n: int, seed: int):
    kind = k % 3
    if kind == 0:
        r = max(2, int(round(math.sqrt(n))))
        return G.grid_triangulated(r, max(2, int(round(n / r))))
    if kind == 1:
        return G.random_geometric(n, 6.0, seed=seed * 7919 + k)
    g = G.chung_lu(n, 2.5, 8.0, seed=seed * 7919 + k)
    g.values = None
    return g


def training_graphs(count: int, lo: int, hi: int, seed: int = 1000, workers: int = 1):
    """Seeded graphs of the benchmark mix with log-uniform sizes (graph k is
    the same whatever the number of worker processes)."""
    rng = np.random.default_rng(seed)
    sizes = [max(16, int(round(s))) for s in np.exp(rng.uniform(math.log(lo), math.log(hi), size=count))]
    if workers <= 1:
        return [_training_graph(k, n, seed) for k, n in enumerate(sizes)]
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    # spawn: the workers start clean (no CUDA state is inherited)
    with ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(_training_graph, range(count), sizes, [seed] * count, chunksize=4))


def mds_start(g, edge_length: float = EDGE_LENGTH, seed: int = 1, device: int = 0) -> np.ndarray:
    """The graph's first two pivot-MDS components (its input features 0 and 1)
    scaled to the given mean edge length."""
    with Mpnn(device=device) as net:
        f, _, _ = net.features(g.rowptr, g.colids, seed=seed)
    y = f[:, :2].astype(np.float64)
    rows = np.repeat(np.arange(g.n), np.diff(g.rowptr))
    el = np.linalg.norm(y[rows] - y[g.colids], axis=1).mean() if g.colids.size else 1.0
    return y * (edge_length / max(el, 1e-30))


def target_layouts(graphs, iterations: int = 600, batch: int = 256, theta: float = 1.2, step0: float = STEP0,
                   device: int = 0):
    """algo 4 from the MDS start of every graph, on the device."""
    out = []
    for g in graphs:
        with Algorithms(g.rowptr, g.colids, device=device) as a:
            a.nCoordinates = mds_start(g, device=device)
            a.run_resident(4, iterations, batch, theta, step0)
            out.append(a.nCoordinates)
    return out


def init_params(seed: int = 0) -> np.ndarray:
    """He initialisation of the message-passing weights, zero biases and a zero
    readout, so an untrained network leaves the MDS start unchanged (FP32)."""
    rng = np.random.default_rng(seed)
    parts = []
    for din in (16, 64, 64):
        parts.append(rng.normal(0.0, math.sqrt(2.0 / (2 * din)), size=64 * 2 * din))
        parts.append(np.zeros(64))
    parts.append(np.zeros(128))
    parts.append(np.zeros(2))
    return np.concatenate(parts).astype(np.float32)


def train(graphs, layouts, epochs: int = 2000, lr: float = 3e-3, seed: int = 1, init_seed: int = 0,
          device: int = 0):
    """-> (params, scale_model, loss history) from bl_learned_train."""
    with Mpnn(init_params(init_seed), device=device) as net:
        return net.train([(g.rowptr, g.colids) for g in graphs], layouts, epochs, lr, seed)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--train", action="store_true")
    ap.add_argument("--out", default=DEFAULT_MODEL)
    ap.add_argument("--graphs", type=int, default=48)
    ap.add_argument("--lo", type=int, default=1000)
    ap.add_argument("--hi", type=int, default=100000)
    ap.add_argument("--iterations", type=int, default=600)
    ap.add_argument("--epochs", type=int, default=2000)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--seed", type=int, default=1000)
    ap.add_argument("--workers", type=int, default=os.cpu_count() or 1,
                    help="processes generating the training graphs")
    args = ap.parse_args(argv)
    if not args.train:
        ap.print_help()
        return
    from .build import build
    build()
    t0 = time.time()
    gs = training_graphs(args.graphs, args.lo, args.hi, args.seed, args.workers)
    t1 = time.time()
    lays = target_layouts(gs, args.iterations)
    t2 = time.time()
    params, sm, hist = train(gs, lays, args.epochs, args.lr, seed=args.seed)
    t3 = time.time()
    save_model(args.out, params, sm)
    nv = sum(g.n for g in gs)
    print(f"graphs {len(gs)} vertices {nv} | generate {t1 - t0:.1f} s, target layouts {t2 - t1:.1f} s, "
          f"training {t3 - t2:.1f} s ({args.epochs} epochs) | loss {hist[0]:.4f} -> {hist[-1]:.4f} | "
          f"scale model {sm.tolist()} | {args.out}")


if __name__ == "__main__":
    main()
