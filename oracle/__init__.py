"""ctypes binding of the FP64 CPU oracle (oracle/oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py.  Never imported by batchlayoutcode_gb300.

Two builds of the same source:
  _build/liboracle.so       -O2, no fast-math, no FMA contraction (parity)
  _build/liboracle_fast.so  the reference Makefile's optimisation flags
                            (-O3 -ffast-math -fopenmp, +AVX-512 on x86_64),
                            used only as the timed CPU baseline
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "oracle.cpp")


def _flags(fast: bool) -> list[str]:
    base = ["-shared", "-fPIC", "-fopenmp", "-std=c++17"]
    if fast:
        arch = ["-mavx512f", "-mavx512dq"] if platform.machine() == "x86_64" else []
        return base + ["-O3", "-ffast-math"] + arch
    return base + ["-O2", "-ffp-contract=off"]


def build(quiet: bool = True) -> None:
    """Compile both oracle variants (seconds)."""
    os.makedirs(BUILD, exist_ok=True)
    procs = []
    for fast, name in ((False, "liboracle.so"), (True, "liboracle_fast.so")):
        out = os.path.join(BUILD, name)
        if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(SRC):
            continue
        procs.append(subprocess.Popen(["g++", *_flags(fast), "-o", out, SRC],
                                      stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
    for p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + out.decode())


def reference_dir() -> str | None:
    """Where the reference's sources are: $BL_REFERENCE_DIR, else a checkout
    named `reference` beside this repository; None when neither holds
    sample/algorithms.cpp."""
    cands = [os.environ.get("BL_REFERENCE_DIR", ""),
             os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")]
    for c in cands:
        if c and os.path.isfile(os.path.join(c, "sample", "algorithms.cpp")):
            return c
    return None


def build_reference(ref: str | None = None, quiet: bool = True) -> bool:
    """Compile the reference from its own sources into oracle/_ref/ with
    oracle/build_ref.sh (test infrastructure).  False when no sources."""
    ref = ref or reference_dir()
    if not ref:
        return False
    subprocess.run([os.path.join(HERE, "build_ref.sh"), ref], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return True


_libs: dict[bool, C.CDLL] = {}

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C")


def lib(fast: bool = False) -> C.CDLL:
    if fast in _libs:
        return _libs[fast]
    build()
    L = C.CDLL(os.path.join(BUILD, "liboracle_fast.so" if fast else "liboracle.so"))
    L.orc_morton_sort.argtypes = [C.c_int, _f64p, _f64p, _u64p, _i32p]
    L.orc_bh_tree.argtypes = [C.c_int, _f64p, C.c_int, _i32p, _i32p, _i32p, _i32p, _f64p]
    L.orc_bh_repulsion.argtypes = [C.c_int, _f64p, C.c_int, _f64p, C.c_double, _f64p, C.c_int, C.c_void_p]
    L.orc_layout.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, C.c_int, C.c_int, C.c_double,
                             C.c_double, C.c_double, C.c_double, C.c_int, C.c_void_p, _f64p]
    L.orc_smu_iteration.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, C.c_int, C.c_double,
                                    C.c_double, C.c_void_p, C.c_int]
    L.orc_smu_iteration.restype = C.c_double
    L.orc_bh_iteration.argtypes = [C.c_int, _i32p, _i32p, _f64p, C.c_int, C.c_double, C.c_double,
                                   C.c_double, C.c_void_p, C.c_int]
    L.orc_bh_iteration.restype = C.c_double
    L.orc_forces_on_trajectory.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, C.c_int, C.c_double,
                                           C.c_double, _f64p, C.c_int]
    L.orc_forces_on_trajectory.restype = C.c_double
    L.orc_greedy_walks.argtypes = [C.c_int, _i32p, _i32p, np.ctypeslib.ndpointer(np.int64, flags="C"),
                                   C.c_void_p, C.c_longlong]
    L.orc_greedy_walks.restype = C.c_longlong
    _libs[fast] = L
    return L


def _threads(nthreads: int | None) -> int:
    return nthreads if nthreads else (os.cpu_count() or 1)


def morton_sort(xy: np.ndarray):
    """-> (frame[minX, minY, MAXMIN], sorted keys uint64, permutation int32)."""
    xy = np.ascontiguousarray(xy, dtype=np.float64)
    n = xy.shape[0]
    frame = np.zeros(3)
    keys = np.zeros(n, np.uint64)
    perm = np.zeros(n, np.int32)
    if lib().orc_morton_sort(n, xy.ravel(), frame, keys, perm) != 0:
        raise ValueError("morton_sort")
    return frame, keys, perm


def bh_tree(xy: np.ndarray) -> dict:
    """Canonical compressed quadtree (nodes with >= 2 children, pre-order)."""
    xy = np.ascontiguousarray(xy, dtype=np.float64)
    n = xy.shape[0]
    cap = 2 * n + 8
    lo, hi, dep, nc = (np.zeros(cap, np.int32) for _ in range(4))
    cxy = np.zeros(2 * cap)
    m = lib().orc_bh_tree(n, xy.ravel(), cap, lo, hi, dep, nc, cxy)
    if m < 0:
        raise RuntimeError("tree capacity")
    return dict(lo=lo[:m], hi=hi[:m], depth=dep[:m], nchild=nc[:m], centroid=cxy[: 2 * m].reshape(m, 2))


def bh_repulsion(tree_xy: np.ndarray, queries: np.ndarray, theta: float, nthreads=None, visits: bool = False):
    """Barnes-Hut repulsion of every query; with visits=True also the number
    of tree records (nodes tested, leaf points reached) each walk reads."""
    t = np.ascontiguousarray(tree_xy, dtype=np.float64)
    q = np.ascontiguousarray(queries, dtype=np.float64)
    out = np.zeros_like(q)
    vis = np.zeros(q.shape[0], np.int64) if visits else None
    lib().orc_bh_repulsion(t.shape[0], t.ravel(), q.shape[0], q.ravel(), theta, out.ravel(), _threads(nthreads),
                           vis.ctypes.data if visits else None)
    return (out, vis) if visits else out


def layout(algo: int, rowptr, colids, xy, iterations: int, batch: int = 256, theta: float = 1.2,
           weight: float = 1.0, engt: float = 0.01, step: float = -1.0, nthreads=None,
           fast: bool = False, want_forces: bool = False):
    """Run a whole layout method; returns (xy_out, energy, loops[, forces])."""
    rp = np.ascontiguousarray(rowptr, dtype=np.int32)
    ci = np.ascontiguousarray(colids, dtype=np.int32)
    pos = np.ascontiguousarray(xy, dtype=np.float64).copy()
    n = pos.shape[0]
    res = np.zeros(2)
    forces = np.zeros((n, 2)) if want_forces else None
    fptr = forces.ctypes.data if want_forces else None
    rc = lib(fast).orc_layout(algo, n, rp, ci, pos.ravel(), iterations, batch, theta, weight, engt,
                              step, _threads(nthreads), fptr, res)
    if rc != 0:
        raise ValueError(f"orc_layout rc={rc}")
    if want_forces:
        return pos, float(res[0]), int(res[1]), forces
    return pos, float(res[0]), int(res[1])


def smu_iteration(model: int, rowptr, colids, xy, batch: int, weight: float, step: float, nthreads=None):
    """One minibatch iteration; returns (new xy, forces, energy)."""
    pos = np.ascontiguousarray(xy, dtype=np.float64).copy()
    forces = np.zeros_like(pos)
    e = lib().orc_smu_iteration(model, pos.shape[0], np.ascontiguousarray(rowptr, np.int32),
                                np.ascontiguousarray(colids, np.int32), pos.ravel(), batch, weight, step,
                                forces.ctypes.data, _threads(nthreads))
    return pos, forces, e


def bh_iteration(rowptr, colids, xy, batch: int, theta: float, weight: float, step: float, nthreads=None):
    pos = np.ascontiguousarray(xy, dtype=np.float64).copy()
    forces = np.zeros_like(pos)
    e = lib().orc_bh_iteration(pos.shape[0], np.ascontiguousarray(rowptr, np.int32),
                               np.ascontiguousarray(colids, np.int32), pos.ravel(), batch, theta, weight,
                               step, forces.ctypes.data, _threads(nthreads))
    return pos, forces, e


def forces_on_trajectory(algo: int, rowptr, colids, xy_start, xy_end, batch: int, theta: float = 1.2,
                         weight: float = 1.0, nthreads=None):
    """Forces of one iteration where batch b is evaluated from the state
    {xy_end for earlier batches, xy_start otherwise}: the reference's step
    re-seeded from another implementation's batch-start states.  algo 2, 3,
    8 (minibatch), 4 (Barnes-Hut), 7 (SD), 5 (greedy, first phase) or 50
    (greedy, second phase).  -> (forces, energy)"""
    a = np.ascontiguousarray(xy_start, dtype=np.float64)
    b = np.ascontiguousarray(xy_end, dtype=np.float64)
    f = np.zeros_like(a)
    e = lib().orc_forces_on_trajectory(algo, a.shape[0], np.ascontiguousarray(rowptr, np.int32),
                                       np.ascontiguousarray(colids, np.int32), a.ravel(), b.ravel(), batch, theta,
                                       weight, f.ravel(), _threads(nthreads))
    return f, e


def greedy_walks(rowptr, colids):
    """Algo 5's repulsion sources per vertex -> (offsets int64 [n+1], sources int32)."""
    rp = np.ascontiguousarray(rowptr, np.int32)
    ci = np.ascontiguousarray(colids, np.int32)
    n = rp.shape[0] - 1
    off = np.zeros(n + 1, np.int64)
    total = lib().orc_greedy_walks(n, rp, ci, off, None, 0)
    src = np.zeros(max(total, 1), np.int32)
    lib().orc_greedy_walks(n, rp, ci, off, src.ctypes.data, total)
    return off, src[:total]
