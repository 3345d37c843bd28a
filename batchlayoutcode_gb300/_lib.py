"""ctypes binding of libbatchlayout_gb300.so (include/batchlayout_gb300.h).

There is no CPU fallback: if the library is missing or the device call fails,
the error is raised.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libbatchlayout_gb300.so")

# every symbol declared in include/batchlayout_gb300.h
EXPORTS = (
    "bl_algorithms_create", "bl_create_error", "bl_destroy", "bl_last_error", "bl_num_vertices",
    "bl_read_matrix_market", "bl_free", "bl_set_coordinates", "bl_get_coordinates", "bl_get_forces",
    "bl_rand_init", "bl_init_dfs", "bl_file_initialization", "bl_cache_blocking_minibatch",
    "bl_cache_blocking_minibatch_converged", "bl_linlog_cache_blocking_minibatch",
    "bl_fa_cache_blocking_minibatch", "bl_barnes_hut_approximation", "bl_approx_cache_block_bh",
    "bl_write_to_file", "bl_minibatch_iteration", "bl_barnes_hut_iteration", "bl_morton_order",
    "bl_quadtree", "bl_bh_repulsion", "bl_run_resident", "bl_set_graph_mode", "bl_last_kernel_time",
    "bl_kernel_launches", "bl_last_run_ms", "bl_random_coordinates", "bl_greedy_coordinates", "bl_write_coordinates",
    "bl_minibatch_iteration_noalloc", "bl_batch_create", "bl_batched_prepare", "bl_batched_run",
    "bl_batched_result", "bl_batched_layout", "bl_batched_parts", "bl_batched_set_parts",
    "bl_batched_graph_cycles", "bl_mpnn_set_params", "bl_mpnn_get_params", "bl_mpnn_run",
    "bl_learned_features", "bl_learned_train", "bl_learned_init", "bl_learned_layout",
    "bl_learned_load_model", "bl_approx_force_directed", "bl_cache_blocking_minibatch_sd",
    "bl_greedy_iteration", "bl_greedy_walks", "bl_read_matrix_market_cached", "bl_bfs_init",
    "bl_cursor_neighbours", "bl_wait_selftest",
)

_lib = None


class BatchLayoutError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"batchlayout error {code}: {msg}")
        self.code = code


def load() -> C.CDLL:
    """Load the library (build it first with batchlayoutcode_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run `python -m batchlayoutcode_gb300.build`")
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, f64, cp = C.c_void_p, C.c_int, C.c_longlong, C.c_double, C.c_char_p
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int)
    sig = {
        "bl_algorithms_create": (vp, [i32, i32, i64, ip, ip, cp, cp, i32, f64, f64, cp]),
        "bl_create_error": (cp, []),
        "bl_destroy": (None, [vp]),
        "bl_last_error": (cp, [vp]),
        "bl_num_vertices": (i32, [vp]),
        "bl_read_matrix_market": (i32, [cp, C.POINTER(C.c_longlong), dp, C.POINTER(ip), C.POINTER(ip), cp, i32]),
        "bl_free": (None, [vp]),
        "bl_set_coordinates": (i32, [vp, dp, i32]),
        "bl_get_coordinates": (i32, [vp, dp, i32]),
        "bl_get_forces": (i32, [vp, dp, i32]),
        "bl_rand_init": (i32, [vp]),
        "bl_init_dfs": (i32, [vp]),
        "bl_file_initialization": (i32, [vp]),
        "bl_cache_blocking_minibatch": (i32, [vp, i32, i32, i32, i32, dp]),
        "bl_cache_blocking_minibatch_converged": (i32, [vp, i32, i32, i32, i32, dp]),
        "bl_linlog_cache_blocking_minibatch": (i32, [vp, i32, i32, i32, dp]),
        "bl_fa_cache_blocking_minibatch": (i32, [vp, i32, i32, i32, dp]),
        "bl_barnes_hut_approximation": (i32, [vp, i32, i32, i32, f64, i32, dp]),
        "bl_approx_cache_block_bh": (i32, [vp, i32, i32, i32, dp]),
        "bl_write_to_file": (i32, [vp, cp, cp, i32]),
        "bl_minibatch_iteration": (i32, [vp, i32, i32, f64, dp]),
        "bl_barnes_hut_iteration": (i32, [vp, i32, f64, f64, dp]),
        "bl_morton_order": (i32, [vp, dp, C.POINTER(C.c_ulonglong), ip]),
        "bl_quadtree": (i32, [vp, i32, ip, ip, ip, ip, dp]),
        "bl_bh_repulsion": (i32, [vp, f64, dp, C.POINTER(C.c_longlong)]),
        "bl_run_resident": (i32, [vp, i32, i32, i32, f64, f64, dp]),
        "bl_set_graph_mode": (i32, [vp, i32]),
        "bl_last_kernel_time": (i32, [vp, cp, dp]),
        "bl_kernel_launches": (i64, [vp]),
        "bl_last_run_ms": (i32, [vp, dp]),
        "bl_random_coordinates": (i32, [i32, dp]),
        "bl_greedy_coordinates": (i32, [i32, ip, ip, dp]),
        "bl_write_coordinates": (i32, [cp, cp, cp, dp, i32, cp, i32]),
        "bl_minibatch_iteration_noalloc": (i32, [i32, vp, vp, vp, vp, vp, i32, i32, f64, f64, dp, vp]),
        "bl_batch_create": (vp, [i32]),
        "bl_batched_prepare": (i32, [vp, i32, ip, C.POINTER(C.c_longlong), ip, ip, ip, dp]),
        "bl_batched_run": (i32, [vp, i32, i32, f64, f64, dp]),
        "bl_batched_result": (i32, [vp, dp, dp]),
        "bl_batched_layout": (i32, [vp, i32, ip, C.POINTER(C.c_longlong), ip, ip, ip, dp, i32, i32, f64, f64, dp,
                                    dp]),
        "bl_batched_parts": (i32, [vp, ip]),
        "bl_batched_set_parts": (i32, [vp, ip]),
        "bl_batched_graph_cycles": (i32, [vp, C.POINTER(C.c_ulonglong)]),
        "bl_mpnn_set_params": (i32, [vp, C.POINTER(C.c_float)]),
        "bl_mpnn_get_params": (i32, [vp, C.POINTER(C.c_float)]),
        "bl_mpnn_run": (i32, [vp, i32, ip, ip, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                              C.POINTER(C.c_float), C.POINTER(C.c_ushort), C.POINTER(C.c_double),
                              C.POINTER(C.c_float)]),
        "bl_learned_features": (i32, [vp, i32, ip, ip, i32, ip, C.POINTER(C.c_float), C.POINTER(C.c_ushort), ip]),
        "bl_learned_train": (i32, [vp, i32, ip, C.POINTER(C.c_longlong), ip, ip, dp, i32, f64, i32,
                                   C.POINTER(C.c_float), dp, dp]),
        "bl_learned_init": (i32, [vp, C.POINTER(C.c_float), dp, i32]),
        "bl_learned_layout": (i32, [vp, C.POINTER(C.c_float), dp, i32, i32, i32, f64, f64, f64, dp]),
        "bl_learned_load_model": (i32, [cp, C.POINTER(C.c_float), dp]),
        "bl_approx_force_directed": (i32, [vp, i32, i32, i32, dp]),
        "bl_cache_blocking_minibatch_sd": (i32, [vp, i32, i32, i32, i32, dp]),
        "bl_greedy_iteration": (i32, [vp, i32, f64, dp]),
        "bl_greedy_walks": (i32, [vp, C.POINTER(C.c_longlong), ip, ip, i64, C.POINTER(C.c_longlong)]),
        "bl_bfs_init": (i32, [vp]),
        "bl_cursor_neighbours": (i32, [i32, ip, ip, ip, ip]),
        "bl_wait_selftest": (i32, [vp, i32, i32]),
        "bl_read_matrix_market_cached": (i32, [cp, cp, C.POINTER(C.c_longlong), dp, C.POINTER(ip), C.POINTER(ip),
                                               cp, i32]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def read_matrix_market(path: str, cache_dir: str | None = None):
    """SetInputMatricesAsCSR: -> (rowptr, colids, info dict).  With cache_dir,
    through the binary CSR cache (info["cached"] tells whether it was used)."""
    L = load()
    info = (C.c_longlong * 5)()
    secs = C.c_double()
    rp = C.POINTER(C.c_int)()
    ci = C.POINTER(C.c_int)()
    err = C.create_string_buffer(512)
    if cache_dir is None:
        rc = L.bl_read_matrix_market(path.encode(), info, C.byref(secs), C.byref(rp), C.byref(ci), err, 512)
    else:
        rc = L.bl_read_matrix_market_cached(path.encode(), cache_dir.encode(), info, C.byref(secs), C.byref(rp),
                                            C.byref(ci), err, 512)
    if rc != 0:
        raise BatchLayoutError(rc, err.value.decode())
    rows, cols, nnz, sym = (int(v) for v in info[:4])
    cached = bool(info[4]) if cache_dir is not None else False
    rowptr = np.ctypeslib.as_array(rp, shape=(rows + 1,)).copy()
    colids = np.ctypeslib.as_array(ci, shape=(max(nnz, 1),))[:nnz].copy()
    L.bl_free(C.cast(rp, C.c_void_p))
    L.bl_free(C.cast(ci, C.c_void_p))
    return rowptr, colids, dict(rows=rows, cols=cols, nnz=nnz, symmetric=bool(sym), seconds=secs.value,
                                cached=cached)


def random_coordinates(n: int) -> np.ndarray:
    """randInit's sequence (one thread), host only."""
    out = np.zeros((n, 2))
    rc = load().bl_random_coordinates(n, _dp(out))
    if rc != 0:
        raise BatchLayoutError(rc, "bl_random_coordinates")
    return out


def greedy_coordinates(rowptr, colids) -> np.ndarray:
    """initDFS's placement, host only."""
    rp = np.ascontiguousarray(rowptr, dtype=np.int32)
    ci = np.ascontiguousarray(colids, dtype=np.int32)
    n = rp.shape[0] - 1
    out = np.zeros((n, 2))
    rc = load().bl_greedy_coordinates(n, _ip(rp), _ip(ci), _dp(out))
    if rc != 0:
        raise BatchLayoutError(rc, "bl_greedy_coordinates")
    return out


def cursor_neighbours(rowptr, colids):
    """The neighbour lists the reference's kindex cursor matches, host only:
    -> (matched_rowptr, matched_colids)."""
    rp = np.ascontiguousarray(rowptr, dtype=np.int32)
    ci = np.ascontiguousarray(colids, dtype=np.int32)
    n = rp.shape[0] - 1
    L = load()
    mrp = np.zeros(n + 1, dtype=np.int32)
    rc = L.bl_cursor_neighbours(n, _ip(rp), _ip(ci), _ip(mrp), None)
    if rc != 0:
        raise BatchLayoutError(rc, "bl_cursor_neighbours")
    mci = np.zeros(max(int(mrp[-1]), 1), dtype=np.int32)
    rc = L.bl_cursor_neighbours(n, _ip(rp), _ip(ci), _ip(mrp), _ip(mci))
    if rc != 0:
        raise BatchLayoutError(rc, "bl_cursor_neighbours")
    return mrp, mci[:int(mrp[-1])]


def write_coordinates(input: str, outputdir: str, tag: str, xy) -> str:
    """writeToFile's naming and format, host only; returns the path written."""
    a = np.ascontiguousarray(xy, dtype=np.float64)
    buf = C.create_string_buffer(4096)
    rc = load().bl_write_coordinates(input.encode(), outputdir.encode(), tag.encode(), _dp(a), a.shape[0], buf, 4096)
    if rc != 0:
        raise BatchLayoutError(rc, "cannot write " + buf.value.decode())
    return buf.value.decode()


class Algorithms:
    """Python mirror of the reference's `class algorithms` (sample/algorithms.h:50-85)
    over the C ABI.  Method names and arguments follow the reference."""

    def __init__(self, rowptr, colids, input: str = "graph.mtx", outputd: str = "", init: int = 2,
                 weight: float = 1.0, th: float = 0.01, ifile: str = "", device: int = 0):
        L = load()
        self._L = L
        self.rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
        self.colids = np.ascontiguousarray(colids, dtype=np.int32)
        self.n = int(self.rowptr.shape[0] - 1)
        ctx = L.bl_algorithms_create(device, self.n, int(self.rowptr[-1]), _ip(self.rowptr), _ip(self.colids),
                                     input.encode(), outputd.encode(), init, weight, th, ifile.encode())
        if not ctx:
            raise BatchLayoutError(-1, L.bl_create_error().decode())
        self._ctx = ctx

    def close(self):
        if getattr(self, "_ctx", None):
            self._L.bl_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int):
        if rc != 0:
            raise BatchLayoutError(rc, self._L.bl_last_error(self._ctx).decode())

    # ---- coordinates ----
    @property
    def nCoordinates(self) -> np.ndarray:
        out = np.zeros((self.n, 2))
        self._check(self._L.bl_get_coordinates(self._ctx, _dp(out), self.n))
        return out

    @nCoordinates.setter
    def nCoordinates(self, xy):
        a = np.ascontiguousarray(xy, dtype=np.float64).reshape(self.n, 2)
        self._check(self._L.bl_set_coordinates(self._ctx, _dp(a), self.n))

    @property
    def prevCoordinates(self) -> np.ndarray:
        out = np.zeros((self.n, 2))
        self._check(self._L.bl_get_forces(self._ctx, _dp(out), self.n))
        return out

    # ---- initialisers ----
    def randInit(self):
        self._check(self._L.bl_rand_init(self._ctx))

    def bfsInit(self):
        """Breadth-first greedy start on the GPU (no reference counterpart)."""
        self._check(self._L.bl_bfs_init(self._ctx))

    def initDFS(self):
        self._check(self._L.bl_init_dfs(self._ctx))

    def fileInitialization(self):
        self._check(self._L.bl_file_initialization(self._ctx))

    # ---- layout methods (return [ENERGY, seconds]) ----
    def _out(self, k=2):
        return (C.c_double * k)()

    def cacheBlockingminiBatchForceDirectedAlgorithm(self, ITERATIONS, NUMOFTHREADS=0, BATCHSIZE=256, flag=0):
        o = self._out()
        self._check(self._L.bl_cache_blocking_minibatch(self._ctx, ITERATIONS, NUMOFTHREADS, BATCHSIZE, flag, o))
        return [o[0], o[1]]

    def cacheBlockingminiBatchForceDirectedAlgorithmConverged(self, ITERATIONS, NUMOFTHREADS=0, BATCHSIZE=256,
                                                             flag=0):
        o = self._out(3)
        self._check(self._L.bl_cache_blocking_minibatch_converged(self._ctx, ITERATIONS, NUMOFTHREADS, BATCHSIZE,
                                                                  flag, o))
        self.loops = int(o[2])
        return [o[0], o[1]]

    def LinLogcacheBlockingminiBatchForceDirectedAlgorithm(self, ITERATIONS, NUMOFTHREADS=0, BATCHSIZE=256):
        o = self._out()
        self._check(self._L.bl_linlog_cache_blocking_minibatch(self._ctx, ITERATIONS, NUMOFTHREADS, BATCHSIZE, o))
        return [o[0], o[1]]

    def FAcacheBlockingminiBatchForceDirectedAlgorithm(self, ITERATIONS, NUMOFTHREADS=0, BATCHSIZE=256):
        o = self._out()
        self._check(self._L.bl_fa_cache_blocking_minibatch(self._ctx, ITERATIONS, NUMOFTHREADS, BATCHSIZE, o))
        return [o[0], o[1]]

    def BarnesHutApproximation(self, ITERATIONS, NUMOFTHREADS=0, BATCHSIZE=256, TH=1.2, flag=0):
        o = self._out()
        self._check(self._L.bl_barnes_hut_approximation(self._ctx, ITERATIONS, NUMOFTHREADS, BATCHSIZE, TH, flag, o))
        return [o[0], o[1]]

    def approxCacheBlockBH(self, ITERATIONS, NUMOFTHREADS=0, BATCHSIZE=256):
        o = self._out()
        self._check(self._L.bl_approx_cache_block_bh(self._ctx, ITERATIONS, NUMOFTHREADS, BATCHSIZE, o))
        return [o[0], o[1]]

    def approxForceDirectedAlgorithm(self, ITERATIONS, NUMOFTHREADS=0, BATCHSIZE=256):
        o = self._out()
        self._check(self._L.bl_approx_force_directed(self._ctx, ITERATIONS, NUMOFTHREADS, BATCHSIZE, o))
        return [o[0], o[1]]

    def cacheBlockingminiBatchForceDirectedAlgorithmSD(self, ITERATIONS, NUMOFTHREADS=0, BATCHSIZE=256, flag=0):
        o = self._out()
        self._check(self._L.bl_cache_blocking_minibatch_sd(self._ctx, ITERATIONS, NUMOFTHREADS, BATCHSIZE, flag, o))
        return [o[0], o[1]]

    def writeToFile(self, f: str) -> str:
        buf = C.create_string_buffer(4096)
        self._check(self._L.bl_write_to_file(self._ctx, f.encode(), buf, 4096))
        return buf.value.decode()

    # ---- building blocks ----
    def minibatch_iteration(self, model: int, batch: int, step: float) -> float:
        e = C.c_double()
        self._check(self._L.bl_minibatch_iteration(self._ctx, model, batch, step, C.byref(e)))
        return e.value

    def greedy_iteration(self, batch: int, step: float) -> float:
        """One first-phase iteration of algo 5."""
        e = C.c_double()
        self._check(self._L.bl_greedy_iteration(self._ctx, batch, step, C.byref(e)))
        return e.value

    def greedy_walks(self):
        """Algo 5's walk sources -> (offsets int64 [n+1], sources int32, counts int32)."""
        off = np.zeros(self.n + 1, np.int64)
        total = C.c_longlong()
        llp = C.POINTER(C.c_longlong)
        self._check(self._L.bl_greedy_walks(self._ctx, off.ctypes.data_as(llp), None, None, 0, C.byref(total)))
        src = np.zeros(max(total.value, 1), np.int32)
        cnt = np.zeros(max(total.value, 1), np.int32)
        self._check(self._L.bl_greedy_walks(self._ctx, off.ctypes.data_as(llp), _ip(src), _ip(cnt), total.value,
                                            C.byref(total)))
        return off, src[:total.value], cnt[:total.value]

    def barnes_hut_iteration(self, batch: int, theta: float, step: float) -> float:
        e = C.c_double()
        self._check(self._L.bl_barnes_hut_iteration(self._ctx, batch, theta, step, C.byref(e)))
        return e.value

    def morton_order(self):
        frame = np.zeros(3)
        keys = np.zeros(self.n, np.uint64)
        perm = np.zeros(self.n, np.int32)
        self._check(self._L.bl_morton_order(self._ctx, _dp(frame), keys.ctypes.data_as(C.POINTER(C.c_ulonglong)),
                                            _ip(perm)))
        return frame, keys, perm

    def quadtree(self) -> dict:
        cap = 2 * self.n + 8
        lo, hi, dep, nc = (np.zeros(cap, np.int32) for _ in range(4))
        cen = np.zeros(2 * cap)
        m = self._L.bl_quadtree(self._ctx, cap, _ip(lo), _ip(hi), _ip(dep), _ip(nc), _dp(cen))
        if m < 0:
            self._check(m)
        return dict(lo=lo[:m], hi=hi[:m], depth=dep[:m], nchild=nc[:m], centroid=cen[: 2 * m].reshape(m, 2))

    def bh_repulsion(self, theta: float):
        out = np.zeros((self.n, 2))
        st = (C.c_longlong * 2)()
        self._check(self._L.bl_bh_repulsion(self._ctx, theta, _dp(out), st))
        return out, (int(st[0]), int(st[1]))

    def run_resident(self, algo: int, iterations: int, batch: int = 256, theta: float = 1.2,
                     step: float = 1.0, want_energy: bool = True):
        """Device-resident iterations; the last iteration's energy (None when
        want_energy is False, algo 4 only: then no energy is computed)."""
        e = C.c_double()
        self._check(self._L.bl_run_resident(self._ctx, algo, iterations, batch, theta, step,
                                            C.byref(e) if want_energy else None))
        return e.value if want_energy else None

    def last_run_ms(self) -> float:
        """CUDA-event device time of the last run_resident call."""
        ms = C.c_double()
        self._check(self._L.bl_last_run_ms(self._ctx, C.byref(ms)))
        return ms.value

    def set_coordinates_ptr(self, ptr: int):
        """bl_set_coordinates from a raw host pointer (e.g. pinned memory)."""
        self._check(self._L.bl_set_coordinates(self._ctx, C.cast(ptr, C.POINTER(C.c_double)), self.n))

    def get_coordinates_ptr(self, ptr: int):
        self._check(self._L.bl_get_coordinates(self._ctx, C.cast(ptr, C.POINTER(C.c_double)), self.n))

    def set_graph_mode(self, enabled: bool):
        self._check(self._L.bl_set_graph_mode(self._ctx, 1 if enabled else 0))

    def kernel_time(self, kernel: str | None = None):
        ms = (C.c_double * 2)()
        self._check(self._L.bl_last_kernel_time(self._ctx, kernel.encode() if kernel else None, ms))
        return ms[0], int(ms[1])

    def kernel_launches(self) -> int:
        return int(self._L.bl_kernel_launches(self._ctx))

    def learnedInit(self, params, scale_model, seed: int = 1):
        """Coordinates predicted by the learned initializer (bl_learned_init)."""
        p = np.ascontiguousarray(params, np.float32)
        sm = np.ascontiguousarray(scale_model, np.float64)
        self._check(self._L.bl_learned_init(self._ctx, _fp(p), _dp(sm), seed))

    def learnedLayout(self, params, scale_model, max_iterations: int, target_energy: float, batch: int = 256,
                      theta: float = 1.2, step0: float = 0.3, seed: int = 1) -> dict:
        """bl_learned_layout: learned start + Barnes-Hut until target_energy (greedy fallback)."""
        p = np.ascontiguousarray(params, np.float32)
        sm = np.ascontiguousarray(scale_model, np.float64)
        o = (C.c_double * 5)()
        self._check(self._L.bl_learned_layout(self._ctx, _fp(p), _dp(sm), seed, max_iterations, batch, theta,
                                              target_energy, step0, o))
        return dict(energy=o[0], seconds=o[1], iterations=int(o[2]), fell_back=bool(o[3]), init_seconds=o[4])


class BatchedLayout:
    """Many independent graphs laid out by one persistent launch (no
    counterpart in the reference, which runs one graph per process).

    graphs: sequence of (rowptr, colids) CSR pairs with local vertex ids;
    algo: per-graph algorithm (2, 3, 8 minibatch or 4 Barnes-Hut), or one int
    for all; xy: per-graph (n, 2) starting coordinates."""

    def __init__(self, graphs, algo, xy, device: int = 0):
        L = load()
        self._L = L
        ctx = L.bl_batch_create(device)
        if not ctx:
            raise BatchLayoutError(-2, "bl_batch_create failed")
        self._ctx = ctx
        G = len(graphs)
        sizes = np.array([len(rp) - 1 for rp, _ in graphs], np.int64)
        self.vertex_offset = np.zeros(G + 1, np.int32)
        self.vertex_offset[1:] = np.cumsum(sizes)
        self.edge_offset = np.zeros(G + 1, np.int64)
        self.edge_offset[1:] = np.cumsum([len(ci) for _, ci in graphs])
        self.rowptr = np.ascontiguousarray(np.concatenate([np.asarray(rp, np.int32) for rp, _ in graphs]))
        self.colids = np.ascontiguousarray(
            np.concatenate([np.asarray(ci, np.int32) for _, ci in graphs] + [np.zeros(1, np.int32)]))
        self.algo = np.ascontiguousarray(np.broadcast_to(np.asarray(algo, np.int32), (G,)).copy())
        self.xy0 = np.ascontiguousarray(np.concatenate([np.asarray(x, np.float64).reshape(-1, 2) for x in xy]))
        self.sizes = sizes
        self._check(L.bl_batched_prepare(ctx, G, _ip(self.vertex_offset),
                                         self.edge_offset.ctypes.data_as(C.POINTER(C.c_longlong)),
                                         _ip(self.rowptr), _ip(self.colids), _ip(self.algo), _dp(self.xy0)))

    def _check(self, rc: int):
        if rc != 0:
            raise BatchLayoutError(rc, self._L.bl_last_error(self._ctx).decode())

    def run(self, iterations: int, batch: int = 256, theta: float = 1.2, weight: float = 1.0) -> float:
        """Lay out every graph; returns the device seconds of the run."""
        secs = C.c_double()
        self._check(self._L.bl_batched_run(self._ctx, iterations, batch, theta, weight, C.byref(secs)))
        return secs.value

    def result(self):
        """-> (list of per-graph (n, 2) coordinates, per-graph energies)."""
        xy = np.zeros((int(self.vertex_offset[-1]), 2))
        e = np.zeros(len(self.sizes))
        self._check(self._L.bl_batched_result(self._ctx, _dp(xy), _dp(e)))
        vo = self.vertex_offset
        return [xy[vo[g]:vo[g + 1]] for g in range(len(self.sizes))], e

    def parts(self):
        """Source ranges per target chosen for minibatch graphs (< 512, < 2048, >= 2048 vertices)."""
        out = np.zeros(3, np.int32)
        self._check(self._L.bl_batched_parts(self._ctx, _ip(out)))
        return out

    def graph_cycles(self) -> np.ndarray:
        """SM cycles the block spent on each graph in the last run."""
        out = np.zeros(len(self.sizes), np.uint64)
        self._check(self._L.bl_batched_graph_cycles(self._ctx, out.ctypes.data_as(C.POINTER(C.c_ulonglong))))
        return out

    def set_parts(self, parts3):
        a = np.ascontiguousarray(parts3, np.int32)
        self._check(self._L.bl_batched_set_parts(self._ctx, _ip(a)))

    def kernel_launches(self) -> int:
        return int(self._L.bl_kernel_launches(self._ctx))

    def learnedInit(self, params, scale_model, seed: int = 1):
        """Coordinates predicted by the learned initializer (bl_learned_init)."""
        p = np.ascontiguousarray(params, np.float32)
        sm = np.ascontiguousarray(scale_model, np.float64)
        self._check(self._L.bl_learned_init(self._ctx, _fp(p), _dp(sm), seed))

    def learnedLayout(self, params, scale_model, max_iterations: int, target_energy: float, batch: int = 256,
                      theta: float = 1.2, step0: float = 0.3, seed: int = 1) -> dict:
        """bl_learned_layout: learned start + Barnes-Hut until target_energy (greedy fallback)."""
        p = np.ascontiguousarray(params, np.float32)
        sm = np.ascontiguousarray(scale_model, np.float64)
        o = (C.c_double * 5)()
        self._check(self._L.bl_learned_layout(self._ctx, _fp(p), _dp(sm), seed, max_iterations, batch, theta,
                                              target_energy, step0, o))
        return dict(energy=o[0], seconds=o[1], iterations=int(o[2]), fell_back=bool(o[3]), init_seconds=o[4])

    def close(self):
        if getattr(self, "_ctx", None):
            self._L.bl_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


MPNN_PARAMS = 18754
MPNN_FEATURES = 16


def _fp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Mpnn:
    """The learned initializer's network on the GPU (bl_mpnn_*)."""

    def __init__(self, params=None, device: int = 0):
        L = load()
        self._L = L
        ctx = L.bl_batch_create(device)
        if not ctx:
            raise BatchLayoutError(-2, "bl_batch_create failed")
        self._ctx = ctx
        if params is not None:
            self.set_params(params)

    def _check(self, rc: int):
        if rc != 0:
            raise BatchLayoutError(rc, self._L.bl_last_error(self._ctx).decode())

    def set_params(self, params):
        p = np.ascontiguousarray(params, np.float32)
        assert p.shape == (MPNN_PARAMS,)
        self._check(self._L.bl_mpnn_set_params(self._ctx, _fp(p)))

    def get_params(self) -> np.ndarray:
        p = np.zeros(MPNN_PARAMS, np.float32)
        self._check(self._L.bl_mpnn_get_params(self._ctx, _fp(p)))
        return p

    def run(self, rowptr, colids, features, target=None, vweight=None, want_h=False):
        """-> dict(xy, h (3, n, 64) BF16 bits or None, loss, grad)."""
        rp = np.ascontiguousarray(rowptr, np.int32)
        ci = np.ascontiguousarray(colids, np.int32) if len(colids) else np.zeros(1, np.int32)
        n = rp.shape[0] - 1
        f = np.ascontiguousarray(features, np.float32).reshape(n, MPNN_FEATURES)
        xy = np.zeros((n, 2), np.float32)
        h = np.zeros((3, n, 64), np.uint16) if want_h else None
        loss = C.c_double()
        grad = np.zeros(MPNN_PARAMS, np.float32)
        t = np.ascontiguousarray(target, np.float32).reshape(n, 2) if target is not None else None
        w = np.ascontiguousarray(vweight, np.float32) if vweight is not None else None
        self._check(self._L.bl_mpnn_run(self._ctx, n, _ip(rp), _ip(ci), _fp(f), _fp(t) if t is not None else None,
                                        _fp(w) if w is not None else None, _fp(xy),
                                        h.ctypes.data_as(C.POINTER(C.c_ushort)) if h is not None else None,
                                        C.byref(loss), _fp(grad)))
        return dict(xy=xy, h=h, loss=loss.value if t is not None else None, grad=grad if t is not None else None)

    def train(self, graphs, layouts, epochs: int, lr: float = 3e-3, seed: int = 1):
        """bl_learned_train on [(rowptr, colids)] and their (n, 2) target layouts;
        the context's parameters are the start.  -> (params, scale_model, loss history)."""
        G = len(graphs)
        vo = np.zeros(G + 1, np.int32)
        vo[1:] = np.cumsum([len(rp) - 1 for rp, _ in graphs])
        eo = np.zeros(G + 1, np.int64)
        eo[1:] = np.cumsum([len(ci) for _, ci in graphs])
        rp = np.ascontiguousarray(np.concatenate([np.asarray(r, np.int32) for r, _ in graphs]))
        ci = np.ascontiguousarray(np.concatenate([np.asarray(c, np.int32) for _, c in graphs] + [np.zeros(1, np.int32)]))
        lay = np.ascontiguousarray(np.concatenate([np.asarray(x, np.float64).reshape(-1, 2) for x in layouts]))
        params = self.get_params()
        sm = np.zeros(3)
        hist = np.zeros(max(epochs, 1))
        self._check(self._L.bl_learned_train(self._ctx, G, _ip(vo), eo.ctypes.data_as(C.POINTER(C.c_longlong)),
                                             _ip(rp), _ip(ci), _dp(lay), epochs, lr, seed, _fp(params), _dp(sm),
                                             _dp(hist)))
        return params, sm, hist[:epochs]

    def features(self, rowptr, colids, seed: int = 1, pivots=None):
        """-> (features (n, 16) float32, hop distances (n, 16) uint16, pivots (16,))."""
        rp = np.ascontiguousarray(rowptr, np.int32)
        ci = np.ascontiguousarray(colids, np.int32) if len(colids) else np.zeros(1, np.int32)
        n = rp.shape[0] - 1
        f = np.zeros((n, MPNN_FEATURES), np.float32)
        d = np.zeros((n, 16), np.uint16)
        pv = np.zeros(16, np.int32)
        pin = np.ascontiguousarray(pivots, np.int32) if pivots is not None else None
        self._check(self._L.bl_learned_features(self._ctx, n, _ip(rp), _ip(ci), seed,
                                                _ip(pin) if pin is not None else None, _fp(f),
                                                d.ctypes.data_as(C.POINTER(C.c_ushort)), _ip(pv)))
        return f, d, pv

    def close(self):
        if getattr(self, "_ctx", None):
            self._L.bl_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
