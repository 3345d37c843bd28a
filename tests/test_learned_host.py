"""Model files of the learned initializer: the Python writer and the
library's reader agree (host only, no GPU)."""
import ctypes as C
import os

import numpy as np


def test_model_file_round_trip(tmp_path):
    import batchlayoutcode_gb300 as B
    from batchlayoutcode_gb300 import learned as LR
    B.build()
    rng = np.random.default_rng(3)
    p = rng.normal(size=LR.MPNN_PARAMS).astype(np.float32)
    sm = np.array([1.5, -0.25, 3.0])
    path = str(tmp_path / "m.blw")
    LR.save_model(path, p, sm)
    p2, sm2 = LR.load_model(path)
    assert np.array_equal(p, p2) and np.array_equal(sm, sm2)
    L = B.load()
    p3 = np.zeros(LR.MPNN_PARAMS, np.float32)
    sm3 = np.zeros(3)
    rc = L.bl_learned_load_model(path.encode(), p3.ctypes.data_as(C.POINTER(C.c_float)),
                                 sm3.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0
    assert np.array_equal(p, p3) and np.array_equal(sm, sm3)
    bad = str(tmp_path / "bad.blw")
    with open(bad, "wb") as f:
        f.write(b"NOTAMODEL" + bytes(16))
    assert L.bl_learned_load_model(bad.encode(), p3.ctypes.data_as(C.POINTER(C.c_float)),
                                   sm3.ctypes.data_as(C.POINTER(C.c_double))) == -6
    # truncated, and non-finite weights or scales: rejected as not a model
    with open(path, "rb") as f:
        good = f.read()
    with open(bad, "wb") as f:
        f.write(good[:-5])
    assert L.bl_learned_load_model(bad.encode(), p3.ctypes.data_as(C.POINTER(C.c_float)),
                                   sm3.ctypes.data_as(C.POINTER(C.c_double))) == -6
    for pn, smn in ((np.where(np.arange(LR.MPNN_PARAMS) == 17, np.nan, p).astype(np.float32), sm),
                    (p, np.array([1.5, np.inf, 3.0]))):
        LR.save_model(bad, pn, smn)
        assert L.bl_learned_load_model(bad.encode(), p3.ctypes.data_as(C.POINTER(C.c_float)),
                                       sm3.ctypes.data_as(C.POINTER(C.c_double))) == -6


def test_shipped_model_loads():
    from batchlayoutcode_gb300 import learned as LR
    assert os.path.exists(LR.DEFAULT_MODEL)
    p, sm = LR.load_model()
    assert p.shape == (LR.MPNN_PARAMS,) and np.all(np.isfinite(p)) and np.all(np.isfinite(sm))
    assert np.any(p[-130:] != 0)  # a trained readout, not the zero start


def test_training_graphs_are_the_benchmark_mix():
    from batchlayoutcode_gb300 import learned as LR
    gs = LR.training_graphs(6, 200, 2000, seed=5)
    assert len(gs) == 6
    for g in gs:
        assert 16 <= g.n <= 2200
        rows = np.repeat(np.arange(g.n), np.diff(g.rowptr))
        assert np.all(rows != g.colids)  # no self loops
        # symmetric
        a = set(zip(rows.tolist(), g.colids.tolist()))
        assert all((c, r) in a for r, c in a)
