"""The allocation-free minibatch entry point (bl_minibatch_iteration_noalloc).

It exists for callers that cannot allocate device memory while they run --
memory reserved up front in their own pool, real-time loops that forbid
allocation after start-up, streams owned by another component.  Its scratch is
a fixed device array inside the library; inputs and outputs are the caller's
device buffers.  Here the caller's buffers come from torch, and two
consecutive iterations are checked against bl_minibatch_iteration (the context
path, which allocates its own scratch) on the same graph and start, within the
tolerances of the other parity tests.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

FORCE_TOL = 1e-5


def test_noalloc_matches_context_path_on_two_calls():
    torch = pytest.importorskip("torch")
    import batchlayoutcode_gb300 as B
    from batchlayoutcode_gb300 import _lib

    B.build()
    L = _lib.load()
    z = load_golden("chunglu")  # rows sorted, no duplicates: the cursor lists are the rows
    rp, ci, xy = z["csr_rowptr"], z["csr_colids"], z["init_xy"]
    n = len(rp) - 1
    steps = (1.0, 0.999)

    expected = []
    with B.Algorithms(rp, ci) as a:
        a.nCoordinates = xy
        for step in steps:
            e = a.minibatch_iteration(2, 32, step)
            expected.append((e, a.prevCoordinates, a.nCoordinates))

    dev = torch.device("cuda:0")
    d_rp = torch.from_numpy(np.ascontiguousarray(rp, dtype=np.int32)).to(dev)
    d_ci = torch.from_numpy(np.ascontiguousarray(ci, dtype=np.int32)).to(dev)
    d_xy = torch.from_numpy(np.ascontiguousarray(xy, dtype=np.float32)).to(dev)
    d_f = torch.zeros((n, 2), dtype=torch.float64, device=dev)
    d_e = torch.zeros(n, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream

    got = []
    for step in steps:
        e = C.c_double()
        rc = L.bl_minibatch_iteration_noalloc(n, d_rp.data_ptr(), d_ci.data_ptr(), d_xy.data_ptr(),
                                              d_f.data_ptr(), d_e.data_ptr(), 2, 32, 1.0, step, C.byref(e),
                                              stream)
        assert rc == 0
        got.append((e.value, d_f.cpu().numpy(), d_xy.cpu().numpy().astype(np.float64)))

    for (e, f, x), (er, fr, xr) in zip(got, expected):
        assert abs(e - er) <= 2 * FORCE_TOL * er
        assert np.linalg.norm(f - fr) <= FORCE_TOL * np.linalg.norm(fr)
        assert np.abs(x - xr).max() <= 1e-4
    # per-vertex energies are the caller's output too
    assert np.allclose(d_e.cpu().numpy(), (got[-1][1] ** 2).sum(1), rtol=1e-12, atol=0.0)

    # beyond the fixed scratch: a clear error, nothing launched
    e = C.c_double()
    rc = L.bl_minibatch_iteration_noalloc(n, d_rp.data_ptr(), d_ci.data_ptr(), d_xy.data_ptr(), d_f.data_ptr(),
                                          d_e.data_ptr(), 2, 300, 1.0, 1.0, C.byref(e), stream)
    assert rc == -5  # BL_ERR_TOO_LARGE: batch > 256


def _with_isolated_vertex(rp, ci, at):
    """The same graph with an isolated vertex inserted at id `at` (later ids
    shift by one): its row is empty but a non-empty row follows it."""
    rp = np.asarray(rp, dtype=np.int64)
    ci = np.asarray(ci, dtype=np.int64)
    ci2 = np.where(ci >= at, ci + 1, ci)
    rp2 = np.concatenate([rp[:at + 1], rp[at:]])
    return rp2.astype(np.int32), ci2.astype(np.int32)


def test_noalloc_empty_middle_row_through_matched_lists():
    """A caller hands the no-alloc entry point the lists bl_cursor_neighbours
    builds (not the raw rows): an empty row that is not the last one matches
    the next row's first neighbour, as in the reference's cursor and the
    context path.  Checked on a graph with an isolated vertex in the middle."""
    torch = pytest.importorskip("torch")
    import batchlayoutcode_gb300 as B
    from batchlayoutcode_gb300 import _lib

    B.build()
    L = _lib.load()
    z = load_golden("chunglu")
    at = (len(z["csr_rowptr"]) - 1) // 2
    rp, ci = _with_isolated_vertex(z["csr_rowptr"], z["csr_colids"], at)
    n = len(rp) - 1
    xy = np.insert(z["init_xy"], at, [0.25, -0.5], axis=0)
    mrp, mci = _lib.cursor_neighbours(rp, ci)
    assert mrp[at + 1] - mrp[at] == 1 and mci[mrp[at]] == ci[rp[at]]  # the empty row's one match

    with B.Algorithms(rp, ci) as a:
        a.nCoordinates = xy
        e_ref = a.minibatch_iteration(2, 32, 1.0)
        f_ref, x_ref = a.prevCoordinates, a.nCoordinates

    dev = torch.device("cuda:0")
    d_rp = torch.from_numpy(mrp).to(dev)
    d_ci = torch.from_numpy(mci).to(dev)
    d_xy = torch.from_numpy(np.ascontiguousarray(xy, dtype=np.float32)).to(dev)
    d_f = torch.zeros((n, 2), dtype=torch.float64, device=dev)
    d_e = torch.zeros(n, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    e = C.c_double()
    rc = L.bl_minibatch_iteration_noalloc(n, d_rp.data_ptr(), d_ci.data_ptr(), d_xy.data_ptr(), d_f.data_ptr(),
                                          d_e.data_ptr(), 2, 32, 1.0, 1.0, C.byref(e),
                                          torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    f = d_f.cpu().numpy()
    assert abs(e.value - e_ref) <= 2 * FORCE_TOL * e_ref
    assert np.linalg.norm(f - f_ref) <= FORCE_TOL * np.linalg.norm(f_ref)
    assert np.linalg.norm(f[at] - f_ref[at]) <= 1e-4 * np.linalg.norm(f_ref[at])
    assert np.abs(d_xy.cpu().numpy().astype(np.float64) - x_ref).max() <= 1e-4
