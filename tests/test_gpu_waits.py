"""Bounded device waits end in an error code, not a hang.

Every spin-wait in the layout kernels has a limit on %globaltimer: the grid
barrier of the cooperative kernels (2 s) and the mbarrier wait for
tensor-core completion (1 s).  bl_wait_selftest runs those same waits with
their arrival withheld (a flag nothing sets), so the wait runs to its limit;
the kernel records the site and returns, and the call must report
BL_ERR_DEVICE_TIMEOUT with the reason, after about the limit, with the
context left usable (the next layout call gives the bits a fresh context
gives).  With the arrival made the same call returns BL_OK at once.
"""
import time

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

BL_ERR_DEVICE_TIMEOUT = -3


@pytest.fixture(scope="module")
def B():
    import batchlayoutcode_gb300 as B
    B.build()
    return B


@pytest.mark.parametrize("site,limit_s,reason", [(0, 2.0, "grid barrier timed out"),
                                                 (1, 1.0, "tensor-core MMA completion wait timed out")])
def test_withheld_arrival_runs_out_into_device_timeout(B, site, limit_s, reason):
    z = load_golden("grid12")
    rp, ci, xy = z["csr_rowptr"], z["csr_colids"], z["init_xy"]
    with B.Algorithms(rp, ci) as a:
        L, ctx = a._L, a._ctx
        t0 = time.perf_counter()
        assert L.bl_wait_selftest(ctx, site, 1) == 0
        assert time.perf_counter() - t0 < 0.5 * limit_s
        t0 = time.perf_counter()
        rc = L.bl_wait_selftest(ctx, site, 0)
        dt = time.perf_counter() - t0
        assert rc == BL_ERR_DEVICE_TIMEOUT
        assert reason in L.bl_last_error(ctx).decode()
        assert 0.9 * limit_s <= dt <= limit_s + 10.0
        # the context is still usable and the recorded error is cleared
        assert L.bl_wait_selftest(ctx, site, 1) == 0
        a.nCoordinates = xy
        e = a.minibatch_iteration(2, 32, 1.0)
        got = a.nCoordinates
    with B.Algorithms(rp, ci) as a:
        a.nCoordinates = xy
        assert a.minibatch_iteration(2, 32, 1.0) == e
        assert np.array_equal(a.nCoordinates, got)


def test_wait_selftest_rejects_unknown_site(B):
    z = load_golden("grid12")
    with B.Algorithms(z["csr_rowptr"], z["csr_colids"]) as a:
        assert a._L.bl_wait_selftest(a._ctx, 7, 1) == -1
