"""Failure paths on the GPU that fault nothing.

The tensor-core kernels bound every mbarrier wait; on expiry they raise a
device-side flag, unwind and return, and the call reports
MIDAS_ERR_DEVICE_TIMEOUT.  A test-only kernel makes such a wait run out (an
mbarrier that nothing arrives at, a small poll limit, no copy in flight) and the
context must stay usable afterwards.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_expires_and_reports_timeout(gpulib):
    from midas_gb300.solver import Context
    ctx = Context()
    expired = ctypes.c_int(-1)
    st = gpulib.midas_gpu_wait_selftest(ctx.h, 4096, ctypes.byref(expired))
    assert st == 7, gpulib.midas_gpu_last_error(ctx.h)   # MIDAS_ERR_DEVICE_TIMEOUT
    assert expired.value == 1
    assert b"bounded device wait expired" in gpulib.midas_gpu_last_error(ctx.h)
    # the flag was cleared and the context still solves
    rng = np.random.default_rng(0)
    A = np.eye(96) * 2.0 + 0.1 * (rng.standard_normal((96, 96)) + 1j * rng.standard_normal((96, 96))) / 10
    B = rng.standard_normal((96, 2)) + 0j
    X = ctx.dense_solve(A, B)
    assert np.linalg.norm(A @ X - B) / np.linalg.norm(B) < 1e-12
    assert ctx.gemm_selftest() == "tcgen05"
    ctx.close()


def test_wait_selftest_rejects_bad_limits(gpulib):
    from midas_gb300.solver import Context
    ctx = Context()
    e = ctypes.c_int(0)
    assert gpulib.midas_gpu_wait_selftest(ctx.h, 0, ctypes.byref(e)) == 1
    assert gpulib.midas_gpu_wait_selftest(ctx.h, 1 << 21, ctypes.byref(e)) == 1
    ctx.close()
