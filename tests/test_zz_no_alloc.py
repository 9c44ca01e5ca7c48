"""The allocation-free dense solve, through the C ABI.

midas_gpu_dense_solve_noalloc() serves callers that cannot call cudaMalloc (code
inside a CUDA-graph capture, plug-ins whose host owns all device memory): its
scratch is a static device array inside the library.  Its answers must match
the regular midas_gpu_dense_solve() on consecutive calls, whatever the previous
call left in the shared array.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _system(n, nrhs, seed):
    rng = np.random.default_rng(seed)
    A = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * (0.4 / np.sqrt(n))
    A += np.eye(n) * (1.5 + 0.3j)
    B = rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs))
    return np.asfortranarray(A), np.asfortranarray(B)


def _noalloc(L, A, B):
    X = np.array(B, dtype=np.complex128, order="F", copy=True)
    berr = ctypes.c_double(-1.0)
    st = L.midas_gpu_dense_solve_noalloc(0, None, A.shape[0], B.shape[1], A.ctypes.data, X.ctypes.data,
                                         ctypes.byref(berr))
    return st, X, berr.value


def test_noalloc_matches_dense_solve_twice(gpulib):
    from midas_gb300.solver import Context
    ctx = Context()
    # calls in a row with different sizes and data: each must not see the previous one's
    # leftovers; (512, 32) is the documented maximum and must fit the static scratch
    for n, nrhs, seed in [(300, 3, 1), (131, 5, 2), (512, 32, 5)]:
        A, B = _system(n, nrhs, seed)
        st, X, berr = _noalloc(gpulib, A, B)
        assert st == 0
        Xr = ctx.dense_solve(A, B)
        assert np.linalg.norm(X - Xr) / np.linalg.norm(Xr) < 1e-12
        assert 0 <= berr <= 1e-13
    ctx.close()


def test_noalloc_rejects_sizes_beyond_the_static_scratch(gpulib):
    A, B = _system(600, 2, 3)
    st, _, _ = _noalloc(gpulib, A, B)
    assert st == 1   # MIDAS_ERR_ARG
    A, B = _system(64, 40, 4)
    st, _, _ = _noalloc(gpulib, A, B)
    assert st == 1
