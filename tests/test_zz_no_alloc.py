"""The allocation-free dense solve, through the C ABI.

midas_gpu_dense_solve_noalloc() serves callers that cannot call cudaMalloc:
plug-ins whose host application owns and caps all device memory, and paths
where an allocation could block.  Its scratch is a static device array inside
the library.  Its answers must match the regular midas_gpu_dense_solve() on
consecutive calls, whatever the previous call left in the shared array, and the
device's free memory must not move across its calls.  This file is collected
last on purpose.
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


def _noalloc(L, A, B, stream=None):
    X = np.array(B, dtype=np.complex128, order="F", copy=True)
    berr = ctypes.c_double(-1.0)
    st = L.midas_gpu_dense_solve_noalloc(0, stream, A.shape[0], B.shape[1], A.ctypes.data, X.ctypes.data,
                                         ctypes.byref(berr))
    return st, X, berr.value


def _free_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info(0)[0]


def test_noalloc_matches_dense_solve_twice(gpulib):
    from midas_gb300.solver import Context
    ctx = Context()
    # calls in a row with different sizes and data: each must not see the previous one's
    # leftovers; (512, 32) is the documented maximum and must fit the static scratch
    cases = [(300, 3, 1), (131, 5, 2), (512, 32, 5), (512, 32, 6)]
    refs = []
    for n, nrhs, seed in cases:
        A, B = _system(n, nrhs, seed)
        refs.append(ctx.dense_solve(A, B))
    ctx.close()
    # one call first, so that lazily loaded kernels are resident before free memory is read
    A, B = _system(64, 1, 9)
    assert _noalloc(gpulib, A, B)[0] == 0
    free0 = _free_bytes()
    for (n, nrhs, seed), Xr in zip(cases, refs):
        A, B = _system(n, nrhs, seed)
        st, X, berr = _noalloc(gpulib, A, B)
        assert st == 0   # MIDAS_ERR_ALLOC (3) would mean a slot was too small for a request
        assert np.linalg.norm(X - Xr) / np.linalg.norm(Xr) < 1e-12
        assert 0 <= berr <= 1e-13
    assert _free_bytes() == free0, "device free memory changed across the allocation-free calls"


def test_noalloc_rejects_sizes_beyond_the_static_scratch(gpulib):
    A, B = _system(600, 2, 3)
    st, _, _ = _noalloc(gpulib, A, B)
    assert st == 1   # MIDAS_ERR_ARG
    A, B = _system(64, 40, 4)
    st, _, _ = _noalloc(gpulib, A, B)
    assert st == 1


def test_noalloc_refuses_a_capturing_stream(gpulib):
    """The solve synchronises and reads convergence on the host, so a call on a stream
    under capture is refused before it issues work; the capture stays valid."""
    import torch
    A, B = _system(64, 2, 7)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    buf = torch.zeros(4, device="cuda")
    with torch.cuda.stream(s):
        g.capture_begin(capture_error_mode="relaxed")
        try:
            buf.add_(1.0)
            st, X, _ = _noalloc(gpulib, A, B, stream=s.cuda_stream)
        finally:
            g.capture_end()
    assert st == 1   # MIDAS_ERR_ARG
    assert np.array_equal(X, B)   # untouched
    g.replay()
    torch.cuda.synchronize()
    assert float(buf.sum()) == 4.0
