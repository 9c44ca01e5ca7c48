"""Tensor-core GEMM engine, dense mixed-precision solve and the MoM path on the GPU."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpulib):
    from midas_gb300.solver import Context
    c = Context()
    yield c
    c.close()


def test_gemm_engine_selftest(ctx):
    assert ctx.gemm_selftest() == "tcgen05"


@pytest.mark.parametrize("n,nrhs", [(64, 1), (200, 3), (517, 8)])
def test_dense_solve_mixed(ctx, n, nrhs):
    rng = np.random.default_rng(n)
    A = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n) * 0.4
    A += np.eye(n) * (1.5 + 0.3j)
    B = rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs))
    X = ctx.dense_solve(A, B)
    Xr = np.linalg.solve(A, B)
    assert np.linalg.norm(X - Xr) / np.linalg.norm(Xr) < 1e-12
    assert ctx.info.backward_error <= 1e-13 and ctx.info.ir_iters >= 1


def _true_backward_error(A, X, B):
    """max over columns of |B - A X|_inf / (|A|_inf |X|_inf + |B|_inf), FP64 on the host,
    with the solver's vector norm max(|Re|, |Im|)."""
    R = B - A @ X
    vn = lambda V: np.maximum(np.abs(V.real), np.abs(V.imag)).max(axis=0)
    an = np.abs(A).sum(axis=1).max()
    return float(np.max(vn(R) / (an * vn(X) + vn(B))))


@pytest.mark.parametrize("n,nrhs,d,c", [(1000, 5, 1.5 + 0.3j, 0.4), (1000, 20, 1.5 + 0.3j, 0.4),
                                         (640, 70, 1.0, 0.9)])
def test_dense_solve_true_backward_error(ctx, n, nrhs, d, c):
    """The refinement's residuals (FP32 first residual, double-float full residuals, FP32
    updates r -= Z d) track the true FP64 residual: the backward error of the returned x,
    measured on the host in FP64, is within the 1e-13 tolerance.  Both residual tile
    shapes (<= 16 and > 16 right-hand sides), and a system d I + c G / sqrt(n) with its
    eigenvalues out to 0.1 of the origin (c = 0.9), where the TF32 factors gain about a
    digit per step and several double-float residuals run before the FP32 updates."""
    rng = np.random.default_rng(n + nrhs)
    A = c * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(2 * n) + d * np.eye(n)
    B = rng.standard_normal((n, nrhs)) + 1j * rng.standard_normal((n, nrhs))
    X = ctx.dense_solve(A, B)
    be = _true_backward_error(A, X, B)
    assert be <= 2e-13, (be, ctx.info.backward_error, ctx.info.ir_iters)
    assert ctx.info.backward_error <= 1e-13
    Xr = np.linalg.solve(A, B)
    assert np.linalg.norm(X - Xr) / np.linalg.norm(Xr) < 1e-11


def test_dense_solve_torch_reference(ctx):
    """The LU/IR result against a plain PyTorch reference solve of the same system."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    n = 384
    A = np.eye(n) * 2 + 0.3 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n)
    B = rng.standard_normal((n, 2)) + 1j * rng.standard_normal((n, 2))
    X = ctx.dense_solve(A, B)
    Xt = torch.linalg.solve(torch.from_numpy(A), torch.from_numpy(B)).numpy()
    assert np.linalg.norm(X - Xt) / np.linalg.norm(Xt) < 1e-12


@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_mom_solve_matches_oracle(gpulib, oracle, mode):
    from midas_gb300 import _lib
    from midas_gb300.solver import Context, compute_efields_mom
    m, sc, k0 = 1.5 + 0.01j, 0.2, 2.0
    xyz = oracle.sphere_cells(2.0, sc)
    cells = oracle.Cells(xyz, sc, m * m, k0)
    th, ph = [90.0, 40.0], [90.0, 200.0]
    rth = np.linspace(0, 180, 19)
    rph = np.zeros_like(rth) + 90.0
    ref = oracle.mom_solve(cells, th, ph, rth, rph)
    sm = _lib.SOLVE_MIXED if mode == "mixed" else _lib.SOLVE_FP64
    c = Context(solve_mode=sm).set_cells(xyz, sc, m * m, k0)
    E, S, ce, ca = compute_efields_mom(c, th, ph, rth, rph)
    rel = np.linalg.norm(E - ref["E"]) / np.linalg.norm(ref["E"])
    assert rel < 1e-10, rel
    assert np.max(np.abs(ce - ref["cext"]) / np.abs(ref["cext"])) < 1e-10
    assert np.max(np.abs(ca - ref["cabs"]) / np.abs(ref["cabs"])) < 1e-10
    assert np.max(np.abs(S - ref["S"])) / np.max(np.abs(ref["S"])) < 1e-10
    if mode == "mixed":
        assert c.info.backward_error <= 1e-13
    c.close()


def test_mom_solve_off_lattice_dense_residuals(gpulib, oracle):
    """Cells off any lattice (jittered centroids): the mixed solve refines with the
    dense double-float residuals instead of the FFT lattice operator."""
    from midas_gb300.solver import Context
    m, sc, k0 = 1.5 + 0.01j, 0.2, 2.0
    rng = np.random.default_rng(5)
    xyz = oracle.sphere_cells(2.0, sc)
    xyz = xyz + rng.uniform(-0.01, 0.01, xyz.shape)
    cells = oracle.Cells(xyz, sc, m * m, k0)
    th, ph = [90.0, 40.0], [90.0, 200.0]
    ref = oracle.mom_solve(cells, th, ph)
    c = Context().set_cells(xyz, sc, m * m, k0)
    E = c.mom_solve(th, ph)
    assert np.linalg.norm(E - ref["E"]) / np.linalg.norm(ref["E"]) < 1e-10
    assert c.info.backward_error <= 1e-13
    with pytest.raises(Exception):
        c.lattice_matvec(np.ones((3 * len(xyz), 1), complex))
    c.close()


def test_mom_solve_inhomogeneous_fast_fill(gpulib, oracle):
    from midas_gb300 import _lib, geometry as G
    from midas_gb300.solver import Context
    rng = np.random.default_rng(11)
    xyz = G.cube_cells(9, 0.1)
    eps = rng.uniform(1.5, 3.5, len(xyz)) + 1j * rng.uniform(0, 0.2, len(xyz))
    k0 = 2 * np.pi / (9 * 0.1 / 2)
    cells = oracle.Cells(xyz, 0.1, eps, k0)
    th, ph = [10.0, 70.0, 130.0], [30.0, 200.0, 300.0]
    ref = oracle.mom_solve(cells, th, ph)
    c = Context(fill_mode=_lib.FILL_FAST).set_cells(xyz, 0.1, eps, k0)
    E = c.mom_solve(th, ph)
    assert np.linalg.norm(E - ref["E"]) / np.linalg.norm(ref["E"]) < 1e-10
    c.close()


def test_dense_c3_like_mixed_vs_fp64(gpulib, oracle):
    """The inhomogeneous-cube dense solve (eps' ~ U[1.5,3.5], eps'' ~ U[0,0.2], 64 plane-wave
    right-hand sides) at 1,600 voxels: the mixed TF32 LU + FP64 refinement reaches a backward
    error <= 1e-8 (it goes to ~1e-14) and matches the FP64 LU and the oracle's LAPACK solve."""
    from midas_gb300 import _lib, workloads as W
    from midas_gb300.solver import Context
    wl = W.mom_c3(n_cells=1600, ndir=32)
    cm = Context(fill_mode=_lib.FILL_FAST).set_cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
    Em = cm.mom_solve(wl["th"], wl["ph"])
    assert Em.shape[1] == 64 and cm.info.backward_error <= 1e-8
    cd = Context(solve_mode=_lib.SOLVE_FP64).set_cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
    Ed = cd.mom_solve(wl["th"], wl["ph"])
    assert np.linalg.norm(Em - Ed) / np.linalg.norm(Ed) < 1e-10
    ref = oracle.mom_solve(oracle.Cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"]), wl["th"], wl["ph"])
    assert np.linalg.norm(Em - ref["E"]) / np.linalg.norm(ref["E"]) < 1e-10
    cm.close()
    cd.close()


def test_errors_are_reported(gpulib):
    from midas_gb300._lib import MidasError
    from midas_gb300.solver import Context
    c = Context()
    with pytest.raises(MidasError) as e:
        c.mom_solve([0.0], [0.0])
    assert e.value.status == 6   # MIDAS_ERR_STATE: no cells
    c.set_cells(np.zeros((2, 3)) + [[0, 0, 0], [0.1, 0, 0]], 0.1, 2.0, 1.0)
    with pytest.raises(MidasError) as e:
        c.mom_fill(0, 7, 0, 6)
    assert e.value.status == 1   # block outside the matrix
    c.close()


@pytest.mark.parametrize("m", [7, 64, 182, 380])
def test_heev_jacobi(ctx, m):
    """Graded spectrum (singular values 1 .. 1e-9), as the Gram matrices of the CBF step."""
    rng = np.random.default_rng(m)
    U, _ = np.linalg.qr(rng.standard_normal((3 * m, m)) + 1j * rng.standard_normal((3 * m, m)))
    Q, _ = np.linalg.qr(rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m)))
    X = (U * np.logspace(0, -9, m)) @ Q
    A = X.conj().T @ X
    W, V = ctx.heev(A)
    ref = np.sort(np.linalg.eigvalsh(A))[::-1]
    assert np.all(np.diff(W) <= 0)
    assert np.max(np.abs(W - ref)) <= 1e-13 * ref[0]
    # the range the CBF threshold (sigma ratio >= 1e-4) uses: a backward-stable solver
    # gets these to eps ||A|| / lambda, i.e. 2.2e-8 relative at lambda = 1e-8 ||A||
    sel = ref > 1e-8 * ref[0]
    assert np.max(np.abs(W[sel] - ref[sel]) / ref[sel]) < 4e-8
    assert np.max(np.abs(V.conj().T @ A @ V - np.diag(W))) <= 1e-12 * ref[0]


@pytest.mark.parametrize("m,rank", [(182, 60), (96, 1)])
def test_heev_rank_deficient(ctx, m, rank):
    """Gram matrix of fewer independent solutions than excitations: m - rank eigenvalues at
    the roundoff level (the split test against eps ||T|| deflates them)."""
    rng = np.random.default_rng(m + rank)
    X = rng.standard_normal((3 * m, rank)) + 1j * rng.standard_normal((3 * m, rank))
    X = X @ (rng.standard_normal((rank, m)) + 1j * rng.standard_normal((rank, m)))
    A = X.conj().T @ X
    W, V = ctx.heev(A)
    ref = np.sort(np.linalg.eigvalsh(A))[::-1]
    assert np.all(np.diff(W) <= 0)
    assert np.max(np.abs(W - ref)) <= 1e-13 * ref[0]
    assert np.max(np.abs(V.conj().T @ V - np.eye(m))) <= 1e-12
    assert np.max(np.abs(A @ V[:, :rank] - V[:, :rank] * W[:rank])) <= 1e-12 * ref[0]


@pytest.mark.parametrize("M,N,K", [(130, 65, 828), (300, 40, 2000)])
def test_zgemm_x3_fp32_grade(ctx, M, N, K):
    """Split-TF32 product against FP64: error at the FP32 level, not the TF32 level."""
    rng = np.random.default_rng(K)
    A = rng.standard_normal((M, K)) + 1j * rng.standard_normal((M, K))
    B = rng.standard_normal((K, N)) + 1j * rng.standard_normal((K, N))
    D = ctx.zgemm_x3(A, B)
    ref = A @ B
    scale = np.abs(A) @ np.abs(B)
    err = np.max(np.abs(D - ref) / scale)
    assert err < 2e-7, err   # IEEE FP32 (numpy complex64) reaches ~4e-8 here
