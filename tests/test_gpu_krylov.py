"""GMRES on the FFT lattice operator against the dense solve (its judge).

midas_gpu_gmres_solve solves the MoM system of Compute_EFields_MoM
(src/Compute_EFields_MoM.f90:153-198) for lattice cells without forming Z, and
accepts convergence only on the true FP64 residual.  The dense mixed solve
(LU + refinement to 1e-13) is the reference answer.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cube(gpulib):
    from midas_gb300 import workloads as W
    from midas_gb300.solver import Context
    wl = W.mom_c3(n_cells=1600, ndir=3)
    ctx = Context().set_cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
    Ed = ctx.mom_solve(wl["th"], wl["ph"])
    yield ctx, wl, Ed
    ctx.close()


@pytest.mark.parametrize("jacobi", [False, True])
def test_gmres_matches_dense_solve(cube, jacobi):
    ctx, wl, Ed = cube
    E, it, rel = ctx.gmres_solve(wl["th"], wl["ph"], restart=50, maxit=1000, tol=1e-10, jacobi=jacobi)
    assert rel <= 1e-10 and it > 0
    err = np.linalg.norm(E - Ed) / np.linalg.norm(Ed)
    print("gmres jacobi", jacobi, "iterations", it, "true rel residual", rel, "field error", err)
    assert err < 1e-8, err


def test_gmres_initial_guess_saves_iterations(cube):
    """A good initial guess (the dense answer perturbed by 1e-3) needs fewer steps than zero;
    the exact answer needs none."""
    ctx, wl, Ed = cube
    _, it0, _ = ctx.gmres_solve(wl["th"], wl["ph"], tol=1e-10, maxit=1000)
    rng = np.random.default_rng(0)
    guess = Ed * (1 + 1e-3 * rng.standard_normal(Ed.shape))
    E1, it1, rel1 = ctx.gmres_solve(wl["th"], wl["ph"], E0=guess, tol=1e-10, maxit=1000)
    assert rel1 <= 1e-10 and it1 < it0, (it0, it1)
    _, it2, rel2 = ctx.gmres_solve(wl["th"], wl["ph"], E0=Ed, tol=1e-8, maxit=1000)
    assert it2 == 0 and rel2 <= 1e-8


def test_gmres_reports_non_convergence(cube):
    ctx, wl, _ = cube
    from midas_gb300._lib import MidasError
    with pytest.raises(MidasError) as e:
        ctx.gmres_solve(wl["th"], wl["ph"], tol=1e-12, maxit=3)
    assert e.value.status == 5   # MIDAS_ERR_NOT_CONVERGED
    E, it, rel = ctx.gmres_solve(wl["th"], wl["ph"], tol=1e-12, maxit=3, check=False)
    assert it == 3 and rel > 1e-12
