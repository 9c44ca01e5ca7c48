"""The FFT lattice operator (fft.cu) against the dense FP64 MoM matrix.

For cells on one lattice, midas_gpu_lattice_matvec applies the matrix of
compute_Green_s_tr_single_element (src/Compute_EFields_MoM.f90:433-523) as a
zero-padded FFT convolution.  Bar: 1e-13 relative to the dense product formed
with the GPU's FP64 fill (itself parity-tested against the oracle).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _x(N, nrhs, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((N, nrhs)) + 1j * rng.standard_normal((N, nrhs))


@pytest.mark.parametrize("ncell", [1600, 8000])
def test_lattice_matvec_matches_dense_cube(gpulib, ncell):
    from midas_gb300 import workloads as W
    from midas_gb300.solver import Context
    wl = W.mom_c3(n_cells=ncell)
    ctx = Context().set_cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
    N = 3 * ncell
    X = _x(N, 3, 1)
    Y = ctx.lattice_matvec(X)
    # dense rows in chunks (a row subset at the larger size)
    rows = [(0, N)] if N <= 6000 else [(0, 600), (N // 2 - 300, 600), (N - 600, 600)]
    num = den = 0.0
    for r0, nr in rows:
        Zr = ctx.mom_fill(r0, nr, 0, N)
        Yd = Zr @ X
        num += np.linalg.norm(Y[r0:r0 + nr] - Yd) ** 2
        den += np.linalg.norm(Yd) ** 2
    rel = np.sqrt(num / den)
    print(ncell, "rel", rel)
    assert rel < 1e-13, rel
    ctx.close()


def test_lattice_matvec_sphere_and_new_cells(gpulib, oracle):
    """A sphere (cells inside a ball), then new cells on the same context: the
    spectra follow the cells."""
    from midas_gb300.solver import Context
    ctx = Context()
    for sc, m in ((0.2, 1.5 + 0.01j), (0.25, 1.3 + 0.1j)):
        xyz = oracle.sphere_cells(2.0, sc)
        ctx.set_cells(xyz, sc, m * m, 2.0)
        N = 3 * len(xyz)
        X = _x(N, 2, 2)
        Y = ctx.lattice_matvec(X)
        Yd = ctx.mom_fill() @ X
        rel = np.linalg.norm(Y - Yd) / np.linalg.norm(Yd)
        assert rel < 1e-13, rel
    ctx.close()


def test_lattice_matvec_rejects_off_lattice_cells(gpulib):
    from midas_gb300._lib import MidasError
    from midas_gb300.solver import Context
    rng = np.random.default_rng(3)
    xyz = rng.uniform(-1, 1, (50, 3))
    ctx = Context().set_cells(xyz, 0.1, 2.0 + 0.1j, 2.0)
    with pytest.raises(MidasError) as e:
        ctx.lattice_matvec(_x(150, 1, 0))
    assert e.value.status == 8   # MIDAS_ERR_UNSUPPORTED
    ctx.close()
