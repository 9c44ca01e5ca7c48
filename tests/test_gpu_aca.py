"""Partial-pivot ACA on the GPU against the oracle's Calcul_MatrixZij_ACA, alone
and inside the CBFM-E ACA driver (Compute_EFields_CBFME_ACA)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _trimer(sc=0.25):
    """Three spheres (diameter 2) at 4 and 4.5 diameters apart, each split into
    two half-sphere blocks: pairs inside one sphere stay dense (rank cap), pairs
    across spheres are low-rank."""
    from midas_gb300 import geometry as G
    s = G.sphere_cells(2.0, sc)
    centers = np.array([[0.0, 0.0, 0.0], [4.0, 0.0, 0.0], [0.0, 4.5, 0.0]])
    xyz = np.concatenate([s + c for c in centers])
    sid = np.repeat(np.arange(3), len(s))
    key = sid * 2 + (xyz[:, 0] > centers[sid, 0]).astype(int)
    perm = np.argsort(key, kind="stable")
    xyz = np.ascontiguousarray(xyz[perm])
    offs = np.concatenate([[0], np.cumsum(np.bincount(key))]).astype(np.int32)
    ext = G.extend_blocks(xyz, offs, sc, sc)
    return xyz, sc, offs, ext


@pytest.mark.parametrize("fill", ["faithful", "fast"])
@pytest.mark.parametrize("pair", [(0, 2), (4, 1), (0, 1), (5, 3)])
def test_aca_pair_matches_oracle(gpulib, oracle, pair, fill):
    from midas_gb300 import _lib
    from midas_gb300.solver import Context
    xyz, sc, offs, _ = _trimer()
    eps = np.full(len(xyz), (1.5 + 0.01j) ** 2)
    k0 = 2.0
    i, j = pair
    r0, nr = 3 * int(offs[i]), 3 * int(offs[i + 1] - offs[i])
    c0, nc = 3 * int(offs[j]), 3 * int(offs[j + 1] - offs[j])
    cells = oracle.Cells(xyz, sc, eps, k0)
    ko, Uo, Vo = oracle.aca(cells, r0, nr, c0, nc, eps=oracle.EPS_ACA_DEFAULT, itmax=50)
    mode = _lib.FILL_FAITHFUL if fill == "faithful" else _lib.FILL_FAST
    ctx = Context(fill_mode=mode).set_cells(xyz, sc, eps, k0)
    k, U, V = ctx.aca(r0, nr, c0, nc, eps=oracle.EPS_ACA_DEFAULT, itmax=50)
    assert k == ko, (k, ko)
    kk = min(k, 50)
    # same pivots and the same FP64 residual arithmetic: U and V agree to rounding
    eu = np.linalg.norm(U[:, :kk] - Uo[:, :kk]) / np.linalg.norm(Uo[:, :kk])
    ev = np.linalg.norm(V[:kk, :] - Vo[:kk, :]) / np.linalg.norm(Vo[:kk, :])
    assert eu < 1e-12 and ev < 1e-12, (eu, ev)
    if k < 50:
        Z = oracle.green_partial(cells, np.arange(offs[i], offs[i + 1]), np.arange(offs[j], offs[j + 1]))
        assert np.linalg.norm(U[:, :k] @ V[:k, :] - Z) / np.linalg.norm(Z) < 1e-3
    ctx.close()


def test_aca_rejects_overlapping_blocks(gpulib):
    from midas_gb300._lib import MidasError
    from midas_gb300.solver import Context
    xyz, sc, offs, _ = _trimer()
    ctx = Context().set_cells(xyz, sc, np.full(len(xyz), 2.25 + 0.03j), 2.0)
    with pytest.raises(MidasError) as e:
        ctx.aca(0, 3 * int(offs[1]), 3, 3 * int(offs[1]))
    assert e.value.status == 1
    with pytest.raises(MidasError):
        ctx.aca(0, 3 * int(offs[1]), 3 * int(offs[1]), 3 * int(offs[2] - offs[1]), itmax=129)
    ctx.close()


@pytest.mark.parametrize("fill", ["faithful", "fast"])
def test_cbfm_aca_matches_oracle(gpulib, oracle, fill):
    from midas_gb300 import _lib, geometry as G
    from midas_gb300.solver import Context
    xyz, sc, offs, ext = _trimer()
    eps = np.full(len(xyz), (1.5 + 0.01j) ** 2)
    k0 = 2.0
    th, ph = np.array([90.0, 30.0, 140.0]), np.array([90.0, 10.0, 250.0])
    niws = 91
    cells = oracle.Cells(xyz, sc, eps, k0)
    keep = {}
    ref = oracle.cbfm_solve(cells, oracle.Partition(offs, ext), th, ph, niws, use_aca=True, homog=1, keep=keep)
    far = sum(1 for k in keep["aca_rank"].values() if k < oracle.NB_IT_MAX_DEFAULT)
    assert 0 < far < len(keep["aca_rank"])
    cth, cph = G.transmitters_un(niws)
    mode = _lib.FILL_FAITHFUL if fill == "faithful" else _lib.FILL_FAST
    ctx = Context(fill_mode=mode).set_cells(xyz, sc, eps, k0)
    E, K = ctx.cbfm_solve(offs, ext, cth, cph, th, ph, flags=_lib.CBFM_SR | _lib.CBFM_HOMOG | _lib.CBFM_ACA)
    assert np.array_equal(K, ref["K"]), (K, ref["K"])
    assert ctx.info.n_far_aca == far
    rel = np.linalg.norm(E - ref["E"]) / np.linalg.norm(ref["E"])
    assert rel < 1e-6, rel
    ce, ca = ctx.cext_cabs(th, ph, E)
    ce_o, ca_o = oracle.cext_cabs(cells, th, ph, ref["E"])
    assert np.max(np.abs(ce - ce_o) / np.abs(ce_o)) < 1e-6
    assert np.max(np.abs(ca - ca_o) / np.abs(ca_o)) < 1e-6
    ctx.close()
