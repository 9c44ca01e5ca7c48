"""Physics anchors of the oracle (the reference's own validation is a Mie comparison)."""
import numpy as np
import pytest

from mie import mie_q


def test_mie_anchor_small_sphere(oracle):
    m, a, k0, sc = 1.5 + 0.01j, 1.0, 2.0, 0.2
    xyz = oracle.sphere_cells(2 * a, sc)
    c = oracle.Cells(xyz, sc, m * m, k0)
    res = oracle.mom_solve(c, [90.0], [90.0])
    aeq = (3 * c.n * sc ** 3 / (4 * np.pi)) ** (1 / 3)
    qe_mie, qs_mie = mie_q(m, k0 * aeq)
    qext = res["cext"][0] / (np.pi * aeq ** 2)
    qabs = res["cabs"][0] / (np.pi * aeq ** 2)
    assert abs(qext - qe_mie) / qe_mie < 0.03
    assert abs(qabs - (qe_mie - qs_mie)) / (qe_mie - qs_mie) < 0.05


def test_homogeneous_reciprocity(oracle):
    m = 1.3 + 0.05j
    c = oracle.Cells(oracle.sphere_cells(2.0, 0.4), 0.4, m * m, 2.5)
    Z = oracle.mom_fill(c)
    assert np.array_equal(Z, Z.T)
    Z4 = oracle.green_partial(c, np.arange(c.n), np.arange(c.n))
    assert np.array_equal(Z4, Z4.T)
    assert np.max(np.abs(Z4 - Z)) / np.max(np.abs(Z)) < 1e-6


def test_sr_dense_consistent(oracle):
    m = 1.5 + 0.01j
    c = oracle.Cells(oracle.sphere_cells(2.0, 0.25), 0.25, m * m, 2.0)
    idx = np.arange(c.n, dtype=np.int32)
    Zfull = oracle.green_partial(c, idx, idx)
    for homog in (0, 1):
        Z, nnz, fn = oracle.sr_dense(c, idx, 1e3, homog)
        kept = Z != 0
        assert np.array_equal(Z[kept], Zfull[kept])
        if homog == 0:
            assert nnz == np.count_nonzero(kept)
            assert abs(fn - np.linalg.norm(Z)) / fn < 1e-6
        assert np.array_equal(Z, Z.T)


def test_aca_reproduces_far_block(oracle):
    """Two well-separated clusters: ACA reaches eps at a rank far below the block size."""
    m = 1.5 + 0.01j
    xyz = oracle.sphere_cells(2.0, 0.2)
    n = len(xyz)
    c = oracle.Cells(np.concatenate([xyz, xyz + np.array([6.0, 0.0, 0.0])]), 0.2, m * m, 2.0)
    k, U, V = oracle.aca(c, 0, 3 * n, 3 * n, 3 * n, eps=1e-4, itmax=50)
    assert 2 <= k < 50
    Z = oracle.green_partial(c, np.arange(n), np.arange(n, 2 * n))
    A = U[:, :k] @ V[:k, :]
    assert np.linalg.norm(A - Z) / np.linalg.norm(Z) < 3e-4


def test_cbfm_close_to_mom(oracle):
    from midas_gb300 import geometry as G
    m = 1.5 + 0.01j
    sc = 0.2
    xyz = G.sphere_cells(2.0, sc)
    perm, offs = G.box_partition(xyz, 2, 1, 1)
    xyz = xyz[perm]
    part = oracle.Partition(offs, G.extend_blocks(xyz, offs, sc, sc))
    c = oracle.Cells(xyz, sc, m * m, 2.0)
    r = oracle.cbfm_solve(c, part, [90.0], [90.0], niws=190, homog=1)
    e = oracle.mom_solve(c, [90.0], [90.0])["E"]
    assert np.linalg.norm(r["E"] - e) / np.linalg.norm(e) < 0.05
