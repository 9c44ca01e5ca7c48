"""Scene preparation on the device against the host restatements.

The sphere voxeliser follows Discretization (src/Discretization.f90:246-310)
and must give the oracle's centroids in the oracle's order; the partition and
the extension (Extend_blocks, src/Extend_blocks.f90:46-151) must give the host
geometry module's permutation, offsets and extension lists exactly.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpulib):
    from midas_gb300.solver import Context
    c = Context()
    yield c
    c.close()


@pytest.mark.parametrize("dm,sc", [(2.0, 0.2), (2.0, 1 / 4.775), (2.0, 0.1), (1.6, 0.16), (2.0, 0.047)])
def test_sphere_voxeliser_matches_oracle(ctx, oracle, dm, sc):
    xyz = ctx.voxelise_sphere(dm, sc)
    ref = oracle.sphere_cells(dm, sc)
    assert xyz.shape == ref.shape and np.array_equal(xyz, ref)


def test_union_of_spheres_matches_host(ctx):
    from midas_gb300 import geometry as G
    for n_mono, seed in ((4, 1), (24, 2), (64, 3)):
        cen = G.fractal_aggregate(n_mono, a=1.0, seed=seed)
        xyz, d = ctx.voxelise_spheres(cen, 1.0, 6)
        ref, dref = G.voxelise_spheres(cen, 1.0, 6)
        assert d == dref and np.array_equal(xyz, ref)


def test_partition_and_extension_match_host(ctx):
    from midas_gb300 import workloads as W, geometry as G
    for builder, nb in ((W.cbfm_c2_small, 2), (W.cbfm_c2, 3)):
        wl = builder()
        xyz0 = wl["xyz"]
        perm, offs = ctx.box_partition(xyz0, nb, nb, nb)
        perm_h, offs_h = G.box_partition(xyz0, nb, nb, nb)
        assert np.array_equal(perm, perm_h) and np.array_equal(offs, offs_h)
        xyz = np.ascontiguousarray(xyz0[perm])
        box, _ = G.block_contours(xyz, offs)
        edge = float((box[:, 1] - box[:, 0]).max(axis=1).mean())
        ext = ctx.extend_blocks(xyz, offs, 0.15 * edge, wl["sc"])
        ext_h = G.extend_blocks(xyz, offs, 0.15 * edge, wl["sc"])
        assert len(ext) == len(ext_h)
        for a, b in zip(ext, ext_h):
            assert np.array_equal(a, b)


def test_prep_rejects_bad_input(ctx):
    from midas_gb300._lib import MidasError
    with pytest.raises(MidasError):
        ctx.voxelise_sphere(-1.0, 0.1)
    with pytest.raises(MidasError):
        ctx.extend_blocks(np.zeros((4, 3)), [0, 2, 2, 4], 0.1, 0.1)   # empty block
