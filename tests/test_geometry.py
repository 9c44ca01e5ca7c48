"""Host-side scene preparation (numpy) against the C oracle's restatements."""
import numpy as np
import pytest

from midas_gb300 import geometry as G


@pytest.mark.parametrize("dm,sc", [(2.0, 0.2), (2.0, 0.1), (1.6, 0.0755)])
def test_sphere_voxeliser_matches_oracle(oracle, dm, sc):
    assert np.array_equal(G.sphere_cells(dm, sc), oracle.sphere_cells(dm, sc))


@pytest.mark.parametrize("niws", [91, 190, 231, 325])
def test_transmitters_match_oracle(oracle, niws):
    th, ph = G.transmitters_un(niws)
    th2, ph2 = oracle.transmitters_un(niws)
    assert np.array_equal(th, th2) and np.array_equal(ph, ph2)


def test_partition_and_extension():
    xyz = G.sphere_cells(2.0, 0.1)
    perm, offs = G.box_partition(xyz, 3, 3, 3)
    assert offs[-1] == len(xyz) and np.all(np.diff(offs) > 0)
    assert sorted(perm.tolist()) == list(range(len(xyz)))
    xs = xyz[perm]
    ext = G.extend_blocks(xs, offs, 0.1, 0.1)
    for b, e in enumerate(ext):
        own = set(range(offs[b], offs[b + 1]))
        assert own.isdisjoint(set(e.tolist()))
        assert len(e) > 0


def test_gaussian_sphere_seeded():
    a = G.gaussian_sphere(1.0, 0.15, 20.0, 0.1, seed=5)
    b = G.gaussian_sphere(1.0, 0.15, 20.0, 0.1, seed=5)
    c = G.gaussian_sphere(1.0, 0.15, 20.0, 0.1, seed=6)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    vol = len(a) * 0.1 ** 3
    assert 0.6 * 4.19 < vol < 1.4 * 4.19


def test_nipws():
    assert G.init_nipws(0.3) == 91 and G.init_nipws(2.5) == 190 and G.init_nipws(12) == 231


@pytest.mark.parametrize("n", [4, 23, 64])
def test_fractal_aggregate(n):
    """Touching, non-overlapping monomers on the fractal law N = kf (Rg/a)^df."""
    P = G.fractal_aggregate(n, a=1.0, df=1.8, kf=1.3, seed=n)
    assert P.shape == (n, 3) and np.allclose(P.mean(axis=0), 0.0, atol=1e-12)
    D = np.linalg.norm(P[:, None] - P[None], axis=2) + np.eye(n) * 1e9
    assert D.min() >= 2.0 * (1 - 1e-9)                       # no overlaps
    assert np.all(D.min(axis=1) <= 2.0 * (1 + 1e-9))          # every monomer touches one
    rg = np.sqrt(np.mean(np.sum(P ** 2, axis=1)))
    assert abs(rg - (n / 1.3) ** (1 / 1.8)) < 1e-6 * rg      # the law holds wherever it was reachable
    assert np.array_equal(P, G.fractal_aggregate(n, a=1.0, df=1.8, kf=1.3, seed=n))   # seeded


def test_voxelise_spheres():
    P = G.fractal_aggregate(12, seed=3)
    xyz, d = G.voxelise_spheres(P, 1.0, 6)
    assert d == 1.0 / 3.0
    dist = np.min(np.linalg.norm(xyz[:, None] - P[None], axis=2), axis=1)
    assert np.all(dist < 1.0)                                   # every cell centre inside a monomer
    assert abs(len(xyz) - 12 * 4 / 3 * np.pi * 27) < 0.05 * len(xyz)
    g = (xyz - xyz.min(axis=0)) / d                             # on one lattice, no duplicates
    assert np.allclose(g, np.round(g), atol=1e-9) and len(np.unique(np.round(g), axis=0)) == len(xyz)
    single, _ = G.voxelise_spheres(np.zeros((1, 3)), 1.0, 6)   # a lone sphere: 6 cells across
    assert np.ptp(single[:, 0]) == pytest.approx(5 * d)


def test_list_receivers_layout():
    th, ph = np.array([10.0, 100.0]), np.array([30.0, 300.0])
    rth, rph = G.list_receivers_with_extras([0.0, 45.0, 90.0], [0.0, 90.0, 180.0], th, ph)
    assert np.array_equal(rth, [0.0, 45.0, 90.0, 10.0, 100.0, 170.0, 80.0])
    assert np.array_equal(rph, [0.0, 90.0, 180.0, 30.0, 300.0, 210.0, 120.0])
