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
