"""Host logic of the learned initial guess (midas_gb300/learned.py), on the CPU."""
import numpy as np

from midas_gb300 import learned as LG


def test_scenes_are_seeded_and_sized():
    a = LG.scenes(5, 4, 16)
    b = LG.scenes(5, 4, 16)
    for s, t in zip(a, b):
        assert np.array_equal(s["mask"], t["mask"]) and np.array_equal(s["eps"], t["eps"]) and s["x"] == t["x"]
        assert s["n"] >= 8 and len(s["xyz"]) == s["n"] and len(s["eps"]) == s["n"]
        assert 1.0 <= s["x"] <= 8.0 + 1e-12
        assert np.all(s["eps"].real >= 1.3) and np.all(s["eps"].imag >= 0)
    assert {s["kind"] for s in a} == {"gaussian", "aggregate"}


def test_grid_and_cell_layouts_round_trip():
    sc = LG.scenes(2, 1, 12)[0]
    rng = np.random.default_rng(0)
    E = rng.standard_normal((3 * sc["n"], 2)) + 1j * rng.standard_normal((3 * sc["n"], 2))
    Eg = LG.cells_to_grid(sc, E)
    assert Eg.shape == (2, 12 ** 3, 6)
    assert np.allclose(LG.grid_to_cells(sc, Eg), E.astype(np.complex64), rtol=0, atol=1e-6)
    assert np.all(Eg[:, ~sc["mask"]] == 0)


def test_incident_grid_matches_the_moM_right_hand_side(oracle):
    """At the cells, the network's incident-field channels are the MoM right-hand side."""
    sc = LG.scenes(3, 1, 12)[0]
    inp, m = LG.grid_inputs(sc)
    c = oracle.Cells(sc["xyz"], sc["sc"], sc["eps"], sc["k0"])
    V = oracle.mom_rhs(c, sc["th"], sc["ph"])          # (3n, 2)
    idx = np.flatnonzero(sc["mask"])
    for pol in range(2):
        g = inp[pol, idx, 2:8].astype(np.float64)
        e = (g[:, 0::2] + 1j * g[:, 1::2]).reshape(-1)
        assert np.max(np.abs(e - V[:, pol])) < 1e-6
    chi = inp[0, idx, 0] + 1j * inp[0, idx, 1]
    assert np.allclose(chi, (sc["eps"] - 1).astype(np.complex64))
    assert np.all(m[0] == sc["mask"])
