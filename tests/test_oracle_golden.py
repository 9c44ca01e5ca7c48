"""The C oracle against the golden fixtures of an independent Python restatement."""
import json
import os

import numpy as np
import pytest

G = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden_small.json")))


def _cells(O):
    eps = np.array([complex(a, b) for a, b in G["eps"]])
    return O.Cells(np.array(G["xyz"]), G["sc"], eps, G["k0"])


def _mat(rows):
    return np.array([np.array(r) + 1j * np.array(i) for r, i in rows])


def test_ref_pi(oracle):
    assert oracle.ref_pi() == float(np.arccos(np.float32(-1.0))) == 3.1415927410125732


def test_cell_params_exact(oracle):
    c = _cells(oracle)
    assert np.array_equal(c.a_n, G["a_n"])
    assert np.array_equal(c.che, [complex(a, b) for a, b in G["che"]])
    assert np.array_equal(c.znnpp, [complex(a, b) for a, b in G["znnpp"]])
    assert np.array_equal(c.kappa, G["kappa"])


def test_mom_element_fp64_exact(oracle):
    c = _cells(oracle)
    assert np.array_equal(oracle.mom_fill(c), _mat(G["Z8"]))


def test_block_element_complex4_exact(oracle):
    c = _cells(oracle)
    idx = np.arange(c.n)
    assert np.array_equal(oracle.green_partial(c, idx, idx), _mat(G["Z4"]))


def test_incident_fields_exact(oracle):
    c = _cells(oracle)
    assert np.array_equal(oracle.mom_rhs(c, G["th"], G["ph"]), _mat(G["V8"]))
    assert np.array_equal(oracle.incident_c4(c, G["th"], G["ph"]), _mat(G["E4"]))


@pytest.mark.parametrize("niws", [91, 190, 231])
def test_transmitters_un(oracle, niws):
    th, ph = oracle.transmitters_un(niws)
    t = G["transmitters"][str(niws)]
    assert len(th) == t["ntr"]
    assert np.array_equal(th[: t["nth"]], t["theta_first_col"])
    assert ph[t["nth"]] == t["phi_step"]


def test_nipws_table(oracle):
    for r, v in G["nipws"].items():
        assert oracle.init_nipws(float(r)) == v


def test_sphere_counts(oracle):
    for key, cnt in G["sphere_counts"].items():
        dm, s = (float(v) for v in key.split("_"))
        assert len(oracle.sphere_cells(dm, s)) == cnt


def test_incident_spherical_exact(oracle):
    """Incident_Field_Spherical (src/Incident_Field.f90:65-166) against the independent
    restatement, on the cells in a permuted order (the block centre sums in cell order)."""
    c = _cells(oracle)
    E = oracle.incident_sph(c, G["th"], G["ph"], idx=np.array(G["sph_order"], np.int32))
    assert np.array_equal(E, _mat(G["E4_sph"]))
