"""The oracle's far-field S matrix and internal-field cross sections against the
golden fixtures of an independent Python restatement (tests/golden/make_golden_post.py)."""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden_post as MP   # noqa: E402

G = json.load(open(os.path.join(HERE, "golden", "golden_post.json")))


def _cells(O):
    return O.Cells(np.array(MP.XYZ), MP.SC, np.array(MP.EPS), MP.K0)


def test_smatrix_exact(oracle):
    S = oracle.smatrix(_cells(oracle), np.array(MP.RTH), np.array(MP.RPH), MP.field())
    ref = np.array([np.array(r) + 1j * np.array(i) for r, i in G["S"]])
    assert np.array_equal(S, ref), np.max(np.abs(S - ref))


def test_cross_sections_exact(oracle):
    ce, ca = oracle.cext_cabs(_cells(oracle), np.array(MP.TH), np.array(MP.PH), MP.field())
    assert np.array_equal(ce, G["cext"]), (ce, G["cext"])
    assert np.array_equal(ca, G["cabs"]), (ca, G["cabs"])
