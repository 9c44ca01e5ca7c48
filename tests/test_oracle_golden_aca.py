"""The oracle's ACA (or_aca) against the golden fixtures of an independent Python
restatement of Calcul_MatrixZij_ACA (tests/golden/make_golden_aca.py)."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden_aca as MA   # noqa: E402

G = json.load(open(os.path.join(HERE, "golden", "golden_aca.json")))


def _c(rows):
    return np.array([[complex(a, b) for a, b in r] for r in rows])


@pytest.mark.parametrize("case", G["cases"], ids=lambda c: f"eps{c['eps']:.0e}-it{c['itmax']}")
def test_aca_exact(oracle, case):
    cells = oracle.Cells(np.array(MA.XYZ), MA.SC, np.array(MA.EPS), MA.K0)
    nr, nc = 3 * len(MA.ROWS), 3 * len(MA.COLS)
    k, U, V = oracle.aca(cells, 0, nr, nr, nc, eps=case["eps"], itmax=case["itmax"])
    assert k == case["k"]
    assert np.array_equal(U, _c(case["U"])), np.max(np.abs(U - _c(case["U"])))
    assert np.array_equal(V, _c(case["V"])), np.max(np.abs(V - _c(case["V"])))


def test_block_matches_golden_element(oracle):
    """The far block the restatement factors is the oracle's complex(4) block."""
    cells = oracle.Cells(np.array(MA.XYZ), MA.SC, np.array(MA.EPS), MA.K0)
    nr = len(MA.ROWS)
    Z = oracle.green_partial(cells, np.arange(nr), np.arange(nr, len(MA.XYZ)))
    assert np.array_equal(Z, np.array(MA.block()))
