"""The oracle's SR thresholding (Green_s_tr_partial_FN, SR_Green_s_tr_partial_FN,
setfSR) against the golden fixtures of an independent Python restatement
(tests/golden/make_golden_sr.py): counts and the chosen fSR exact, norms to 1e-13
(the oracle sums them in parallel chunks)."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden_sr as MS   # noqa: E402

G = json.load(open(os.path.join(HERE, "golden", "golden_sr.json")))


@pytest.mark.parametrize("name", ["inhomog", "homog"])
def test_sr_thresholding_matches_golden(oracle, name):
    g = G[name]
    eps = MS.EPS_HOMOG if g["homog"] else MS.EPS_INHOMOG
    cells = oracle.Cells(np.array(MS.XYZ), MS.SC, np.array(eps), MS.K0)
    idx = np.arange(len(MS.XYZ))
    nz = oracle.green_partial_fn(cells, idx, idx, g["homog"])
    assert abs(nz - g["norm_z"]) <= 1e-13 * g["norm_z"]
    for fsr, nnz, fn in g["ladder"]:
        _, n, f = oracle.sr_dense(cells, idx, fsr, g["homog"], want_matrix=False)
        assert n == nnz, (fsr, n, nnz)
        assert abs(f - fn) <= 1e-13 * fn
    assert oracle.set_fsr(cells, idx, g["homog"]) == (g["fsr"], g["nnz"])
    assert len({n for _, n, _ in g["ladder"]}) >= 3   # the ladder crosses the threshold
