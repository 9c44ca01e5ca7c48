"""The C oracle of the orientation-averaging step against the golden fixtures of an
independent plain-Python restatement (tests/golden/make_golden_q.py)."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden_q as MG   # noqa: E402

G = json.load(open(os.path.join(HERE, "golden", "golden_q.json")))


@pytest.mark.parametrize("entry", G["qag"], ids=lambda e: e["name"])
def test_qag_matches_golden(oracle, entry):
    f = MG.qag_column(entry["name"])
    r, _, _, bad = oracle.qag_grid(f, entry["a0"], entry["b0"])
    assert not bad and r == entry["result"], (r, entry["result"])


@pytest.mark.parametrize("case", G["cases"], ids=lambda c: f"{c['quad_tr']}-{c['quad_rx']}")
def test_quantities_match_golden(oracle, case):
    inp = MG.inputs(case)
    st, qd, qa = oracle.scattering_quantities(case["quad_tr"], case["quad_rx"], tuple(case["tr"]), tuple(case["rx"]),
                                              inp["tth"], inp["tph"], inp["rth"], inp["rph"], inp["S"],
                                              inp["cext"], inp["cabs"], inp["dm"], inp["k0"],
                                              cext_intfields=case["intf"], w_tr=inp["w_tr"], w_rx=inp["w_rx"])
    assert st == 0
    assert np.array_equal(qd, np.array(case["q_dir"])), np.max(np.abs(qd - np.array(case["q_dir"])))
    assert np.array_equal(qa, np.array(case["q_avg"])), (qa, case["q_avg"])
