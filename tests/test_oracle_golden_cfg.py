"""The configuration fixtures (tests/golden/cfg_*.npz) on the CPU.

Checks that each fixture belongs to the scene the workload generator builds
today (the GPU tests compare only then), that its digest is well formed, and
that the smallest one is reproduced by the oracle exactly.
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import cfg_digest as D  # noqa: E402

CASES = {"c1_lit": lambda W: W.mom_tiny(), "c1": lambda W: W.mom_c1(), "c3": lambda W: W.mom_c3(n_cells=8000),
         "c2": lambda W: W.cbfm_c2()}


@pytest.mark.parametrize("name", sorted(CASES))
def test_fixture_matches_generated_scene(name):
    from midas_gb300 import workloads as W
    p = D.fixture_path(name)
    assert os.path.exists(p), p
    fx = np.load(p)
    wl = CASES[name](W)
    assert np.array_equal(D.scene_signature(wl), fx["signature"])
    N = 3 * len(wl["xyz"])
    ncol = 2 * len(wl["th"])
    assert fx["E_rows"].shape == (min(N, D.N_ROWS), ncol)
    assert np.array_equal(fx["rows"], D.row_subset(N))
    assert fx["colnorm"].shape == (ncol,) and np.all(fx["colnorm"] > 0)
    assert fx["cext"].shape == (len(wl["th"]),) and fx["S"].shape[1] == 4 * len(wl["th"])
    if name == "c2":
        assert fx["K"].shape == (len(wl["offs"]) - 1,) and np.all(fx["K"] > 0)


def test_smallest_fixture_reproduced_by_oracle(oracle):
    from midas_gb300 import workloads as W
    wl = W.mom_tiny()
    fx = np.load(D.fixture_path("c1_lit"))
    c = oracle.Cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
    r = oracle.mom_solve(c, wl["th"], wl["ph"], *D.receivers("polar181"))
    res = D.compare(fx, r["E"], r["cext"], r["cabs"], r["S"])
    # LAPACK's blocking can depend on the thread count: equal to rounding
    assert res["E_rows_rel"] < 1e-13 and res["cext_rel"] < 1e-13 and res["S_rel"] < 1e-13, res
