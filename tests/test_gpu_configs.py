"""GPU answers at the benchmark configurations against the oracle's fixtures.

The fixtures (tests/golden/cfg_*.npz, written by make_cfg_fixtures.py) hold a
digest of the oracle's solution of each configuration at full size: a seeded
row subset and the column norms of the internal field, Cext / Cabs, S on a
receiver set and K per block.  Bars (the metric's): internal field <= 1e-6
relative, Cext / Cabs <= 1e-6, S <= 1e-5 of max |S|, K identical.
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import cfg_digest as D  # noqa: E402

pytestmark = pytest.mark.gpu

E_TOL, CX_TOL, S_TOL = 1e-6, 1e-6, 1e-5


def _load(name):
    p = D.fixture_path(name)
    if not os.path.exists(p):
        pytest.fail(f"fixture {p} missing: run tests/golden/make_cfg_fixtures.py {name}")
    return dict(np.load(p))


def _check(res):
    assert res["E_rows_rel"] <= E_TOL, res
    assert res["colnorm_rel"] <= E_TOL, res
    assert res["cext_rel"] <= CX_TOL and res["cabs_rel"] <= CX_TOL, res
    assert res["S_rel"] <= S_TOL, res
    if "K_equal" in res:
        assert res["K_equal"], res


@pytest.mark.parametrize("name,builder,rx", [("c1_lit", "mom_tiny", "polar181"), ("c1", "mom_c1", "polar181"),
                                            ("c3", "mom_c3_8000", "grid37x2")])
def test_mom_config_matches_oracle(gpulib, name, builder, rx):
    from midas_gb300 import _lib, workloads as W
    from midas_gb300.solver import Context
    wl = W.mom_c3(n_cells=8000) if builder == "mom_c3_8000" else getattr(W, builder)()
    fx = _load(name)
    assert np.array_equal(D.scene_signature(wl), fx["signature"]), "scene differs from the fixture's"
    ctx = Context(fill_mode=_lib.FILL_FAST).set_cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
    E = ctx.mom_solve(wl["th"], wl["ph"])
    ce, ca = ctx.cext_cabs(wl["th"], wl["ph"], E)
    S = ctx.smatrix(*D.receivers(rx), E)
    res = D.compare(fx, E, ce, ca, S)
    print(name, res, "ir", ctx.info.ir_iters, ctx.info.backward_error)
    _check(res)
    ctx.close()


def test_cbfm_c2_benchmark_scene_matches_oracle(gpulib):
    """The benchmarked CBFM scene itself (40,992 cells, 27 blocks, 24 directions x 2
    polarisations) with the benchmark's flags, against the oracle's full solve."""
    from midas_gb300 import _lib, workloads as W
    from midas_gb300.solver import Context
    wl = W.cbfm_c2()
    fx = _load("c2")
    assert np.array_equal(D.scene_signature(wl), fx["signature"]), "scene differs from the fixture's"
    ctx = Context(fill_mode=_lib.FILL_FAST).set_cells(wl["xyz"], wl["sc"], wl["eps"], wl["k0"])
    flags = _lib.CBFM_SR | _lib.CBFM_HOMOG
    E, K = ctx.cbfm_solve(wl["offs"], wl["ext"], wl["cth"], wl["cph"], wl["th"], wl["ph"], flags=flags)
    ce, ca = ctx.cext_cabs(wl["th"], wl["ph"], E)
    S = ctx.smatrix(*D.receivers("grid37x2"), E)
    res = D.compare(fx, E, ce, ca, S, K)
    print("c2", res)
    _check(res)
    ctx.close()
