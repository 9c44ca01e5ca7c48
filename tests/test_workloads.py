"""Benchmark scenes: sizes and partition arrays in the C-ABI layout (CPU only)."""
import numpy as np


def test_mom_scene_size():
    from midas_gb300.workloads import mom_c1
    wl = mom_c1()
    assert len(wl["xyz"]) == 4224 and wl["method"] == "mom"


def test_small_cbfm_scene_partition():
    from midas_gb300.workloads import cbfm_args, cbfm_c2_small
    wl = cbfm_c2_small()
    n = len(wl["xyz"])
    bo, eo, ei = cbfm_args(wl)
    assert bo[0] == 0 and bo[-1] == n and np.all(np.diff(bo) > 0)
    assert len(bo) == 9                     # 2 x 2 x 2 blocks, none empty
    assert eo[0] == 0 and eo[-1] == len(ei) and np.all(np.diff(eo) >= 0)
    for b in range(len(bo) - 1):
        e = ei[eo[b]:eo[b + 1]]
        # extension cells lie outside the block and are distinct
        assert np.all((e < bo[b]) | (e >= bo[b + 1])) and len(np.unique(e)) == len(e)
    # every block has more unknowns than CBF excitations (a well-posed reduced system)
    assert np.min(3 * np.diff(bo)) > 2 * len(wl["cth"])
    assert wl["niws"] in (91, 190, 231) and len(wl["th"]) == 24   # initializeNipws table


def test_dense_cube_scenes():
    from midas_gb300.workloads import mom_c3, mom_c3_small
    wl = mom_c3()
    assert len(wl["xyz"]) == 20000 and len(wl["th"]) == 32 and wl["ir_tol"] == 1e-8
    assert np.all((wl["eps"].real >= 1.5) & (wl["eps"].real <= 3.5))
    assert np.all((wl["eps"].imag >= 0) & (wl["eps"].imag <= 0.2))
    assert len(mom_c3_small()["xyz"]) == 4000


def test_c4_batch_scene():
    """C4: 256 seeded aggregates of 4-64 monomers, 48 directions, 'rf' receivers with the
    positional forward / backward extras; instances built on demand."""
    from midas_gb300 import workloads as W
    wl = W.c4()
    assert len(wl["n_mono"]) == 256 and wl["n_mono"].min() >= 4 and wl["n_mono"].max() <= 64
    assert len(wl["th"]) == 48 and len(wl["rx_th"]) == wl["nrx"] + 2 * 48
    xyz, d = W.c4_instance(wl, 0)
    assert d == 1.0 / 3.0 and 90 * wl["n_mono"][0] < len(xyz) < 130 * wl["n_mono"][0]
    assert np.array_equal(xyz, W.c4_instance(wl, 0)[0])


def test_c4_batch_runner_calls(capsys):
    """The batch runner's host logic with a stand-in context: every aggregate is set,
    solved for all directions, and its efficiencies requested with 'rf' lists whose
    receiver array carries the positional forward / backward blocks."""
    from midas_gb300 import workloads as W
    wl = W.c4(n_instances=3, ndir=4, nrx=10)
    calls = []

    class FakeCtx:
        def set_cells(self, xyz, sc, eps, k0):
            self.n = len(xyz)
            calls.append(("cells", len(xyz), sc, k0))
            return self

        def mom_solve(self, th, ph):
            return np.ones((3 * self.n, 2 * len(th)), complex)

        def smatrix(self, rth, rph, E):
            return np.ones((len(rth), 2 * E.shape[1]), complex)

        def cext_cabs(self, th, ph, E):
            return np.full(len(th), 2.0), np.full(len(th), 0.5)

        def scattering_quantities(self, qt, qr, tg, rg, th, ph, rth, rph, S, ce, ca, dm, k0):
            assert (qt, qr) == ("rf", "rf") and tg == (len(th), 1) and rg == (10, 1)
            assert len(rth) == 10 + 2 * len(th) and S.shape == (len(rth), 4 * len(th))
            assert np.allclose(rth[10:10 + len(th)], th) and np.allclose(rth[10 + len(th):], 180.0 - th)
            assert dm > 0 and k0 == wl["k0"]
            calls.append(("q", dm))
            return np.zeros((len(th), 5)), np.array([1.0, 0.1, 0.9, 0.05, 0.3])

        def close(self):
            calls.append(("close",))

    assert W.run_batch(FakeCtx(), wl, 1, lanes=1) == 0
    assert [c[0] for c in calls] == ["cells", "q"] * 3 + ["close"]
    out = capsys.readouterr().out
    assert "orientation-averaged solves/s" in out and "3 instances" in out
