"""Orientation averaging on the GPU (midas_gpu_scattering_quantities) against the
oracle: every integration rule, the internal-field option, a solved sphere end
to end, and the reference's error cases."""
import numpy as np
import pytest

import scatq_cases as C

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpulib):
    from midas_gb300.solver import Context
    c = Context()
    yield c
    c.close()


def _rel(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


@pytest.mark.parametrize("tr,rx,kw", [
    ("un", "un", {}), ("un", "un", {"tr": (1, 1), "rx": (181, 25)}), ("tr", "tr", {}), ("gl", "gl", {}),
    ("un", "sd", {}), ("un", "lb", {}), ("gl", "un", {}), ("un", "tr", {"tr": (7, 5)}),
    ("sd", "sd", {}), ("lb", "lb", {}), ("rf", "rf", {}),
    ("sd", "sd", {"list_same": True}), ("lb", "lb", {"list_same": True})])
@pytest.mark.parametrize("intf", [0, 1])
def test_rules_match_oracle(ctx, oracle, tr, rx, kw, intf):
    """Same formulas, same operation order, rounded intrinsics on the GPU: the
    per-direction and averaged efficiencies match the oracle (the host builds the
    sine / cosine tables with the same libm on both sides), bit for bit in practice;
    the bar is 1e-12 relative."""
    c = C.case(tr, rx, seed=sum(map(ord, tr + rx)) + 7 * intf, **kw)
    st, qd_o, qa_o = C.oracle_call(oracle, c, cext_intfields=intf)
    assert st == 0
    qd, qa = C.gpu_call(ctx, c, cext_intfields=intf)
    assert _rel(qd, qd_o) <= 1e-12, (_rel(qd, qd_o), np.argwhere(qd != qd_o)[:5])
    assert _rel(qa, qa_o) <= 1e-12 or (np.all(qa_o == 0) and np.all(qa == 0)), (qa, qa_o)


def test_sphere_end_to_end(gpulib, oracle):
    """The reference's sphere example layout (one incident direction, theta 0..180
    x phi 0..360 receivers, 'un'/'un') on a 489-cell sphere solved on the GPU:
    S and Cext/Cabs from the GPU, then the efficiencies, against the oracle's
    whole chain (internal fields agree to 1e-10, so the float quadratures agree
    to 1e-6)."""
    from midas_gb300 import geometry as G
    from midas_gb300.solver import Context, compute_efields_mom
    m, a, k0 = 1.5 + 0.01j, 1.0, 2.0
    sc = a / 4.775
    xyz = oracle.sphere_cells(2 * a, sc)
    th, ph = np.array([0.0]), np.array([0.0])
    rth, rph = G.uniform_directions(0, 180, 181, 0, 360, 25)
    rth, rph = G.receivers_with_extras(rth, rph, th, ph)
    ref = oracle.mom_solve(oracle.Cells(xyz, sc, m * m, k0), th, ph, rth, rph)
    st, qd_o, qa_o = oracle.scattering_quantities("un", "un", (1, 1), (181, 25), th, ph, rth, rph, ref["S"],
                                                  ref["cext"], ref["cabs"], 2 * a, k0)
    assert st == 0
    c = Context().set_cells(xyz, sc, m * m, k0)
    E, S, ce, ca = compute_efields_mom(c, th, ph, rth, rph)
    qd, qa = c.scattering_quantities("un", "un", (1, 1), (181, 25), th, ph, rth, rph, S, ce, ca, 2 * a, k0)
    c.close()
    assert _rel(qa, qa_o) < 1e-6, (qa, qa_o)
    q_ext_int = ce[0] / (np.pi * a * a)
    assert abs(qa[2] - (q_ext_int - qa[1])) / qa[2] < 0.03   # energy balance


def test_errors_are_reported(ctx):
    """Each error is caught before or by the kernels (bounded, in-range reads) and
    returned as MIDAS_ERR_ARG with the reason."""
    from midas_gb300 import geometry as G
    from midas_gb300._lib import MidasError

    def err(c):
        with pytest.raises(MidasError) as e:
            C.gpu_call(ctx, c)
        assert e.value.status == 1
        return str(e.value)

    # a grid whose theta row count no longer matches nrx_theta
    c = C.case("un", "un")
    c["rx_th"] = c["rx_th"].copy()
    c["rx_th"][5] += 1.0
    assert "distinct" in err(c)
    # forward / backward directions missing from the receivers (the reference stops)
    c = C.case("un", "un", rx=(19, 4))          # phi 0, 120, 240, 360: no phi = 180 receivers
    n = 19 * 4
    assert len(c["rx_th"]) > n
    c["rx_th"], c["rx_ph"], c["S"] = c["rx_th"][:n], c["rx_ph"][:n], c["S"][:n]
    assert "scattering direction" in err(c)
    # an 'un' grid starting at theta = 40: the reference's index map runs past it
    c = C.case("un", "un", tr=(1, 1))
    c["tr_th"], c["tr_ph"] = np.array([90.0]), np.array([90.0])
    rth, rph = G.uniform_directions(40.0, 180.0, 15, 0.0, 360.0, 9)
    c["rx_th"], c["rx_ph"], c["rx_grid"] = rth, rph, (15, 9)
    c["S"] = c["S"][:1].repeat(len(rth), axis=0)
    assert "outside its grid" in err(c)
    # list transmitters need list receivers
    err(C.case("sd", "un"))
