"""C4 batch instances on the GPU against the oracle pipeline, instance by instance.

Each aggregate goes through the library (MoM solve, S matrix, cross sections,
list-rule orientation averages, Compute_Scattering_Quantities_2,
src/Compute_Scattering_Quantities.f90) on concurrent lanes, and its five
averaged efficiencies must equal the oracle's (LAPACK solve of the same
matrix) to 1e-6.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_c4_small_instances_match_oracle(gpulib, oracle):
    from midas_gb300 import _lib, workloads as W
    from midas_gb300.solver import Context
    wl = W.c4(n_instances=8, ndir=6, nrx=40)
    cells = [W.c4_instance(wl, k) for k in range(8)]
    ctx = Context(fill_mode=_lib.FILL_FAST)
    contexts = [ctx, ctx.sibling(), ctx.sibling()]
    res = W.batch_step(contexts, wl, cells)
    th, ph, rth, rph = wl["th"], wl["ph"], wl["rx_th"], wl["rx_ph"]
    ntr = len(th)
    sizes = [len(x) for x, _ in cells]
    for k in np.argsort(sizes)[:3]:   # the three smallest: the oracle's LAPACK solves stay short
        xyz, d = cells[k]
        c = oracle.Cells(xyz, d, wl["m"] ** 2, wl["k0"])
        r = oracle.mom_solve(c, th, ph, rth, rph)
        dm = 2.0 * (3.0 * len(xyz) * d ** 3 / (4.0 * math.pi)) ** (1.0 / 3.0)
        st, _, qa = oracle.scattering_quantities("rf", "rf", (ntr, 1), (wl["nrx"], 1), th, ph, rth, rph, r["S"],
                                                 r["cext"], r["cabs"], dm, wl["k0"])
        assert st == 0
        q = res[k][0]
        rel = np.max(np.abs(q - qa) / np.maximum(np.abs(qa), 1e-30))
        print(k, 3 * len(xyz), "unknowns", q, qa, rel)
        assert rel < 1e-6, (k, q, qa)
    for cx in contexts:
        cx.close()
