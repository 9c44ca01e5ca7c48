"""Seeded inputs of the orientation-averaging step (Compute_Scattering_Quantities_1/_2)
shared by the oracle and GPU tests: direction sets built the way get_trans_Receiv
builds them, a synthetic S matrix with the forward-peaked magnitude of a real
one, and cross sections."""
from __future__ import annotations

import numpy as np

from midas_gb300 import geometry as G


def _sets(rule, th0, th1, nth, ph0, ph1, nph, rng):
    """(theta, phi, grid, weights) of a direction set with the given rule."""
    if rule in ("un", "tr"):
        th, ph = G.uniform_directions(th0, th1, nth, ph0, ph1, nph)
        return th, ph, (nth, nph), None
    if rule == "gl":
        th, ph, w = G.gauss_legendre_directions(th0, th1, nth, ph0, ph1, nph)
        return th, ph, (nth, nph), w
    n = nth * nph   # a list: seeded directions
    th, ph = G.random_directions(n, seed=int(rng.integers(1 << 30)))
    w = rng.uniform(0.5, 1.5, n) if rule == "lb" else None
    if w is not None:
        w /= w.sum()
    return th, ph, (n, 1), w


def case(quad_tr, quad_rx, tr=(4, 3), rx=(19, 9), seed=0, list_same=False):
    """A full input set.  Grid sets span theta 0..180 and phi 0..360 (the
    ranges the reference's adaptive index map needs).  With list transmitters
    the extra receivers are appended positionally (forward block, then
    backward block), as get_trans_Receiv does for 'sd' / 'lb'
    (src/get_trans_Receiv.f90:527-550)."""
    rng = np.random.default_rng(seed)
    tth, tph, tgrid, wtr = _sets(quad_tr, 0.0, 180.0, tr[0], 0.0, 360.0, tr[1], rng)
    if list_same and quad_tr in ("sd", "lb", "rf") and quad_rx in ("sd", "lb", "rf"):
        rth, rph, rgrid, wrx = tth.copy(), tph.copy(), tgrid, wtr
    else:
        rth, rph, rgrid, wrx = _sets(quad_rx, 0.0, 180.0, rx[0], 0.0, 360.0, rx[1], rng)
    ntr = tgrid[0] * tgrid[1]
    if quad_tr in ("sd", "lb", "rf"):
        fth, fph = tth, tph
        bth, bph = 180.0 - tth, np.fmod(tph + 180.0, 360.0)
        same = (ntr == rgrid[0] * rgrid[1]) and quad_rx in ("sd", "lb", "rf")
        if same and quad_rx in ("sd", "lb"):
            rth_all, rph_all = np.concatenate([rth, bth]), np.concatenate([rph, bph])
        elif same:
            rth_all, rph_all = np.concatenate([rth, bth]), np.concatenate([rph, bph])
        else:
            rth_all, rph_all = np.concatenate([rth, fth, bth]), np.concatenate([rph, fph, bph])
    else:
        rth_all, rph_all = G.receivers_with_extras(rth, rph, tth, tph)
    nrx_tot = len(rth_all)
    # |S| peaked towards each transmitter's forward direction, random phases
    S = np.empty((nrx_tot, 4 * ntr), np.complex128)
    for t in range(ntr):
        cosang = (np.cos(np.radians(rth_all)) * np.cos(np.radians(tth[t]))
                  + np.sin(np.radians(rth_all)) * np.sin(np.radians(tth[t])) * np.cos(np.radians(rph_all - tph[t])))
        amp = 0.3 + 2.0 * np.exp(2.0 * (cosang - 1.0))
        for k in range(4):
            scale = 1.0 if k in (0, 3) else 0.1
            S[:, 4 * t + k] = scale * amp * np.exp(2j * np.pi * rng.random(nrx_tot)) * rng.uniform(0.8, 1.2, nrx_tot)
    dm, k0 = 2.0, 2.0
    cext = rng.uniform(5.0, 7.0, ntr)
    cabs = rng.uniform(0.2, 0.4, ntr)
    return dict(quad_tr=quad_tr, quad_rx=quad_rx, tr_grid=tgrid, rx_grid=rgrid, tr_th=tth, tr_ph=tph,
                rx_th=rth_all, rx_ph=rph_all, S=S, cext=cext, cabs=cabs, dm=dm, k0=k0, w_tr=wtr, w_rx=wrx)


def oracle_call(O, c, cext_intfields=0):
    return O.scattering_quantities(c["quad_tr"], c["quad_rx"], c["tr_grid"], c["rx_grid"], c["tr_th"], c["tr_ph"],
                                   c["rx_th"], c["rx_ph"], c["S"], c["cext"], c["cabs"], c["dm"], c["k0"],
                                   cext_intfields=cext_intfields, w_tr=c["w_tr"], w_rx=c["w_rx"])


def gpu_call(ctx, c, cext_intfields=0):
    return ctx.scattering_quantities(c["quad_tr"], c["quad_rx"], c["tr_grid"], c["rx_grid"], c["tr_th"], c["tr_ph"],
                                     c["rx_th"], c["rx_ph"], c["S"], c["cext"], c["cabs"], c["dm"], c["k0"],
                                     cext_intfields=cext_intfields, w_tr=c["w_tr"], w_rx=c["w_rx"])
