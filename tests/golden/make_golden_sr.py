"""Generate tests/golden/golden_sr.json: known answers of the SR thresholding of the
CBFM block matrices, from a second, independent restatement written here in plain
Python with numpy.float32 scalars for the complex(4) and real(4) quantities:
  Green_s_tr_partial_FN       src/Green_functions.f90:176-287  (Frobenius norm; real(4)
                              |F|**2 terms, off-diagonal dyad terms weighted by 2)
  SR_Green_s_tr_partial_FN    src/Green_functions.f90:564-806  (entries of |g| =
                              |-F f_kapChe| above |1 - Znnpp(1)| / fSR: count and norm)
  setfSR                      src/getParameters_CBFM.f90:113-168 (the fSR ladder)
The complex(4) element is make_golden.py's restatement of Green_s_tr_partial.
The norms are sums over the block; the C oracle accumulates them in parallel
chunks, so the test holds them to 1e-13 and every count, and the chosen fSR,
exactly.  |1 - Znnpp| is hypot(), as in the oracle.

Run:  python tests/golden/make_golden_sr.py
"""
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import F, c4mul, cell_params, f4   # noqa: E402

K0, SC = 2.0, 0.2
XYZ = [(0.2 * i, 0.2 * j, 0.2 * k) for k in range(3) for j in range(4) for i in range(4)]   # 48 cells
EPS_INHOMOG = [complex(1.8 + 0.05 * (c % 7), 0.01 * (c % 5)) for c in range(len(XYZ))]
EPS_HOMOG = [complex(2.4, 0.1)] * len(XYZ)
LADDER = [float(F(v)) for v in (1e2, 1e3, 2e3, 3e3, 4e3, 5e3, 6e3, 7e3, 8e3, 9e3, 1e4)]
RES_SR = float(F(1e-2))


def abs4(v):
    re, im = F(v[0]), F(v[1])
    return np.sqrt(re * re + im * im)          # real(4)


def fn_full(cells, homog):
    val = 0.0
    n = len(XYZ)
    for s in range(n):
        che, kap = cells[s][1], cells[s][3]
        fk = kap * che
        afk = abs4((F(fk.real), F(fk.imag)))
        for o in range(s if homog else 0, n):
            if o == s:
                a = math.hypot(1 - cells[s][2].real, -cells[s][2].imag)
                val = val + 3. * (a * a)
                continue
            D = f4(tuple(XYZ[o][k] - XYZ[s][k] for k in range(3)), K0)
            a = {pq: abs4(D[pq]) for pq in ((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))}
            t = a[0, 0] * a[0, 0] + F(2.0) * (a[0, 1] * a[0, 1]) + F(2.0) * (a[0, 2] * a[0, 2]) \
                + a[1, 1] * a[1, 1] + F(2.0) * (a[1, 2] * a[1, 2]) + a[2, 2] * a[2, 2]
            val = val + float(t * (afk * afk))
    return math.sqrt(val)


def sr_fn(cells, fsr, homog):
    n = len(XYZ)
    vmax = math.hypot(1 - cells[0][2].real, -cells[0][2].imag)
    thr = vmax / fsr
    nnz, g2 = 0, 0.0
    for io in range(n):
        for is_ in range(io if homog else 0, n):
            if io == is_:
                a = math.hypot(1 - cells[io][2].real, -cells[io][2].imag)
                for _ in range(3):
                    nnz += 1
                    g2 = g2 + a * a
                continue
            fk = cells[is_][3] * cells[is_][1]
            fk4 = (F(fk.real), F(fk.imag))
            D = f4(tuple(XYZ[io][k] - XYZ[is_][k] for k in range(3)), K0)
            for p in range(3):
                for q in range(3):
                    g = c4mul(D[(p, q)], fk4)
                    ag = abs4((-g[0], -g[1]))
                    if float(ag) > thr:
                        nnz += 1
                        g2 = g2 + float(ag * ag)
    return nnz, math.sqrt(g2)


def set_fsr(cells, homog, norm_z, ladder_out):
    jj, res, fsr, nnz = 0, 1e3, LADDER[0], 0
    while jj < len(LADDER) and res > RES_SR:
        fsr = LADDER[jj]
        nnz, fn = ladder_out[jj]
        res = abs(norm_z - fn) / norm_z * 100.
        jj += 1
    return fsr, nnz


def main():
    out = {}
    for name, eps, homog in (("inhomog", EPS_INHOMOG, 0), ("homog", EPS_HOMOG, 1)):
        cells = [cell_params(SC, e, K0) for e in eps]
        norm_z = fn_full(cells, homog)
        ladder = [sr_fn(cells, f, homog) for f in LADDER]
        fsr, nnz = set_fsr(cells, homog, norm_z, ladder)
        out[name] = {"homog": homog, "norm_z": norm_z, "ladder": [[f, n, v] for f, (n, v) in zip(LADDER, ladder)],
                     "fsr": fsr, "nnz": nnz}
        print(name, "norm", norm_z, "nnz per fSR", [n for n, _ in ladder], "-> fSR", fsr, "nnz", nnz)
    with open(os.path.join(HERE, "golden_sr.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    main()
