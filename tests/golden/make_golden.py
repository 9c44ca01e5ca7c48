"""Generate tests/golden/golden_small.json.

The reference (Fortran + MKL) cannot be built in this environment and ships no
known-answer vectors, so these fixtures come from a second, independent
restatement of the reference formulas written here in plain Python: Python
complex arithmetic for the complex(8) expressions and numpy.float32 for every
assignment to a complex(4)/real(4) local, following
  src/SetCellsParams.f90:31-49,
  src/Compute_EFields_MoM.f90:433-598 (FP64 element and RHS),
  src/Green_functions.f90:96-173 (complex(4) block element),
  src/Incident_Field.f90:1-63 (complex(4) incident field),
  src/Incident_Field.f90:65-166 (spherical-wave incident field),
  src/getParameters_CBFM.f90:34-75,294-348 and src/Discretization.f90:246-310.
The C oracle (oracle/midas_oracle.c) must reproduce them exactly; the GPU
library is then compared with the C oracle.

Run:  python tests/golden/make_golden.py
"""
import json
import math
import os

import numpy as np

F = np.float32
PI = float(np.arccos(F(-1.0)))          # Acos(-1.) in single precision
THIRD = float(F(1.0) / F(3.0))
TWO3 = float(F(2.0) / F(3.0))


def cell_params(sc, eps, k0):
    a = sc * (0.75 / PI) ** THIRD
    che = eps - 1.0
    ka = k0 * a
    e = complex(math.cos(ka), math.sin(ka))
    t = complex(TWO3 * e.real, TWO3 * e.imag) * complex(1.0, -ka)
    t = complex(t.real - 1.0, t.imag)
    zn = t * che
    kap = 4 * PI * (math.sin(ka) - ka * math.cos(ka)) / math.pow(k0, 3.0)
    return a, che, zn, kap


def f8(r3, k0):
    rx, ry, rz = r3
    r = math.sqrt(rx * rx + ry * ry + rz * rz)
    den = 4 * PI * (r * r)
    gr = complex(math.cos(k0 * r) / den, math.sin(k0 * r) / den)
    tau = complex(-(1 / r), k0)
    k2 = k0 * k0
    out = {}
    for p, d in enumerate(r3):
        s = 3.0 * (d * d) / (r * r)
        inner = complex((tau.real + k2 * (r - d * d / r)) - s * tau.real, tau.imag - s * tau.imag)
        out[(p, p)] = gr * inner
    w = complex(-k2 - (3.0 * tau.real) / r, -((3.0 * tau.imag) / r))
    for p, q in ((0, 1), (1, 2), (0, 2)):
        g = complex((gr.real / r) * (r3[p] * r3[q]), (gr.imag / r) * (r3[p] * r3[q]))
        out[(p, q)] = out[(q, p)] = g * w
    return out


def f4(r3, k0):
    rx, ry, rz = r3
    r = math.sqrt(rx * rx + ry * ry + rz * rz)
    den = 4 * PI * (r * r)
    gr4 = (F(math.cos(k0 * r) / den), F(math.sin(k0 * r) / den))
    tau4 = (F(-(1 / r)), F(k0))
    gr = complex(float(gr4[0]), float(gr4[1]))
    tau = complex(float(tau4[0]), float(tau4[1]))
    k2 = k0 * k0
    out = {}
    for p, d in enumerate(r3):
        s = 3.0 * (d * d) / (r * r)
        v = gr * complex((tau.real + k2 * (r - d * d / r)) - s * tau.real, tau.imag - s * tau.imag)
        out[(p, p)] = (F(v.real), F(v.imag))
    t3 = (F(3.0) * tau4[0], F(3.0) * tau4[1])
    w = complex(-k2 - float(t3[0]) / r, -(float(t3[1]) / r))
    for p, q in ((0, 1), (1, 2), (0, 2)):
        g = complex((gr.real / r) * (r3[p] * r3[q]), (gr.imag / r) * (r3[p] * r3[q]))
        v = g * w
        out[(p, q)] = out[(q, p)] = (F(v.real), F(v.imag))
    return out


def c4mul(a, b):
    return (a[0] * b[0] - a[1] * b[1], a[0] * b[1] + a[1] * b[0])


def main():
    rng = np.random.default_rng(2024)
    k0 = 2.0
    sc = 0.2
    xyz = [(-0.1, 0.3, 0.5), (0.1, -0.1, 0.3), (0.5, 0.3, -0.3), (-0.3, -0.5, 0.1)]
    eps = [complex(2.25, 0.03), complex(3.1, 0.2), complex(1.7, 0.0), complex(2.9, 0.11)]
    cells = [cell_params(sc, e, k0) for e in eps]
    g = {"k0": k0, "sc": sc, "xyz": xyz, "eps": [[e.real, e.imag] for e in eps]}
    g["a_n"] = [c[0] for c in cells]
    g["che"] = [[c[1].real, c[1].imag] for c in cells]
    g["znnpp"] = [[c[2].real, c[2].imag] for c in cells]
    g["kappa"] = [c[3] for c in cells]
    # MoM element matrix (FP64) and complex(4) block matrix over all 4 cells
    n = len(xyz)
    Z8 = np.zeros((3 * n, 3 * n), complex)
    Z4 = np.zeros((3 * n, 3 * n), complex)
    for io in range(n):
        for is_ in range(n):
            if io == is_:
                for p in range(3):
                    Z8[3 * io + p, 3 * is_ + p] = 1 - cells[is_][2]
                    Z4[3 * io + p, 3 * is_ + p] = 1 - cells[is_][2]
                continue
            r3 = tuple(xyz[io][k] - xyz[is_][k] for k in range(3))
            fk = cells[is_][3] * cells[is_][1]
            fk4 = (F(fk.real), F(fk.imag))
            D8, D4 = f8(r3, k0), f4(r3, k0)
            for p in range(3):
                for q in range(3):
                    Z8[3 * io + p, 3 * is_ + q] = -(D8[(p, q)] * fk)
                    v = c4mul(D4[(p, q)], fk4)
                    Z4[3 * io + p, 3 * is_ + q] = complex(-float(v[0]), -float(v[1]))
    g["Z8"] = [[Z8.real[i].tolist(), Z8.imag[i].tolist()] for i in range(3 * n)]
    g["Z4"] = [[Z4.real[i].tolist(), Z4.imag[i].tolist()] for i in range(3 * n)]
    # incident fields for two directions
    th = [90.0, 33.0]
    ph = [90.0, 250.0]
    V8 = np.zeros((3 * n, 4), complex)
    E4 = np.zeros((3 * n, 4), complex)
    for t in range(2):
        tr, pr = th[t] * PI / 180.0, ph[t] * PI / 180.0
        st, ct, sp, cp = math.sin(tr), math.cos(tr), math.sin(pr), math.cos(pr)
        kx, ky, kz = k0 * ct, k0 * st * cp, k0 * st * sp
        kx4, ky4, kz4 = float(F(kx)), float(F(ky)), float(F(kz))
        for c in range(n):
            x, y, z = xyz[c]
            e8 = (complex(math.cos(kx * x), math.sin(kx * x)) * complex(math.cos(ky * y), math.sin(ky * y))) * \
                complex(math.cos(kz * z), math.sin(kz * z))
            e4 = (complex(math.cos(kx4 * x), math.sin(kx4 * x)) * complex(math.cos(ky4 * y), math.sin(ky4 * y))) * \
                complex(math.cos(kz4 * z), math.sin(kz4 * z))
            V8[3 * c, t] = complex(-(e8.real * st), -(e8.imag * st))
            V8[3 * c + 1, t] = complex((e8.real * ct) * cp, (e8.imag * ct) * cp)
            V8[3 * c + 2, t] = complex((e8.real * ct) * sp, (e8.imag * ct) * sp)
            V8[3 * c + 1, t + 2] = complex(-(e8.real * sp), -(e8.imag * sp))
            V8[3 * c + 2, t + 2] = complex(e8.real * cp, e8.imag * cp)
            r4 = lambda v: complex(float(F(v.real)), float(F(v.imag)))
            E4[3 * c, t] = r4(complex(-(e4.real * st), -(e4.imag * st)))
            E4[3 * c + 1, t] = r4(complex((e4.real * ct) * cp, (e4.imag * ct) * cp))
            E4[3 * c + 2, t] = r4(complex((e4.real * ct) * sp, (e4.imag * ct) * sp))
            E4[3 * c + 1, t + 2] = r4(complex(-(e4.real * sp), -(e4.imag * sp)))
            E4[3 * c + 2, t + 2] = r4(complex(e4.real * cp, e4.imag * cp))
    g["th"], g["ph"] = th, ph
    # Incident_Field_Spherical (src/Incident_Field.f90:65-166) on the cells in the
    # order [2, 0, 3, 1]: centre = mean centroid summed in that order, Rsource =
    # 10 max(Rbl, 2 Pi / k0), complex(4) phase exp(i k0 R) / R, FP64 local angles
    order = [2, 0, 3, 1]
    pts = [xyz[i] for i in order]
    cen = [0.0, 0.0, 0.0]
    for q in pts:
        for k in range(3):
            cen[k] += q[k]
    cen = [v / len(pts) for v in cen]
    rbl = math.sqrt(max((q[0] - cen[0]) ** 2 + (q[1] - cen[1]) ** 2 + (q[2] - cen[2]) ** 2 for q in pts))
    rsrc = 10.0 * max(rbl, 2.0 * PI / k0)
    r4 = lambda v: complex(float(F(v.real)), float(F(v.imag)))
    ES = np.zeros((3 * n, 4), complex)
    for t in range(2):
        tr, pr = th[t] * PI / 180.0, ph[t] * PI / 180.0
        src = (cen[0] + rsrc * math.cos(tr), cen[1] + rsrc * math.sin(tr) * math.cos(pr),
               cen[2] + rsrc * math.sin(tr) * math.sin(pr))
        for c, q in enumerate(pts):
            d = [q[k] - src[k] for k in range(3)]
            R = math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2])
            u = [v / R for v in d]
            phase = r4(complex(math.cos(k0 * R) / R, math.sin(k0 * R) / R))
            the, phi = math.acos(u[0]), math.atan2(u[2], u[1])
            st, ct, sp, cp = math.sin(the), math.cos(the), math.sin(phi), math.cos(phi)
            ES[3 * c, t] = r4(complex(-phase.real * st, -phase.imag * st))
            ES[3 * c + 1, t] = r4(complex((phase.real * ct) * cp, (phase.imag * ct) * cp))
            ES[3 * c + 2, t] = r4(complex((phase.real * ct) * sp, (phase.imag * ct) * sp))
            ES[3 * c + 1, t + 2] = r4(complex(-phase.real * sp, -phase.imag * sp))
            ES[3 * c + 2, t + 2] = r4(complex(phase.real * cp, phase.imag * cp))
    g["sph_order"] = order
    g["E4_sph"] = [[ES.real[i].tolist(), ES.imag[i].tolist()] for i in range(3 * n)]
    g["V8"] = [[V8.real[i].tolist(), V8.imag[i].tolist()] for i in range(3 * n)]
    g["E4"] = [[E4.real[i].tolist(), E4.imag[i].tolist()] for i in range(3 * n)]
    # 'un' transmitters (counts and a few angles) and Niws table lookups
    tr_out = {}
    for niws in (91, 190, 231):
        delta = float(F(291600.0) + F(4 * (niws - 1) * (360 * 180)))
        step = ((360.0 + 180.0) + math.sqrt(delta)) / (2.0 * (niws - 1))
        nth = int(math.floor(180.0 / step + 0.5)) + 1
        nph = int(math.floor(360.0 / step + 0.5)) + 1
        st_th = (math.cos(180.0 * PI / 180.0) - math.cos(0.0)) / (nth - 1)
        ths = [math.acos(max(1.0 * k * st_th + 1.0, -1.0)) * 180.0 / PI for k in range(nth)]
        tr_out[str(niws)] = {"ntr": nth * nph, "nth": nth, "nph": nph, "theta_first_col": ths,
                             "phi_step": 360.0 / (nph - 1)}
    g["transmitters"] = tr_out
    g["nipws"] = {"0.3": 91, "1.5": 190, "3.2": 231, "7.9": 861, "9.5": 231}
    # sphere voxeliser cell counts
    counts = {}
    for dm, s in ((2.0, 0.2), (2.0, 0.1), (1.6, 0.02 * 8)):
        ap = dm / 2.0
        nd = int(math.floor(dm / s + 0.5))
        nx = int(math.ceil((ap - float(F(0.8)) * ap / float(np.sqrt(F(3.0)))) / s))
        ni = nd - 2 * nx
        api = ni * s / 2.0
        cnt = ni ** 3
        doms = [(-ap, nd, -ap, nd, -ap, nx), (-ap, nx, -ap, nd, -api, ni), (api, nx, -ap, nd, -api, ni),
                (-api, ni, -ap, nx, -api, ni), (-api, ni, api, nx, -api, ni), (-ap, nd, -ap, nd, api, nx)]
        for (sx, nxx, sy, nyy, sz, nzz) in doms:
            for iz in range(1, nzz + 1):
                for iy in range(1, nyy + 1):
                    for ix in range(1, nxx + 1):
                        x, y, z = sx + (ix - 0.5) * s, sy + (iy - 0.5) * s, sz + (iz - 0.5) * s
                        if math.sqrt(x * x + y * y + z * z) < ap:
                            cnt += 1
        counts[f"{dm}_{s}"] = cnt
    g["sphere_counts"] = counts
    _ = rng
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_small.json")
    with open(out, "w") as f:
        json.dump(g, f, indent=1)
    print("wrote", out)


if __name__ == "__main__":
    main()
