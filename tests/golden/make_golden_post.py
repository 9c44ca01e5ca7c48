"""Generate tests/golden/golden_post.json: known answers of the far-field S matrix
and of the cross sections from the internal field, from a second, independent
restatement written here in plain Python with explicit component arithmetic:
  GetFFieldCoeff                   src/Green_functions.f90:1399-1438
  S projection (Vv, Vh, Hv, Hh)    src/Compute_EFields_MoM.f90:306-369
  Compute_ExtAbsCsec_fromIntField  src/Compute_ExtAbsCsec_fromIntField.f90:45-64
                                   (the field components summed before the products)
  Incident_Field (complex(4))      src/Incident_Field.f90:1-63
The cell parameters come from the SetCellsParams restatement of make_golden.py.
The C oracle (oracle/midas_oracle.c) must reproduce them exactly.  |z| is
sqrt(re*re + im*im) and Sc**3. is pow(Sc, 3.0), as in the oracle (the reference's
intrinsics leave those last bits unpinned).

Run:  python tests/golden/make_golden_post.py
"""
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import F, PI, cell_params   # noqa: E402

K0, SC = 2.0, 0.2
XYZ = [(-0.1, 0.3, 0.5), (0.1, -0.1, 0.3), (0.5, 0.3, -0.3), (-0.3, -0.5, 0.1), (0.3, 0.1, 0.1), (-0.5, 0.1, -0.3)]
EPS = [complex(2.25, 0.03), complex(3.1, 0.2), complex(1.7, 0.0), complex(2.9, 0.11), complex(2.0, 0.05),
       complex(2.6, 0.3)]
TH, PH = [90.0, 33.0], [90.0, 250.0]                     # incident directions
RTH, RPH = [0.0, 90.0, 33.0, 147.0, 180.0], [0.0, 90.0, 250.0, 70.0, 180.0]   # receivers


def field():
    """Seeded internal field, (3n, 2 NTr): V columns then H columns."""
    rng = np.random.default_rng(99)
    n = 3 * len(XYZ)
    return rng.normal(size=(n, 2 * len(TH))) + 1j * rng.normal(size=(n, 2 * len(TH)))


def cmul(a, b):
    return complex(a.real * b.real - a.imag * b.imag, a.real * b.imag + a.imag * b.real)


def smatrix(E):
    cells = [cell_params(SC, e, K0) for e in EPS]
    ntr = len(TH)
    S = np.zeros((len(RTH), 4 * ntr), complex)
    for r, (tc, pc) in enumerate(zip(RTH, RPH)):
        t, p = tc * PI / 180., pc * PI / 180.
        xcap, ycap, zcap = math.cos(t), math.sin(t) * math.cos(p), math.sin(t) * math.sin(p)
        ff = []
        for c, (x, y, z) in enumerate(XYZ):
            arg = -K0 * (xcap * x + ycap * y + zcap * z)
            ffc = complex(math.cos(arg), math.sin(arg))                 # exp(-J*k_0*(...))
            a = complex(ffc.real * (K0 * K0), ffc.imag * (K0 * K0))   # *k_0**2.
            che, kap = cells[c][1], cells[c][3]
            a = cmul(a, complex(kap * che.real, kap * che.imag))      # *f_kapChe
            a = complex(a.real / (4 * PI), a.imag / (4 * PI))         # /(4*Pi)
            ff.append(complex(a.real * K0, a.imag * K0))              # *k_0
        for tr in range(ntr):
            ev, eh = [0j, 0j, 0j], [0j, 0j, 0j]
            for c in range(len(XYZ)):
                for q in range(3):
                    av, ah = cmul(ff[c], E[3 * c + q, tr]), cmul(ff[c], E[3 * c + q, tr + ntr])
                    ev[q] = complex(ev[q].real + av.real, ev[q].imag + av.imag)
                    eh[q] = complex(eh[q].real + ah.real, eh[q].imag + ah.imag)
            st, ct, sp, cp = math.sin(t), math.cos(t), math.sin(p), math.cos(p)

            def v_of(e):
                return complex(-e[0].real * st + e[1].real * ct * cp + e[2].real * ct * sp,
                               -e[0].imag * st + e[1].imag * ct * cp + e[2].imag * ct * sp)

            def h_of(e):
                return complex(-e[1].real * sp + e[2].real * cp, -e[1].imag * sp + e[2].imag * cp)
            S[r, 4 * tr:4 * tr + 4] = [v_of(ev), h_of(ev), v_of(eh), h_of(eh)]
    return S


def incident_c4(t):
    """(3n, 2): V and H incident fields of direction t, rounded as complex(4)."""
    tr, pr = TH[t] * PI / 180.0, PH[t] * PI / 180.0
    st, ct, sp, cp = math.sin(tr), math.cos(tr), math.sin(pr), math.cos(pr)
    kx4, ky4, kz4 = float(F(K0 * ct)), float(F(K0 * st * cp)), float(F(K0 * st * sp))
    r4 = lambda v: complex(float(F(v.real)), float(F(v.imag)))
    out = np.zeros((3 * len(XYZ), 2), complex)
    for c, (x, y, z) in enumerate(XYZ):
        e4 = (complex(math.cos(kx4 * x), math.sin(kx4 * x)) * complex(math.cos(ky4 * y), math.sin(ky4 * y))) * \
            complex(math.cos(kz4 * z), math.sin(kz4 * z))
        out[3 * c, 0] = r4(complex(-(e4.real * st), -(e4.imag * st)))
        out[3 * c + 1, 0] = r4(complex((e4.real * ct) * cp, (e4.imag * ct) * cp))
        out[3 * c + 2, 0] = r4(complex((e4.real * ct) * sp, (e4.imag * ct) * sp))
        out[3 * c + 1, 1] = r4(complex(-(e4.real * sp), -(e4.imag * sp)))
        out[3 * c + 2, 1] = r4(complex(e4.real * cp, e4.imag * cp))
    return out


def cross_sections(E):
    cells = [cell_params(SC, e, K0) for e in EPS]
    ntr = len(TH)
    cext, cabs = [], []
    for t in range(ntr):
        Ei = incident_c4(t)
        ev = eh = av = ah = 0.0
        for c in range(len(XYZ)):
            sv = sh = iv = ih = 0j
            for q in range(3):
                sv = complex(sv.real + E[3 * c + q, t].real, sv.imag + E[3 * c + q, t].imag)
                sh = complex(sh.real + E[3 * c + q, t + ntr].real, sh.imag + E[3 * c + q, t + ntr].imag)
                iv = complex(iv.real + Ei[3 * c + q, 0].real, iv.imag + Ei[3 * c + q, 0].imag)
                ih = complex(ih.real + Ei[3 * c + q, 1].real, ih.imag + Ei[3 * c + q, 1].imag)
            s3 = math.pow(SC, 3.0)
            che = cells[c][1]
            asv = math.sqrt(sv.real * sv.real + sv.imag * sv.imag)
            ash = math.sqrt(sh.real * sh.real + sh.imag * sh.imag)
            av = av + che.imag * (asv * asv) * s3
            ah = ah + che.imag * (ash * ash) * s3
            pv = cmul(cmul(che, sv), complex(iv.real, -iv.imag))
            ph_ = cmul(cmul(che, sh), complex(ih.real, -ih.imag))
            ev = ev + pv.imag * s3
            eh = eh + ph_.imag * s3
        cext.append(K0 * (ev + eh) / 2.)
        cabs.append(K0 * (av + ah) / 2.)
    return cext, cabs


def main():
    E = field()
    S = smatrix(E)
    cext, cabs = cross_sections(E)
    g = {"S": [[S.real[i].tolist(), S.imag[i].tolist()] for i in range(S.shape[0])], "cext": cext, "cabs": cabs}
    with open(os.path.join(HERE, "golden_post.json"), "w") as fh:
        json.dump(g, fh, indent=1)
    print("wrote golden_post.json")


if __name__ == "__main__":
    main()
