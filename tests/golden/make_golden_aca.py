"""Generate tests/golden/golden_aca.json: known answers of the adaptive cross
approximation from a second, independent restatement, written here in plain
Python from Calcul_MatrixZij_ACA (src/Calcul_ACA_matrices.f90:6-219) with 1-based
pivot lists and the Fortran control flow.  Rows and columns of the far block come
from the complex(4) dyad element of make_golden.py (computeBlockRow / computeBlockCol,
src/Green_functions.f90:905-1225, evaluate the same element as Green_s_tr_partial).
Where the Fortran leaves the last bits to its compiler the restatement makes the
oracle's choices explicit: |z| = sqrt(re*re + im*im), a / b by the textbook
formula, MATMUL dot products summed in index order, MAXLOC the first maximum.
The C oracle (oracle/midas_oracle.c, or_aca) must reproduce U, V and the
iteration count exactly.

Run:  python tests/golden/make_golden_aca.py
"""
import json
import math
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import F, c4mul, cell_params, f4   # noqa: E402

K0, SC = 2.0, 0.2
ROWS = [(0.0, 0.0, 0.0), (0.2, 0.0, 0.0), (0.0, 0.2, 0.0), (0.2, 0.2, 0.0), (0.0, 0.0, 0.2), (0.2, 0.0, 0.2)]
COLS = [(2.6 + 0.2 * (k % 3), 0.5 + 0.2 * ((k // 3) % 2), -0.4 + 0.2 * (k // 6)) for k in range(8)]
XYZ = ROWS + COLS
EPS = [complex(2.0 + 0.15 * k, 0.02 * (k % 4)) for k in range(len(XYZ))]
EPS_ACA = float(F(1e-4))                 # Epsilon_ACA = 1E-4 (single-precision literal)
# converged at iteration 13 and 7; the last never meets its tolerance (k = itmax + 1)
CASES = [{"eps": EPS_ACA, "itmax": 18}, {"eps": 1e-2, "itmax": 18}, {"eps": 1e-9, "itmax": 6}]


def block():
    """Z of the far block: unknown rows of ROWS' cells x columns of COLS' cells."""
    cells = [cell_params(SC, e, K0) for e in EPS]
    nr, nc = 3 * len(ROWS), 3 * len(COLS)
    Z = [[0j] * nc for _ in range(nr)]
    for io in range(len(ROWS)):
        for js in range(len(COLS)):
            s = len(ROWS) + js
            r3 = tuple(XYZ[io][k] - XYZ[s][k] for k in range(3))
            fk = cells[s][3] * cells[s][1]
            fk4 = (F(fk.real), F(fk.imag))
            D4 = f4(r3, K0)
            for p in range(3):
                for q in range(3):
                    v = c4mul(D4[(p, q)], fk4)
                    Z[3 * io + p][3 * js + q] = complex(-float(v[0]), -float(v[1]))
    return Z


def cmul(a, b):
    return complex(a.real * b.real - a.imag * b.imag, a.real * b.imag + a.imag * b.real)


def cdiv(a, b):
    d = b.real * b.real + b.imag * b.imag
    return complex((a.real * b.real + a.imag * b.imag) / d, (a.imag * b.real - a.real * b.imag) / d)


def cabs(a):
    return math.sqrt(a.real * a.real + a.imag * a.imag)


def maxloc(vals):
    """1-based index of the first largest value."""
    best, bv = 1, -1.0
    for i, v in enumerate(vals, start=1):
        if v > bv:
            best, bv = i, v
    return best


def aca(Z, eps, itmax):
    nr, nc = len(Z), len(Z[0])
    row = lambda i: list(Z[i - 1])                     # computeBlockRow (1-based row)
    col = lambda j: [Z[i][j - 1] for i in range(nr)]   # computeBlockCol (1-based column)
    U = [[0j] * (itmax + 1) for _ in range(nr + 1)]    # U(i, l), 1-based
    V = [[0j] * (nc + 1) for _ in range(itmax + 1)]    # V(l, j), 1-based
    R = [[0j] * (nc + 1) for _ in range(nr + 1)]       # Appro_R
    I = [0] * (itmax + 2)
    J = [0] * (itmax + 2)
    NF = [0.0] * (itmax + 2)
    I[1] = 1
    zr = row(I[1])
    for c in range(1, nc + 1):
        R[I[1]][c] = zr[c - 1]
    J[1] = maxloc([cabs(R[I[1]][c]) for c in range(1, nc + 1)])
    pivot = R[I[1]][J[1]]
    for c in range(1, nc + 1):
        V[1][c] = cdiv(R[I[1]][c], pivot)
    zc = col(J[1])
    for i in range(1, nr + 1):
        R[i][J[1]] = zc[i - 1]
        U[i][1] = R[i][J[1]]
    norm_prec = 0.
    v2 = 0.
    for i in range(1, nr + 1):
        v2 = v2 + cabs(U[i][1]) ** 2
    nu = math.sqrt(v2)
    v2 = 0.
    for c in range(1, nc + 1):
        v2 = v2 + cabs(V[1][c]) ** 2
    nv = math.sqrt(v2)
    NF[1] = math.sqrt(norm_prec ** 2 + nu ** 2 * nv ** 2)
    tmp = [0.0 if i == I[1] else cabs(R[i][J[1]]) for i in range(1, nr + 1)]
    I[2] = maxloc(tmp)
    k = 2
    go = True
    while go and k <= itmax:
        Ik = I[k]
        prod = [0j] * (nc + 1)
        for l in range(1, k):
            for c in range(1, nc + 1):
                p = cmul(U[Ik][l], V[l][c])
                prod[c] = complex(prod[c].real + p.real, prod[c].imag + p.imag)
        zr = row(Ik)
        for c in range(1, nc + 1):
            R[Ik][c] = complex(zr[c - 1].real - prod[c].real, zr[c - 1].imag - prod[c].imag)
        tmp = [0.0 if c in J[1:k] else cabs(R[Ik][c]) for c in range(1, nc + 1)]
        J[k] = maxloc(tmp)
        Jk = J[k]
        pivot = R[Ik][Jk]
        for c in range(1, nc + 1):
            V[k][c] = cdiv(R[Ik][c], pivot)
        prodc = [0j] * (nr + 1)
        for l in range(1, k):
            for i in range(1, nr + 1):
                p = cmul(V[l][Jk], U[i][l])
                prodc[i] = complex(prodc[i].real + p.real, prodc[i].imag + p.imag)
        zc = col(Jk)
        for i in range(1, nr + 1):
            R[i][Jk] = complex(zc[i - 1].real - prodc[i].real, zc[i - 1].imag - prodc[i].imag)
            U[i][k] = R[i][Jk]
        norm_prec = NF[k - 1]
        v2 = 0.
        for i in range(1, nr + 1):
            v2 = v2 + cabs(U[i][k]) ** 2
        nu = math.sqrt(v2)
        v2 = 0.
        for c in range(1, nc + 1):
            v2 = v2 + cabs(V[k][c]) ** 2
        nv = math.sqrt(v2)
        suv = 0.
        for nj in range(1, k):
            su = sv = 0j
            for i in range(1, nr + 1):
                p = cmul(U[i][nj], U[i][k])
                su = complex(su.real + p.real, su.imag + p.imag)
            for c in range(1, nc + 1):
                p = cmul(V[k][c], V[nj][c])
                sv = complex(sv.real + p.real, sv.imag + p.imag)
            suv = suv + cabs(su) * cabs(sv)
        NF[k] = math.sqrt(norm_prec ** 2 + 2 * suv + nu ** 2 * nv ** 2)
        res = (nu * nv) / NF[k]
        if res <= eps:
            go = False
        else:
            tmp = [0.0 if i in I[1:k + 1] else cabs(R[i][J[k]]) for i in range(1, nr + 1)]
            I[k + 1] = maxloc(tmp)
            k = k + 1
    Uo = [[U[i][l] for l in range(1, itmax + 1)] for i in range(1, nr + 1)]
    Vo = [[V[l][c] for c in range(1, nc + 1)] for l in range(1, itmax + 1)]
    return k, Uo, Vo


def main():
    Z = block()
    out = {"cases": []}
    for case in CASES:
        k, U, V = aca(Z, case["eps"], case["itmax"])
        out["cases"].append(dict(case, k=k, U=[[[z.real, z.imag] for z in r] for r in U],
                                 V=[[[z.real, z.imag] for z in r] for r in V]))
    with open(os.path.join(HERE, "golden_aca.json"), "w") as fh:
        json.dump(out, fh)
    print("wrote golden_aca.json:", [c["k"] for c in out["cases"]])


if __name__ == "__main__":
    main()
