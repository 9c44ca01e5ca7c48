"""Generate tests/golden/golden_q.json: known answers of the orientation-averaging
step from a second, independent restatement.

The reference (Fortran) cannot run here and ships no outputs, so -- as for
golden_small.json -- the fixtures come from a plain-Python restatement written
straight from the Fortran with 1-based lists and numpy.float32 scalars for every
real(4) variable:
  qag / qage / qk61 / qsort     src/quadpack.f90:1-890 (QUADPACK QAG, key 6,
                                modified to sample a gridded integrand)
  getAdaptiveQuadPts2           src/Numerical_Integration.f90:213-245
  trap_2Dc                      src/Numerical_Integration.f90:251-305
  getTxRxIndex                  src/get_trans_Receiv.f90:690-713
  Compute_Scattering_Quantities_1 / _2   src/Compute_Scattering_Quantities.f90:1-1012
The C oracle (oracle/midas_oracle_q.c) must reproduce them exactly; the GPU
kernels are compared with the C oracle.  The Gauss-Kronrod table is read from
the oracle source (its values are pinned separately: the rule integrates
polynomials to degree 91 exactly).  Inputs are rebuilt from seeds by inputs().

Run:  python tests/golden/make_golden_q.py
"""
import json
import math
import os
import re

import numpy as np

F = np.float32
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PI = float(np.arccos(F(-1.0)))          # Acos(-1.) in single precision (src/Initialization.f90:39)
EPS = F(np.finfo(np.float32).eps)
TINY = F(np.finfo(np.float32).tiny)


def _table(name):
    src = open(os.path.join(ROOT, "oracle", "midas_oracle_q.c")).read()
    m = re.search(r"GK61_" + name + r"\[\d+\]\s*=\s*\{([^}]*)\}", src)
    return [None] + [F(float(v.strip().rstrip("f"))) for v in m.group(1).split(",") if v.strip()]


XGK, WGK, WG = _table("X"), _table("WK"), _table("WG")     # 1-based like the Fortran data


def nint(x):
    x = float(x)
    return int(math.floor(x + 0.5)) if x >= 0 else -int(math.floor(-x + 0.5))


def qk61(nth, f, a0, b0, a, b):
    """(result, abserr, resabs, resasc); f is 1-based."""
    def sample(x):
        i = nint((x * F(nth - 1)) / (b0 - a0)) + 1
        assert 1 <= i <= nth
        return F(f[i])
    centr = F(0.5) * (b + a)
    hlgth = F(0.5) * (b - a)
    dhlgth = abs(hlgth)
    resg = F(0.0)
    fc = sample(centr)
    resk = WGK[31] * fc
    resabs = abs(resk)
    fv1, fv2 = [None] * 31, [None] * 31
    for jq in range(1, 16):
        jtw = jq * 2
        absc = hlgth * XGK[jtw]
        fval1, fval2 = sample(centr - absc), sample(centr + absc)
        fv1[jtw], fv2[jtw] = fval1, fval2
        fsum = fval1 + fval2
        resg = resg + WG[jq] * fsum
        resk = resk + WGK[jtw] * fsum
        resabs = resabs + WGK[jtw] * (abs(fval1) + abs(fval2))
    for jq in range(1, 16):
        jtwm1 = jq * 2 - 1
        absc = hlgth * XGK[jtwm1]
        fval1, fval2 = sample(centr - absc), sample(centr + absc)
        fv1[jtwm1], fv2[jtwm1] = fval1, fval2
        fsum = fval1 + fval2
        resk = resk + WGK[jtwm1] * fsum
        resabs = resabs + WGK[jtwm1] * (abs(fval1) + abs(fval2))
    reskh = resk * F(0.5)
    resasc = WGK[31] * abs(fc - reskh)
    for jq in range(1, 31):
        resasc = resasc + WGK[jq] * (abs(fv1[jq] - reskh) + abs(fv2[jq] - reskh))
    result = resk * hlgth
    resabs = resabs * dhlgth
    resasc = resasc * dhlgth
    abserr = abs((resk - resg) * hlgth)
    if resasc != F(0.0) and abserr != F(0.0):
        t = (F(200.0) * abserr) / resasc
        abserr = resasc * min(F(1.0), t * np.sqrt(t))    # (.)**1.5 as t*sqrt(t)
    if resabs > TINY / (F(50.0) * EPS):
        abserr = max((EPS * F(50.0)) * resabs, abserr)
    return result, abserr, resabs, resasc


def qsort(limit, last, maxerr, elist, iord, nrmax):
    """Returns (maxerr, ermax, nrmax); elist, iord 1-based, iord updated in place."""
    if last <= 2:
        iord[1], iord[2] = 1, 2
    else:
        errmax = elist[maxerr]
        for _ in range(nrmax - 1):
            isucc = iord[nrmax - 1]
            if errmax <= elist[isucc]:
                break
            iord[nrmax] = isucc
            nrmax -= 1
        jupbn = last
        if limit // 2 + 2 < last:
            jupbn = limit + 3 - last
        errmin = elist[last]
        jbnd = jupbn - 1
        ibeg = nrmax + 1
        found = None
        for i in range(ibeg, jbnd + 1):
            isucc = iord[i]
            if elist[isucc] <= errmax:
                found = i
                break
            iord[i - 1] = isucc
        if found is None:
            iord[jbnd] = maxerr
            iord[jupbn] = last
        else:
            i = found
            iord[i - 1] = maxerr
            k = jbnd
            placed = False
            for _ in range(i, jbnd + 1):
                isucc = iord[k]
                if errmin < elist[isucc]:
                    iord[k + 1] = last
                    placed = True
                    break
                iord[k + 1] = isucc
                k -= 1
            if not placed:
                iord[i] = last
    maxerr = iord[nrmax]
    return maxerr, elist[maxerr], nrmax


def qag(n, f, a0, b0):
    """getAdaptiveQuadPts2 on a 1-based column f of n samples over [a0, b0] (radians)."""
    limit, epsabs, epsrel = 500, F(0.0), F(0.001)
    a, b = F(a0), F(b0)
    alist, blist, rlist, elist = ([F(0.0)] * (limit + 1) for _ in range(4))
    iord = [0] * (limit + 1)
    ier = 0
    alist[1], blist[1] = a, b
    result, abserr, defabs, resabs = qk61(n, f, a, b, a, b)
    rlist[1], elist[1], iord[1] = result, abserr, 1
    errbnd = max(epsabs, epsrel * abs(result))
    if abserr <= F(50.0) * EPS * defabs and errbnd < abserr:
        ier = 2
    if ier != 0 or (abserr <= errbnd and abserr != resabs) or abserr == F(0.0):
        return float(result)
    errmax, maxerr, area, errsum, nrmax, iroff1, iroff2 = abserr, 1, result, abserr, 1, 0, 0
    c = F(6.0)
    last = 1
    for last in range(2, limit + 1):
        a1 = alist[maxerr]
        b1 = F(0.5) * (alist[maxerr] + blist[maxerr])
        a2, b2 = b1, blist[maxerr]
        area1, error1, _, defab1 = qk61(n, f, a, b, a1, b1)
        area2, error2, _, defab2 = qk61(n, f, a, b, a2, b2)
        area12 = area1 + area2
        erro12 = error1 + error2
        errsum = errsum + erro12 - errmax
        area = area + area12 - rlist[maxerr]
        if defab1 != error1 and defab2 != error2:
            if abs(rlist[maxerr] - area12) <= F(1.0e-5) * abs(area12) and F(0.99) * errmax <= erro12:
                iroff1 += 1
            if 10 < last and errmax < erro12:
                iroff2 += 1
        rlist[maxerr] = area1
        rlist[last] = area2
        errbnd = max(epsabs, epsrel * abs(area))
        if errbnd < errsum:
            if iroff1 >= 6 or iroff2 >= 20:
                ier = 2
            if last == limit:
                ier = 1
            if max(abs(a1), abs(b2)) <= (F(1.0) + c * F(1.0e3) * EPS) * (abs(a2) + F(1.0e4) * TINY):
                ier = 3
        if error2 <= error1:
            alist[last] = a2
            blist[maxerr] = b1
            blist[last] = b2
            elist[maxerr] = error1
            elist[last] = error2
        else:
            alist[maxerr] = a2
            alist[last] = a1
            blist[last] = b1
            rlist[maxerr] = area2
            rlist[last] = area1
            elist[maxerr] = error2
            elist[last] = error1
        maxerr, errmax, nrmax = qsort(limit, last, maxerr, elist, iord, nrmax)
        if ier != 0 or errsum <= errbnd:
            break
    s = F(0.0)
    for k in range(1, last + 1):
        s = s + rlist[k]
    return float(s)


def trap_2d(f, a, b, c, d, nx, ny):
    """trap_2Dc; f[(i, j)] 1-based."""
    hx, hy = (b - a) / float(nx - 1), (d - c) / float(ny - 1)
    s = f[1, 1] + f[1, ny] + f[nx, 1] + f[nx, ny]
    for i in range(2, nx):
        s = s + 2.0 * (f[i, 1] + f[i, ny])
    for j in range(2, ny):
        s = s + 2.0 * (f[1, j] + f[nx, j])
    for i in range(2, nx):
        for j in range(2, ny):
            s = s + 4.0 * f[i, j]
    return 0.25 * hx * hy * s


def getTxRxIndex(th_list, ph_list, th, ph):
    eps = float(F(1e-2))
    for ii in range(len(th_list)):
        if abs(th_list[ii] - th) <= eps and abs(ph_list[ii] - ph) <= eps:
            return ii + 1
    return 0


def absq(z):
    a = math.sqrt(z.real * z.real + z.imag * z.imag)
    return a * a


def unique(v):
    out = []
    for x in v:
        if not any(y == x for y in out):
            out.append(x)
    return out


# ---------------------------------------------------------------------------
# inputs (rebuilt by the test from these seeds)
# ---------------------------------------------------------------------------
CASES = [
    {"quad_tr": "un", "quad_rx": "un", "tr": (3, 3), "rx": (19, 5), "seed": 1, "intf": 0},
    {"quad_tr": "gl", "quad_rx": "tr", "tr": (3, 2), "rx": (10, 4), "seed": 2, "intf": 1},
    {"quad_tr": "rf", "quad_rx": "rf", "tr": (5, 1), "rx": (7, 1), "seed": 3, "intf": 0},
    {"quad_tr": "lb", "quad_rx": "lb", "tr": (4, 1), "rx": (4, 1), "seed": 4, "intf": 0, "same": True},
    {"quad_tr": "un", "quad_rx": "sd", "tr": (3, 3), "rx": (9, 1), "seed": 5, "intf": 0},
]
QAG_COLUMNS = [("sin181", 181, 0.0, PI), ("step37", 37, 0.0, 2 * PI), ("rand19", 19, 0.0, PI),
               ("ramp2", 2, 0.0, PI)]


def qag_column(name):
    n = dict((c[0], c[1]) for c in QAG_COLUMNS)[name]
    if name.startswith("sin"):
        return np.sin(np.linspace(0.0, math.pi, n))
    if name.startswith("step"):
        return np.where(np.arange(n) < n // 3, 1.0, 0.25)
    if name.startswith("rand"):
        return np.random.default_rng(7).uniform(0.0, 1.0, n)
    return np.linspace(0.0, 1.0, n)


def _grid(th0, th1, nth, ph0, ph1, nph):
    sth = 0.0 if nth == 1 else (th1 - th0) / (nth - 1)
    sph = 0.0 if nph == 1 else (ph1 - ph0) / (nph - 1)
    th = [th0 + k * sth for k in range(nth)]
    ph = [ph0 + k * sph for k in range(nph)]
    return [t for p in ph for t in th], [p for p in ph for t in th]


def inputs(case):
    """Direction sets, S (nrx_tot x 4 ntr), cross sections, weights and dm, k0 of a case."""
    rng = np.random.default_rng(case["seed"])
    nt, np_ = case["tr"]
    nr, nrp = case["rx"]
    grid_rules = ("un", "tr", "gl")
    if case["quad_tr"] in grid_rules:
        tth, tph = _grid(0.0, 180.0, nt, 0.0, 360.0, np_)
    else:
        tth, tph = list(rng.uniform(0, 180, nt)), list(rng.uniform(0, 360, nt))
    if case["quad_rx"] in grid_rules:
        rth, rph = _grid(0.0, 180.0, nr, 0.0, 360.0, nrp)
    elif case.get("same"):
        rth, rph = list(tth), list(tph)
    else:
        rth, rph = list(rng.uniform(0, 180, nr)), list(rng.uniform(0, 360, nr))
    ntr, nrx = nt * np_, nr * nrp
    if case["quad_tr"] in grid_rules:     # get_trans_Receiv: add the missing forward / backward receivers
        for t in range(ntr):
            for a, b in ((tth[t], tph[t]), (180.0 - tth[t], math.fmod(tph[t] + 180.0, 360.0))):
                if getTxRxIndex(rth[:nrx], rph[:nrx], a, b) == 0:
                    rth.append(a)
                    rph.append(b)
    else:                                 # positional blocks (src/get_trans_Receiv.f90:527-550)
        if not case.get("same"):
            rth += tth
            rph += tph
        rth += [180.0 - t for t in tth]
        rph += [math.fmod(p + 180.0, 360.0) for p in tph]
    nrx_tot = len(rth)
    S = (rng.uniform(0.2, 2.0, (nrx_tot, 4 * ntr)) * np.exp(2j * math.pi * rng.random((nrx_tot, 4 * ntr))))
    cext, cabs = rng.uniform(5, 7, ntr), rng.uniform(0.2, 0.4, ntr)
    w_tr = w_rx = None
    if case["quad_tr"] == "gl":
        w_tr = rng.uniform(0.3, 0.6, nt + np_)
    if case["quad_tr"] == "lb":
        w_tr = rng.uniform(0.1, 0.3, ntr)
    if case["quad_rx"] == "gl":
        w_rx = rng.uniform(0.1, 0.2, nr + nrp)
    if case["quad_rx"] == "lb":
        w_rx = w_tr if case.get("same") else rng.uniform(0.1, 0.3, nrx)
    return dict(tth=np.array(tth), tph=np.array(tph), rth=np.array(rth), rph=np.array(rph), S=S, cext=cext,
                cabs=cabs, w_tr=w_tr, w_rx=w_rx, dm=2.0, k0=2.0)


def quantities(case, inp):
    """Compute_Scattering_Quantities_1 / _2: (q_dir rows [Q_ext, Q_abs, Q_sca, Q_bks, g], q_avg)."""
    qt, qr = case["quad_tr"], case["quad_rx"]
    nt, np_ = case["tr"]
    nr, nrp = case["rx"]
    ntr, nrx = nt * np_, nr * nrp
    tth, tph, rth, rph, S = inp["tth"], inp["tph"], inp["rth"], inp["rph"], inp["S"]
    k_0, dm = inp["k0"], inp["dm"]
    ap, X = dm / 2., k_0 * dm / 2.
    lists = ("sd", "lb", "rf")
    q = {k: [0.0] * (ntr + 1) for k in ("ext", "sca", "bks", "g", "exti", "absi")}
    if qr not in lists:
        thv, phv = unique(list(rth[:nrx])), unique(list(rph[:nrx]))
        th_min, th_max = thv[0] * PI / 180., thv[-1] * PI / 180.
        ph_min, ph_max = phv[0] * PI / 180., phv[-1] * PI / 180.
        Sn = max((ph_max - ph_min), 1.) * (math.cos(th_min) - math.cos(th_max))
    for kkt in range(1, ntr + 1):
        th_i, ph_i = tth[kkt - 1], tph[kkt - 1]
        Kix = -math.sin(th_i * PI / 180.) * math.cos(ph_i * PI / 180.)
        Kiy = -math.sin(th_i * PI / 180.) * math.sin(ph_i * PI / 180.)
        Kiz = -math.cos(th_i * PI / 180.)
        col = lambda k: S[:, 4 * (kkt - 1) + k - 1]   # k = 1..4: vv, vh, hv, hh
        if qt in lists:
            same = ntr == nrx
            ind_fw = kkt if same and qr in ("lb", "sd") else nrx + kkt
            ind_bk = nrx + kkt if same and qr in lists else nrx + ntr + kkt
        else:
            ind_fw = getTxRxIndex(rth, rph, th_i, ph_i)
            ind_bk = getTxRxIndex(rth, rph, 180. - th_i, math.fmod(ph_i + 180., 360.))
        q["ext"][kkt] = (2 / (X * X)) * (abs(col(4)[ind_fw - 1].imag) + abs(col(1)[ind_fw - 1].imag))
        q["exti"][kkt] = inp["cext"][kkt - 1] / (PI * ap ** 2.)
        if qr in lists:
            fxy, fxyg = [], []
            for kkr in range(1, nrx + 1):
                s_it = absq(col(4)[kkr - 1]) + absq(col(1)[kkr - 1]) + absq(col(2)[kkr - 1]) + absq(col(3)[kkr - 1])
                v = inp["w_rx"][kkr - 1] * s_it if qr == "lb" else s_it
                th_s, ph_s = rth[kkr - 1], rph[kkr - 1]
                Ksx = -math.sin(th_s * PI / 180.) * math.cos(ph_s * PI / 180.)
                Ksy = -math.sin(th_s * PI / 180.) * math.sin(ph_s * PI / 180.)
                Ksz = -math.cos(th_s * PI / 180.)
                cg = Kix * Ksx + Kiy * Ksy + Kiz * Ksz
                fxy.append(v)
                fxyg.append(v * cg)
            sf, sg = 0.0, 0.0
            for v in fxy:
                sf = sf + v
            for v in fxyg:
                sg = sg + v
            if qr == "lb":
                c_sca = 1. / (2 * k_0 ** 2) * sf
                q["sca"][kkt] = (4 * PI) / (2 * PI * X * X) * sf
                q["g"][kkt] = 1. / (2. * k_0 ** 2. * c_sca) * sg
            else:
                q_sd = (4 * PI / nrx) * sf
                c_sca = 1. / (2 * k_0 ** 2) * q_sd
                q["sca"][kkt] = 1 / (2 * PI * X * X) * q_sd
                q["g"][kkt] = 1. / (2. * k_0 ** 2. * c_sca) * (4 * PI / nrx) * sg
        else:
            fxy, fxyg = {}, {}
            for ii in range(1, nr + 1):
                th_s = thv[ii - 1]
                s = math.sin(th_s * PI / 180.)
                for jj in range(1, nrp + 1):
                    kkr = (jj - 1) * nr + ii
                    s_it = (absq(col(4)[kkr - 1]) + absq(col(1)[kkr - 1]) + absq(col(2)[kkr - 1])
                            + absq(col(3)[kkr - 1]))
                    fxy[ii, jj] = s_it * s
                    ph_s = phv[jj - 1]
                    Ksx = -math.sin(th_s * PI / 180.) * math.cos(ph_s * PI / 180.)
                    Ksy = -math.sin(th_s * PI / 180.) * math.sin(ph_s * PI / 180.)
                    Ksz = -math.cos(th_s * PI / 180.)
                    cg = Kix * Ksx + Kiy * Ksy + Kiz * Ksz
                    fxyg[ii, jj] = s_it * s * cg
            if qr == "un":
                vals = []
                for f in (fxy, fxyg):
                    fy = [None] + [qag(nr, [None] + [f[i, jj] for i in range(1, nr + 1)], th_min, th_max)
                                   for jj in range(1, nrp + 1)]
                    vals.append(qag(nrp, fy, ph_min, ph_max) if nrp > 1 else fy[1])
                q_int, q_g = vals
            else:
                q_int = trap_2d(fxy, th_min, th_max, ph_min, ph_max, nr, nrp)
                q_g = trap_2d(fxyg, th_min, th_max, ph_min, ph_max, nr, nrp)
            c_sca = 1. / (2 * k_0 ** 2) * q_int
            q["sca"][kkt] = 2. / (Sn * X * X) * q_int
            q["g"][kkt] = 1. / (2. * k_0 ** 2. * c_sca) * q_g
        q["absi"][kkt] = inp["cabs"][kkt - 1] / (PI * ap ** 2.)
        q["bks"][kkt] = (1. / (2. * PI * X * X)) * (absq(col(1)[ind_bk - 1]) + absq(col(4)[ind_bk - 1])
                                                    + absq(col(2)[ind_bk - 1]) + absq(col(3)[ind_bk - 1]))
    Qext = q["exti"] if case["intf"] == 1 else q["ext"]
    Qs = [Qext, q["absi"], q["sca"], q["bks"], q["g"]]
    q_dir = [[Qs[k][t] for k in range(5)] for t in range(1, ntr + 1)]
    if ntr == 1:
        return q_dir, q_dir[0]
    if qt in lists:
        avg = []
        for k in range(5):
            s = 0.0
            if qt == "lb":
                for t in range(1, ntr + 1):
                    s = s + inp["w_tr"][t - 1] * Qs[k][t]
            else:
                for t in range(1, ntr + 1):
                    s = s + Qs[k][t]
                s = s / ntr
            avg.append(s)
        return q_dir, avg
    thv_t, phv_t = unique(list(tth)), unique(list(tph))
    t0, t1 = thv_t[0] * PI / 180., thv_t[-1] * PI / 180.
    p0, p1 = phv_t[0] * PI / 180., phv_t[-1] * PI / 180.
    Snt = max((p1 - p0), 1.) * (math.cos(t0) - math.cos(t1))
    avg = []
    for k in range(5):
        G = {}
        for ii in range(1, nt + 1):
            s = math.sin(tth[ii - 1] * PI / 180.)
            for jj in range(1, np_ + 1):
                G[ii, jj] = Qs[k][(jj - 1) * nt + ii] * s
        if qt == "gl":
            wth, wph = inp["w_tr"][:nt], inp["w_tr"][nt:]
            qi = 0.0
            for ii in range(1, nt + 1):
                for jj in range(1, np_ + 1):
                    qi = qi + wph[jj - 1] * wth[ii - 1] * G[ii, jj]
        elif qt == "un":
            fy = [None] + [qag(nt, [None] + [G[i, jj] for i in range(1, nt + 1)], t0, t1) for jj in range(1, np_ + 1)]
            qi = qag(np_, fy, p0, p1) if np_ > 1 else fy[1]
        else:
            qi = trap_2d(G, t0, t1, p0, p0, nt, np_)
        avg.append(1. / Snt * qi)
    return q_dir, avg


def main():
    out = {"qag": [], "cases": []}
    for name, n, a0, b0 in QAG_COLUMNS:
        f = qag_column(name)
        out["qag"].append({"name": name, "a0": a0, "b0": b0, "result": qag(n, [None] + list(f), a0, b0)})
    for case in CASES:
        q_dir, q_avg = quantities(case, inputs(case))
        out["cases"].append(dict(case, q_dir=q_dir, q_avg=q_avg))
    with open(os.path.join(HERE, "golden_q.json"), "w") as fh:
        json.dump(out, fh, indent=1)
    print(f"wrote golden_q.json: {len(out['qag'])} quadratures, {len(out['cases'])} cases")


if __name__ == "__main__":
    main()
