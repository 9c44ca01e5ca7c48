/*
 * midas_oracle_q.c -- CPU restatement of the orientation-averaging post-processing
 * of MIDAS: efficiencies per incident direction and their averages.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker of
 * midas_gpu_scattering_quantities; the product never links or calls it.
 *
 * Follows (paths relative to the reference project root):
 *   Compute_Scattering_Quantities_1   src/Compute_Scattering_Quantities.f90:1-589
 *     (grid transmitters: 'un', 'tr', 'gl')
 *   Compute_Scattering_Quantities_2   src/Compute_Scattering_Quantities.f90:593-1012
 *     (transmitter lists: 'sd', 'rf', 'lb')
 *   getAdaptiveQuadPts2               src/Numerical_Integration.f90:213-245
 *   qag / qage / qk61 / qsort         src/quadpack.f90:1-110, 112-484, 486-728, 730-890
 *     (QUADPACK's QAG with the 61-point Gauss-Kronrod rule, modified by the
 *      reference to read the integrand from a sampled grid by nearest index)
 *   trap_2Dc                          src/Numerical_Integration.f90:251-305
 *   getTxRxIndex                      src/get_trans_Receiv.f90:690-713
 *   Unique1DArray_D                   src/Compute_Scattering_Quantities.f90:1014-1042
 *
 * Parity status: UNPINNED (the Fortran reference cannot run here).
 *
 * Precision rules restated from the reference:
 *   - the adaptive quadrature runs in real(4): the interval ends, the sampled
 *     values, every sum and the error estimates are single precision, and the
 *     sample index is nint(x*(n-1)/(b0-a0))+1 evaluated in single precision;
 *   - QUADPACK's (.)**1.5 is evaluated as t*sqrt(t) (both correctly rounded);
 *   - Fortran SUM is a left-to-right sum;
 *   - |z|**2. is (sqrt(re*re+im*im))**2 with each operation rounded;
 *   - Pi = Acos(-1.) in single precision (src/Initialization.f90:39);
 *   - getTxRxIndex's tolerance ErrAngEps = 1e-2 is a single-precision literal.
 * This file must be compiled with -ffp-contract=off.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

static double q_pi(void) { return (double)acosf(-1.0f); }

/* Integration rules (NumIntType_t / NumIntType_r). */
enum { Q_UN = 0, Q_TR = 1, Q_GL = 2, Q_SD = 3, Q_LB = 4, Q_RF = 5 };

/* Status codes returned by or_scattering_quantities. */
enum { QS_OK = 0, QS_ARG = 1, QS_FWD = 2, QS_BKW = 3, QS_INDEX = 4 };

/* ------------------------------------------------------------------------- */
/* Gauss-Kronrod 30/61 rule on [-1, 1] (QUADPACK qk61): Kronrod abscissae     */
/* x[0..30] in decreasing order (x[2j-1], j = 1..15, are the 30-point Gauss    */
/* abscissae), their Kronrod weights, and the Gauss weights.  Single precision */
/* as in the reference.                                                        */
/* ------------------------------------------------------------------------- */
static const float GK61_X[31] = {
    0.9994844100504906f, 0.9968934840746495f, 0.9916309968704046f, 0.9836681232797472f,
    0.9731163225011263f, 0.9600218649683075f, 0.9443744447485600f, 0.9262000474292743f,
    0.9055733076999078f, 0.8825605357920527f, 0.8572052335460611f, 0.8295657623827684f,
    0.7997278358218391f, 0.7677774321048262f, 0.7337900624532268f, 0.6978504947933158f,
    0.6600610641266270f, 0.6205261829892429f, 0.5793452358263617f, 0.5366241481420199f,
    0.4924804678617786f, 0.4470337695380892f, 0.4004012548303944f, 0.3527047255308781f,
    0.3040732022736251f, 0.2546369261678898f, 0.2045251166823099f, 0.1538699136085835f,
    0.1028069379667370f, 0.05147184255531770f, 0.0f};
static const float GK61_WK[31] = {
    0.001389013698677008f, 0.003890461127099884f, 0.006630703915931292f, 0.009273279659517763f,
    0.01182301525349634f, 0.01436972950704580f, 0.01692088918905327f, 0.01941414119394238f,
    0.02182803582160919f, 0.02419116207808060f, 0.02650995488233310f, 0.02875404876504129f,
    0.03090725756238776f, 0.03298144705748373f, 0.03497933802806002f, 0.03688236465182123f,
    0.03867894562472759f, 0.04037453895153596f, 0.04196981021516425f, 0.04345253970135607f,
    0.04481480013316266f, 0.04605923827100699f, 0.04718554656929915f, 0.04818586175708713f,
    0.04905543455502978f, 0.04979568342707421f, 0.05040592140278235f, 0.05088179589874961f,
    0.05122154784925877f, 0.05142612853745903f, 0.05149472942945157f};
static const float GK61_WG[15] = {
    0.007968192496166606f, 0.01846646831109096f, 0.02878470788332337f, 0.03879919256962705f,
    0.04840267283059405f, 0.05749315621761907f, 0.06597422988218050f, 0.07375597473770521f,
    0.08075589522942022f, 0.08689978720108298f, 0.09212252223778613f, 0.09636873717464426f,
    0.09959342058679527f, 0.1017623897484055f, 0.1028526528935588f};

#define QAG_LIMIT 500

/* Sample of the gridded integrand nearest to x: f(nint(x*(n-1)/(b0-a0))+1)
 * (src/quadpack.f90:621-627).  An index outside the grid (the reference reads
 * past its array) sets *bad and reads the nearest end. */
static float q_sample(const double *f, int n, float span, float x, int *bad)
{
    const float t = (x * (float)(n - 1)) / span;
    long i;
    if (!(t > -1e9f && t < 1e9f)) { *bad = 1; i = 1; }
    else i = lroundf(t) + 1;
    if (i < 1) { *bad = 1; i = 1; }
    if (i > n) { *bad = 1; i = n; }
    return (float)f[i - 1];
}

/* qk61 (src/quadpack.f90:486-728) over the gridded integrand f[0..n-1] that
 * spans [a0, b0]. */
static void q_qk61(const double *f, int n, float a0, float b0, float a, float b,
                   float *result, float *abserr, float *resabs, float *resasc, int *bad)
{
    const float span = b0 - a0;
    const float centr = 0.5f * (b + a), hlgth = 0.5f * (b - a), dhlgth = fabsf(hlgth);
    float fv1[30], fv2[30];
    const float fc = q_sample(f, n, span, centr, bad);
    float resg = 0.0f, resk = GK61_WK[30] * fc, ra = fabsf(resk);
    for (int j = 1; j <= 15; ++j) {                 /* Gauss abscissae */
        const int k = 2 * j - 1;
        const float absc = hlgth * GK61_X[k];
        const float f1 = q_sample(f, n, span, centr - absc, bad);
        const float f2 = q_sample(f, n, span, centr + absc, bad);
        fv1[k] = f1; fv2[k] = f2;
        const float fs = f1 + f2;
        resg = resg + GK61_WG[j - 1] * fs;
        resk = resk + GK61_WK[k] * fs;
        ra = ra + GK61_WK[k] * (fabsf(f1) + fabsf(f2));
    }
    for (int j = 1; j <= 15; ++j) {                 /* Kronrod-only abscissae */
        const int k = 2 * j - 2;
        const float absc = hlgth * GK61_X[k];
        const float f1 = q_sample(f, n, span, centr - absc, bad);
        const float f2 = q_sample(f, n, span, centr + absc, bad);
        fv1[k] = f1; fv2[k] = f2;
        const float fs = f1 + f2;
        resk = resk + GK61_WK[k] * fs;
        ra = ra + GK61_WK[k] * (fabsf(f1) + fabsf(f2));
    }
    const float reskh = resk * 0.5f;
    float rasc = GK61_WK[30] * fabsf(fc - reskh);
    for (int k = 0; k < 30; ++k) rasc = rasc + GK61_WK[k] * (fabsf(fv1[k] - reskh) + fabsf(fv2[k] - reskh));
    *result = resk * hlgth;
    ra = ra * dhlgth;
    rasc = rasc * dhlgth;
    float err = fabsf((resk - resg) * hlgth);
    if (rasc != 0.0f && err != 0.0f) {
        float t = (200.0f * err) / rasc;
        t = t * sqrtf(t);
        err = rasc * (t < 1.0f ? t : 1.0f);
    }
    if (ra > FLT_MIN / (50.0f * FLT_EPSILON)) {
        const float e2 = (FLT_EPSILON * 50.0f) * ra;
        err = e2 > err ? e2 : err;
    }
    *abserr = err;
    *resabs = ra;
    *resasc = rasc;
}

/* qsort (src/quadpack.f90:730-890), QUADPACK's qpsrt: keeps iord[] (1-based
 * interval numbers) in decreasing order of the error estimates elist[] and
 * returns the interval to bisect next. */
static void q_qpsrt(int limit, int last, int *maxerr, float *ermax, const float *elist, int *iord, int *nrmax)
{
#define EL(i) elist[(i) - 1]   /* 1-based views */
#define IO(i) iord[(i) - 1]
    int i, k;
    if (last <= 2) {
        IO(1) = 1;
        IO(2) = 2;
        goto done;
    }
    {
        const float errmax = EL(*maxerr);
        const int trips = *nrmax - 1;
        for (int t = 0; t < trips; ++t) {
            const int isucc = IO(*nrmax - 1);
            if (errmax <= EL(isucc)) break;
            IO(*nrmax) = isucc;
            *nrmax -= 1;
        }
        int jupbn = last;
        if (limit / 2 + 2 < last) jupbn = limit + 3 - last;
        const float errmin = EL(last);
        const int jbnd = jupbn - 1, ibeg = *nrmax + 1;
        for (i = ibeg; i <= jbnd; ++i) {
            const int isucc = IO(i);
            if (EL(isucc) <= errmax) goto found;
            IO(i - 1) = isucc;
        }
        IO(jbnd) = *maxerr;
        IO(jupbn) = last;
        goto done;
    found:
        IO(i - 1) = *maxerr;
        k = jbnd;
        for (int j = i; j <= jbnd; ++j) {
            const int isucc = IO(k);
            if (errmin < EL(isucc)) {
                IO(k + 1) = last;
                goto done;
            }
            IO(k + 1) = isucc;
            k -= 1;
        }
        IO(i) = last;
    }
done:
    *maxerr = IO(*nrmax);
    *ermax = EL(*maxerr);
#undef EL
#undef IO
}

/* getAdaptiveQuadPts2 -> qag -> qage with key 6 (src/Numerical_Integration.f90:213-245,
 * src/quadpack.f90:1-484): epsabs = 0, epsrel = 1e-3, limit 500.  Returns the
 * real(4) result; *neval / *ier / *bad report the run. */
static float q_qag(const double *f, int n, double a0d, double b0d, int *neval, int *ier, int *bad)
{
    const float epsabs = 0.0f, epsrel = 0.001f;
    const float a = (float)a0d, b = (float)b0d;
    float alist[QAG_LIMIT], blist[QAG_LIMIT], rlist[QAG_LIMIT], elist[QAG_LIMIT];
    int iord[QAG_LIMIT];
    float result, abserr, defabs, resabs;
    *ier = 0;
    alist[0] = a; blist[0] = b; rlist[0] = 0.0f; elist[0] = 0.0f; iord[0] = 0;
    q_qk61(f, n, a, b, a, b, &result, &abserr, &defabs, &resabs, bad);
    const float c = 6.0f;   /* keyf */
    int last = 1;
    rlist[0] = result; elist[0] = abserr; iord[0] = 1;
    float errbnd = epsrel * fabsf(result);
    if (epsabs > errbnd) errbnd = epsabs;
    if (abserr <= (50.0f * FLT_EPSILON) * defabs && errbnd < abserr) *ier = 2;
    if (*ier != 0 || (abserr <= errbnd && abserr != resabs) || abserr == 0.0f) {
        *neval = 61;
        return result;
    }
    float errmax = abserr, area = result, errsum = abserr;
    int maxerr = 1, nrmax = 1, iroff1 = 0, iroff2 = 0, nsub = 0;
    for (last = 2; last <= QAG_LIMIT; ++last) {
        const float a1 = alist[maxerr - 1];
        const float b1 = 0.5f * (alist[maxerr - 1] + blist[maxerr - 1]);
        const float a2 = b1, b2 = blist[maxerr - 1];
        float area1, error1, defab1, area2, error2, defab2, ra;
        q_qk61(f, n, a, b, a1, b1, &area1, &error1, &ra, &defab1, bad);
        q_qk61(f, n, a, b, a2, b2, &area2, &error2, &ra, &defab2, bad);
        nsub++;
        const float area12 = area1 + area2, erro12 = error1 + error2;
        errsum = (errsum + erro12) - errmax;
        area = (area + area12) - rlist[maxerr - 1];
        if (defab1 != error1 && defab2 != error2) {
            if (fabsf(rlist[maxerr - 1] - area12) <= 1.0e-5f * fabsf(area12) && 0.99f * errmax <= erro12) iroff1++;
            if (10 < last && errmax < erro12) iroff2++;
        }
        rlist[maxerr - 1] = area1;
        rlist[last - 1] = area2;
        errbnd = epsrel * fabsf(area);
        if (epsabs > errbnd) errbnd = epsabs;
        if (errbnd < errsum) {
            if (6 <= iroff1 || 20 <= iroff2) *ier = 2;
            if (last == QAG_LIMIT) *ier = 1;
            const float m = fabsf(a1) > fabsf(b2) ? fabsf(a1) : fabsf(b2);
            if (m <= (1.0f + (c * 1.0e3f) * FLT_EPSILON) * (fabsf(a2) + 1.0e4f * FLT_MIN)) *ier = 3;
        }
        if (error2 <= error1) {
            alist[last - 1] = a2;
            blist[maxerr - 1] = b1;
            blist[last - 1] = b2;
            elist[maxerr - 1] = error1;
            elist[last - 1] = error2;
        } else {
            alist[maxerr - 1] = a2;
            alist[last - 1] = a1;
            blist[last - 1] = b1;
            rlist[maxerr - 1] = area2;
            rlist[last - 1] = area1;
            elist[maxerr - 1] = error2;
            elist[last - 1] = error1;
        }
        q_qpsrt(QAG_LIMIT, last, &maxerr, &errmax, elist, iord, &nrmax);
        if (*ier != 0 || errsum <= errbnd) break;
    }
    float s = 0.0f;
    for (int k = 0; k < last; ++k) s = s + rlist[k];
    *neval = 61 * (2 * nsub + 1);
    return s;
}

/* trap_2Dc (src/Numerical_Integration.f90:251-305), f nx x ny column-major. */
static double q_trap2d(const double *f, double a, double b, double c, double d, int nx, int ny)
{
    const double hx = (b - a) / (double)(nx - 1), hy = (d - c) / (double)(ny - 1);
#define F(i, j) f[(size_t)((j) - 1) * nx + ((i) - 1)]
    double s = F(1, 1) + F(1, ny) + F(nx, 1) + F(nx, ny);
    for (int i = 2; i <= nx - 1; ++i) s = s + 2.0 * (F(i, 1) + F(i, ny));
    for (int j = 2; j <= ny - 1; ++j) s = s + 2.0 * (F(1, j) + F(nx, j));
    for (int i = 2; i <= nx - 1; ++i)
        for (int j = 2; j <= ny - 1; ++j) s = s + 4.0 * F(i, j);
#undef F
    return 0.25 * hx * hy * s;
}

/* Unique1DArray_D (src/Compute_Scattering_Quantities.f90:1014-1042): the
 * distinct values in order of first appearance.  Returns their number. */
static int q_unique(const double *v, int n, double *out)
{
    int m = 0;
    for (int i = 0; i < n; ++i) {
        int seen = 0;
        for (int j = 0; j < i && !seen; ++j) seen = (v[j] == v[i]);
        if (!seen) out[m++] = v[i];
    }
    return m;
}

/* getTxRxIndex (src/get_trans_Receiv.f90:690-713): first direction within
 * ErrAngEps of (th, ph), 1-based, 0 when none. */
static int q_txrx_index(int n, const double *th, const double *ph, double t, double p)
{
    const double eps = (double)1e-2f;
    for (int i = 0; i < n; ++i)
        if (fabs(th[i] - t) <= eps && fabs(ph[i] - p) <= eps) return i + 1;
    return 0;
}

static inline double q_abs2(const double *z)
{
    const double a = sqrt(z[0] * z[0] + z[1] * z[1]);
    return a * a;
}

/* The QAG of one column (exported for the unit tests). */
double or_qag_grid(const double *f, int n, double a0, double b0, int *neval, int *ier, int *bad)
{
    *bad = 0;
    return (double)q_qag(f, n, a0, b0, neval, ier, bad);
}

/* Quantities per incident direction and their orientation averages.
 *   quad_tr, quad_rx: integration rules (Q_UN .. Q_RF) of the transmitters and
 *     receivers; ntr_theta x ntr_phi transmitters (theta fastest; a list has
 *     ntr_phi = 1), nrx_theta x nrx_phi grid receivers (a list: nrx_phi = 1),
 *     then nrx_tot - nrx extra (forward / backward) receivers;
 *   S: nrx_tot x 4ntr complex, column-major, columns Vv, Vh, Hv, Hh per
 *     transmitter; cext, cabs: cross sections per transmitter;
 *   w_tr / w_rx: quadrature weights ('gl': theta weights then phi weights;
 *     'lb': one per direction), else NULL;
 *   q_dir (5 x ntr): Q_ext, Q_abs, Q_sca, Q_bks, g per transmitter, as the
 *     reference's Qidtable; q_avg (5): their averages.
 * Returns QS_OK or the first error. */
int or_scattering_quantities(int quad_tr, int quad_rx, int ntr_theta, int ntr_phi, int nrx_theta, int nrx_phi,
                             int nrx_tot, double dm, double k0, int cext_intfields,
                             const double *tr_th, const double *tr_ph, const double *rx_th, const double *rx_ph,
                             const double *S, const double *cext, const double *cabs,
                             const double *w_tr, const double *w_rx, double *q_dir, double *q_avg)
{
    const double Pi = q_pi();
    const int ntr = ntr_theta * ntr_phi, nrx = nrx_theta * nrx_phi;
    const int list_tr = (quad_tr == Q_SD || quad_tr == Q_RF || quad_tr == Q_LB);
    const int list_rx = (quad_rx == Q_SD || quad_rx == Q_RF || quad_rx == Q_LB);
    if (ntr < 1 || nrx < 1 || nrx_tot < nrx) return QS_ARG;
    if (list_tr && !list_rx) return QS_ARG;                        /* _2 reads only lists */
    if (!list_tr && quad_rx == Q_RF) return QS_ARG;
    const double ap = dm / 2., X = k0 * dm / 2.;
    int status = QS_OK, bad = 0;

    double *rtv = NULL, *rpv = NULL, Sn = 0;
    if (!list_rx) {                                                /* :144-166 */
        rtv = (double *)malloc(sizeof(double) * nrx);
        rpv = (double *)malloc(sizeof(double) * nrx);
        if (q_unique(rx_th, nrx, rtv) != nrx_theta || q_unique(rx_ph, nrx, rpv) != nrx_phi) {
            free(rtv); free(rpv);
            return QS_ARG;
        }
        const double th0 = rtv[0] * Pi / 180., th1 = rtv[nrx_theta - 1] * Pi / 180.;
        const double ph0 = rpv[0] * Pi / 180., ph1 = rpv[nrx_phi - 1] * Pi / 180.;
        Sn = fmax(ph1 - ph0, 1.) * (cos(th0) - cos(th1));
    }
    double *fx = (double *)malloc(sizeof(double) * nrx), *fg = (double *)malloc(sizeof(double) * nrx);
    double *fy = (double *)malloc(sizeof(double) * nrx_phi), *fyg = (double *)malloc(sizeof(double) * nrx_phi);
    double *Qe = (double *)malloc(sizeof(double) * 7 * ntr);
    double *Qs = Qe + ntr, *Qb = Qe + 2 * ntr, *Qg = Qe + 3 * ntr, *Qei = Qe + 4 * ntr, *Qai = Qe + 5 * ntr;

    for (int t = 0; t < ntr && status == QS_OK; ++t) {
        const double thi = tr_th[t], phi_ = tr_ph[t];
        const double kix = -sin(thi * Pi / 180.) * cos(phi_ * Pi / 180.);
        const double kiy = -sin(thi * Pi / 180.) * sin(phi_ * Pi / 180.);
        const double kiz = -cos(thi * Pi / 180.);
        const double *Sv = S + 2 * (size_t)nrx_tot * (4 * t + 0), *Svh = S + 2 * (size_t)nrx_tot * (4 * t + 1);
        const double *Shv = S + 2 * (size_t)nrx_tot * (4 * t + 2), *Sh = S + 2 * (size_t)nrx_tot * (4 * t + 3);
        /* forward and backward receivers */
        int ifw, ibk;
        if (!list_tr) {                                            /* :204-210, :410-418 */
            ifw = q_txrx_index(nrx_tot, rx_th, rx_ph, thi, phi_);
            ibk = q_txrx_index(nrx_tot, rx_th, rx_ph, 180. - thi, fmod(phi_ + 180., 360.));
        } else {                                                   /* :760-764, :866-870 */
            const int same = (ntr == nrx);
            ifw = (same && (quad_rx == Q_LB || quad_rx == Q_SD)) ? t + 1 : nrx + t + 1;
            ibk = (same && list_rx) ? nrx + t + 1 : nrx + ntr + t + 1;
            if (ifw > nrx_tot) ifw = 0;
            if (ibk > nrx_tot) ibk = 0;
        }
        if (!ifw) { status = QS_FWD; break; }
        if (!ibk) { status = QS_BKW; break; }
        Qe[t] = (2 / (X * X)) * (fabs(Sh[2 * (ifw - 1) + 1]) + fabs(Sv[2 * (ifw - 1) + 1]));
        Qei[t] = cext[t] / (Pi * (ap * ap));
        /* integrands */
        for (int r = 0; r < nrx; ++r) {
            const double sit = ((q_abs2(Sh + 2 * r) + q_abs2(Sv + 2 * r)) + q_abs2(Svh + 2 * r)) + q_abs2(Shv + 2 * r);
            double ths, phs, s = 1.0;
            if (list_rx) { ths = rx_th[r]; phs = rx_ph[r]; }
            else { ths = rtv[r % nrx_theta]; phs = rpv[r / nrx_theta]; s = sin(ths * Pi / 180.); }
            const double ksx = -sin(ths * Pi / 180.) * cos(phs * Pi / 180.);
            const double ksy = -sin(ths * Pi / 180.) * sin(phs * Pi / 180.);
            const double ksz = -cos(ths * Pi / 180.);
            const double cg = (kix * ksx + kiy * ksy) + kiz * ksz;
            if (list_rx) {
                fx[r] = quad_rx == Q_LB ? w_rx[r] * sit : sit;
                fg[r] = fx[r] * cg;
            } else {
                fx[r] = sit * s;
                fg[r] = (sit * s) * cg;
            }
        }
        const double c2 = 2 * (k0 * k0);
        if (quad_rx == Q_LB) {                                     /* :214-227 */
            double qs = 0, qg = 0;
            for (int r = 0; r < nrx; ++r) qs = qs + fx[r];
            for (int r = 0; r < nrx; ++r) qg = qg + fg[r];
            const double csca = 1. / c2 * qs;
            Qs[t] = (4 * Pi) / (2 * Pi * X * X) * qs;
            Qg[t] = 1. / (c2 * csca) * qg;
        } else if (quad_rx == Q_SD || quad_rx == Q_RF) {           /* :228-250 */
            double qs = 0, qg = 0;
            for (int r = 0; r < nrx; ++r) qs = qs + fx[r];
            for (int r = 0; r < nrx; ++r) qg = qg + fg[r];
            const double qsd = (4 * Pi / nrx) * qs;
            const double csca = 1. / c2 * qsd;
            Qs[t] = 1 / (2 * Pi * X * X) * qsd;
            Qg[t] = 1. / (c2 * csca) * (4 * Pi / nrx) * qg;
        } else {
            const double th0 = rtv[0] * Pi / 180., th1 = rtv[nrx_theta - 1] * Pi / 180.;
            const double ph0 = rpv[0] * Pi / 180., ph1 = rpv[nrx_phi - 1] * Pi / 180.;
            double q, qg;
            if (quad_rx == Q_GL) {                                 /* :276-305 */
                const double *wth = w_rx, *wph = w_rx + nrx_theta;
                q = 0; qg = 0;
                for (int i = 0; i < nrx_theta; ++i)
                    for (int j = 0; j < nrx_phi; ++j) q = q + wph[j] * wth[i] * fx[(size_t)j * nrx_theta + i];
                for (int i = 0; i < nrx_theta; ++i)
                    for (int j = 0; j < nrx_phi; ++j) qg = qg + wph[j] * wth[i] * fg[(size_t)j * nrx_theta + i];
            } else if (quad_rx == Q_UN) {                          /* :307-345 */
                int ne, ier;
                for (int j = 0; j < nrx_phi; ++j) fy[j] = (double)q_qag(fx + (size_t)j * nrx_theta, nrx_theta, th0, th1, &ne, &ier, &bad);
                q = nrx_phi > 1 ? (double)q_qag(fy, nrx_phi, ph0, ph1, &ne, &ier, &bad) : fy[0];
                for (int j = 0; j < nrx_phi; ++j) fyg[j] = (double)q_qag(fg + (size_t)j * nrx_theta, nrx_theta, th0, th1, &ne, &ier, &bad);
                qg = nrx_phi > 1 ? (double)q_qag(fyg, nrx_phi, ph0, ph1, &ne, &ier, &bad) : fyg[0];
            } else {                                               /* 'tr', :347-355 */
                q = q_trap2d(fx, th0, th1, ph0, ph1, nrx_theta, nrx_phi);
                qg = q_trap2d(fg, th0, th1, ph0, ph1, nrx_theta, nrx_phi);
            }
            const double csca = 1. / c2 * q;
            Qs[t] = 2. / (Sn * X * X) * q;
            Qg[t] = 1. / (c2 * csca) * qg;
        }
        Qai[t] = cabs[t] / (Pi * (ap * ap));                       /* :362-364 */
        Qb[t] = (1. / (2. * Pi * X * X)) * (((q_abs2(Sv + 2 * (ibk - 1)) + q_abs2(Sh + 2 * (ibk - 1)))
                                             + q_abs2(Svh + 2 * (ibk - 1))) + q_abs2(Shv + 2 * (ibk - 1)));
    }
    if (status == QS_OK && bad) status = QS_INDEX;
    if (status == QS_OK) {
        double *Q[5] = {cext_intfields == 1 ? Qei : Qe, Qai, Qs, Qb, Qg};   /* :383-392 */
        for (int t = 0; t < ntr; ++t)
            for (int k = 0; k < 5; ++k) q_dir[5 * t + k] = Q[k][t];
        if (ntr == 1) {
            for (int k = 0; k < 5; ++k) q_avg[k] = Q[k][0];
        } else if (list_tr) {                                      /* :941-968 */
            for (int k = 0; k < 5; ++k) {
                double s = 0;
                if (quad_tr == Q_LB)
                    for (int t = 0; t < ntr; ++t) s = s + w_tr[t] * Q[k][t];
                else {
                    for (int t = 0; t < ntr; ++t) s = s + Q[k][t];
                    s = s / ntr;
                }
                q_avg[k] = s;
            }
        } else {                                                   /* :436-520 */
            double *tv = (double *)malloc(sizeof(double) * ntr), *pv = (double *)malloc(sizeof(double) * ntr);
            const int nth = q_unique(tr_th, ntr, tv), nph = q_unique(tr_ph, ntr, pv);
            const double th0 = tv[0] * Pi / 180., th1 = tv[nth - 1] * Pi / 180.;
            const double ph0 = pv[0] * Pi / 180., ph1 = pv[nph - 1] * Pi / 180.;
            const double Snt = fmax(ph1 - ph0, 1.) * (cos(th0) - cos(th1));
            double *G = (double *)malloc(sizeof(double) * ntr), *gy = (double *)malloc(sizeof(double) * ntr_phi);
            for (int k = 0; k < 5; ++k) {
                for (int i = 0; i < ntr_theta; ++i) {
                    const double s = sin(tr_th[i] * Pi / 180.);
                    for (int j = 0; j < ntr_phi; ++j) G[(size_t)j * ntr_theta + i] = Q[k][(size_t)j * ntr_theta + i] * s;
                }
                double q;
                if (quad_tr == Q_GL) {
                    const double *wth = w_tr, *wph = w_tr + ntr_theta;
                    q = 0;
                    for (int i = 0; i < ntr_theta; ++i)
                        for (int j = 0; j < ntr_phi; ++j) q = q + wph[j] * wth[i] * G[(size_t)j * ntr_theta + i];
                } else if (quad_tr == Q_UN) {
                    int ne, ier;
                    for (int j = 0; j < ntr_phi; ++j)
                        gy[j] = (double)q_qag(G + (size_t)j * ntr_theta, ntr_theta, th0, th1, &ne, &ier, &bad);
                    q = ntr_phi > 1 ? (double)q_qag(gy, ntr_phi, ph0, ph1, &ne, &ier, &bad) : gy[0];
                } else {
                    /* 'tr' passes TrPh_min as both phi limits (:509-513) */
                    q = q_trap2d(G, th0, th1, ph0, ph0, ntr_theta, ntr_phi);
                }
                q_avg[k] = 1. / Snt * q;
            }
            free(G); free(gy); free(tv); free(pv);
            if (bad) status = QS_INDEX;
        }
    }
    free(fx); free(fg); free(fy); free(fyg); free(Qe);
    free(rtv); free(rpv);
    return status;
}
