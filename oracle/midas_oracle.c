/*
 * midas_oracle.c -- CPU restatement of the MIDAS VIE-MoM / CBFM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests, the
 * smoke check and the CPU-baseline leg of bench.py load it (through
 * oracle/oracle.py) to compare against the GPU library.  The product path
 * (libmidas_gpu.so) never links, loads or calls anything in this directory.
 *
 * Parity status: UNPINNED.  The reference is Fortran + Intel MKL and cannot be
 * built in this environment, and it ships no golden outputs, so this
 * restatement is pinned only by an independent Python restatement of the same
 * formulas (tests/golden) and by physics checks (reciprocity, Mie).
 *
 * Every routine below follows one reference routine; the file:line of each is
 * given in its comment (paths relative to the reference project root).
 *
 * Precision rules restated from the reference:
 *   - Pi = Acos(-1.) is evaluated in single precision and widened
 *     (src/Initialization.f90:39); every angle and k-dependent factor uses it.
 *   - 1./3. and 2./3. are single-precision literals (src/SetCellsParams.f90:37,44).
 *   - Green_s_tr_partial / computeBlockRow / computeBlockCol / SR_* hold
 *     Gr, Tau, f_kapChe and F in complex(4) locals
 *     (src/Green_functions.f90:109,310,583,919,1134): each assignment to such a
 *     local rounds to float, `3.*Tau` is a single-precision product, and the
 *     final -F*f_kapChe is a complex(4) product.  The reference is built with
 *     ifort -O3 for x86-64 (src/Makefile:7, no -x flag), i.e. SSE2 without FMA,
 *     so complex(4) products are evaluated as re = a.re*b.re - a.im*b.im,
 *     im = a.re*b.im + a.im*b.re with every float operation rounded.  This file
 *     must be compiled with -ffp-contract=off so the same holds on any host.
 *   - Incident_Field keeps K11x/K11y/K11z and Ex/Ey/Ez in complex(4) locals
 *     (src/Incident_Field.f90:17).
 *   - compute_Green_s_tr_single_element / Incident_Field_single_element (the
 *     MoM path) are FP64 throughout (src/Compute_EFields_MoM.f90:446-447,544).
 *
 * Layout conventions (same as the reference): the unknown index of cell c
 * (0-based) and component p in {x,y,z} is 3c+p; matrices are column-major;
 * complex numbers are interleaved (re, im) doubles.  RHS column tr is the V
 * polarisation of transmitter tr and column tr+NTr its H polarisation
 * (src/Compute_EFields_MoM.f90:557-563).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* Pi = Acos(-1.) in single precision, widened (src/Initialization.f90:39). */
static double ref_pi(void) { return (double)acosf(-1.0f); }

double or_pi(void) { return ref_pi(); }

/* ------------------------------------------------------------------------- */
/* complex helpers with an explicit evaluation order                          */
/* ------------------------------------------------------------------------- */
typedef struct { double re, im; } zc8;   /* complex(8) */
typedef struct { float re, im; } zc4;    /* complex(4) */

static inline zc8 z8(double re, double im) { zc8 z; z.re = re; z.im = im; return z; }
static inline zc8 z8mul(zc8 a, zc8 b) { return z8(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static inline zc8 z8of4(zc4 a) { return z8((double)a.re, (double)a.im); }
static inline zc4 z4of8(zc8 a) { zc4 r; r.re = (float)a.re; r.im = (float)a.im; return r; }
/* |z| of a complex(4) value, rounded like the GPU kernels' (see zabs below) */
static inline float absf4(float re, float im) { return sqrtf(re * re + im * im); }
static inline zc4 z4mul(zc4 a, zc4 b)
{
    /* complex(4) product without FMA: every float operation rounded. */
    float p1 = a.re * b.re, p2 = a.im * b.im, p3 = a.re * b.im, p4 = a.im * b.re;
    zc4 r; r.re = p1 - p2; r.im = p3 + p4; return r;
}

/* ------------------------------------------------------------------------- */
/* a1: SetCellsParams (src/SetCellsParams.f90:31-49)                          */
/* ------------------------------------------------------------------------- */
void or_set_cells_params(int n, const double *sc, const double *eps, double k0,
                         double *a_n, double *che, double *znnpp, double *kappa)
{
    const double Pi = ref_pi();
    const double third = (double)(1.0f / 3.0f);   /* 1./3. (single) */
    const double two3 = (double)(2.0f / 3.0f);    /* 2./3. (single) */
    for (int c = 0; c < n; ++c) {
        double a = sc[c] * pow(0.75 / Pi, third);                    /* :37 */
        zc8 ch = z8(eps[2 * c] - 1.0, eps[2 * c + 1]);               /* :40 */
        double ka = k0 * a;
        zc8 e = z8(cos(ka), sin(ka));                                /* exp(J*k_0*a_n) */
        zc8 t = z8(two3 * e.re, two3 * e.im);
        t = z8mul(t, z8(1.0, -ka));                                  /* *(1. - J*k_0*a_n) */
        t.re -= 1.0;                                                 /* - 1 */
        zc8 zn = z8mul(t, ch);                                       /* :44 */
        double kap = 4 * Pi * (sin(ka) - ka * cos(ka)) / pow(k0, 3.0); /* :48 */
        if (a_n) a_n[c] = a;
        che[2 * c] = ch.re; che[2 * c + 1] = ch.im;
        znnpp[2 * c] = zn.re; znnpp[2 * c + 1] = zn.im;
        kappa[c] = kap;
    }
}

/* ------------------------------------------------------------------------- */
/* Dyad kernels                                                              */
/* ------------------------------------------------------------------------- */
/* FP64 dyad, all nine components: compute_Green_s_tr_single_element
 * (src/Compute_EFields_MoM.f90:474-519).  out[p*3+q] = Z(row comp p, col comp q). */
static void dyad8(double rx, double ry, double rz, double k0, double Pi, zc8 fk, zc8 out[9])
{
    double r = sqrt(rx * rx + ry * ry + rz * rz);
    double kr = k0 * r;
    double den = 4 * Pi * (r * r);
    zc8 Gr = z8(cos(kr) / den, sin(kr) / den);
    zc8 Tau = z8(-(1 / r), k0);
    double k2 = k0 * k0;
    double d[3] = {rx, ry, rz};
    zc8 F[9];
    for (int p = 0; p < 3; ++p) {
        double s = 3. * (d[p] * d[p]) / (r * r);
        zc8 in = z8((Tau.re + k2 * (r - d[p] * d[p] / r)) - s * Tau.re, Tau.im - s * Tau.im);
        F[p * 4] = z8mul(Gr, in);
    }
    /* off-diagonal: Gr/r * (rp*rq) * (-k0^2 - 3*Tau/r) */
    zc8 w = z8(-k2 - (3. * Tau.re) / r, -((3. * Tau.im) / r));
    int pq[3][2] = {{0, 1}, {1, 2}, {0, 2}};
    for (int t = 0; t < 3; ++t) {
        int p = pq[t][0], q = pq[t][1];
        double rr = d[p] * d[q];
        zc8 g = z8((Gr.re / r) * rr, (Gr.im / r) * rr);
        zc8 f = z8mul(g, w);
        F[p * 3 + q] = f; F[q * 3 + p] = f;
    }
    for (int i = 0; i < 9; ++i) {
        zc8 z = z8mul(F[i], fk);
        out[i] = z8(-z.re, -z.im);
    }
}

/* complex(4)-local dyad: Green_s_tr_partial (src/Green_functions.f90:139-167),
 * identical arithmetic in computeBlockRow/Col (:941-956,:1155-1171) and
 * SR_Green_s_tr_partial (:342-379). */
static void dyad4(double rx, double ry, double rz, double k0, double Pi, zc4 fk4, zc8 out[9])
{
    double r = sqrt(rx * rx + ry * ry + rz * rz);
    double kr = k0 * r;
    double den = 4 * Pi * (r * r);
    zc4 Gr4 = z4of8(z8(cos(kr) / den, sin(kr) / den));   /* Gr_mn = exp(J*k_0*r)/(4*Pi*r**2.) */
    zc4 Tau4 = z4of8(z8(-(1 / r), k0));                   /* Tau_mn = J*k_0 - 1/r */
    zc8 Gr = z8of4(Gr4), Tau = z8of4(Tau4);
    double k2 = k0 * k0;
    double d[3] = {rx, ry, rz};
    zc4 F4[9];
    for (int p = 0; p < 3; ++p) {
        double s = 3. * (d[p] * d[p]) / (r * r);
        zc8 in = z8((Tau.re + k2 * (r - d[p] * d[p] / r)) - s * Tau.re, Tau.im - s * Tau.im);
        F4[p * 4] = z4of8(z8mul(Gr, in));
    }
    /* 3.*Tau_mn is a complex(4) product (single precision). */
    float t3r = 3.0f * Tau4.re, t3i = 3.0f * Tau4.im;
    zc8 w = z8(-k2 - (double)t3r / r, -((double)t3i / r));
    int pq[3][2] = {{0, 1}, {1, 2}, {0, 2}};
    for (int t = 0; t < 3; ++t) {
        int p = pq[t][0], q = pq[t][1];
        double rr = d[p] * d[q];
        zc8 g = z8((Gr.re / r) * rr, (Gr.im / r) * rr);
        zc4 f = z4of8(z8mul(g, w));
        F4[p * 3 + q] = f; F4[q * 3 + p] = f;
    }
    for (int i = 0; i < 9; ++i) {
        zc4 z = z4mul(F4[i], fk4);                   /* -F*f_kapChe in complex(4) */
        out[i] = z8(-(double)z.re, -(double)z.im);
    }
}

static inline zc8 fk8_of(const double *kappa, const double *che, int c)
{
    return z8(kappa[c] * che[2 * c], kappa[c] * che[2 * c + 1]);
}
static inline zc4 fk4_of(const double *kappa, const double *che, int c)
{
    return z4of8(fk8_of(kappa, che, c));
}

/* ------------------------------------------------------------------------- */
/* a2: MoM element fill (src/Compute_EFields_MoM.f90:433-523)                 */
/* Fills rows [r0,r0+nr) x cols [c0,c0+nc) (0-based unknown indices) of the   */
/* 3n x 3n matrix into Z (nr x nc, column-major, leading dimension nr).       */
/* ------------------------------------------------------------------------- */
void or_mom_fill(int n, const double *x, const double *y, const double *z,
                 const double *kappa, const double *che, const double *znnpp, double k0,
                 int r0, int nr, int c0, int nc, double *Z)
{
    const double Pi = ref_pi();
    (void)n;
#pragma omp parallel for schedule(dynamic, 4)
    for (int jj = 0; jj < nc; ++jj) {
        int gj = c0 + jj, is = gj / 3, qc = gj % 3;
        zc8 fk = fk8_of(kappa, che, is);
        int last_io = -1; zc8 D[9];
        for (int ii = 0; ii < nr; ++ii) {
            int gi = r0 + ii, io = gi / 3, pc = gi % 3;
            double *o = Z + 2 * ((size_t)jj * nr + ii);
            if (io == is) {
                if (pc == qc) { o[0] = 1 - znnpp[2 * is]; o[1] = -znnpp[2 * is + 1]; }
                else { o[0] = 0; o[1] = 0; }
                continue;
            }
            if (io != last_io) {
                dyad8(x[io] - x[is], y[io] - y[is], z[io] - z[is], k0, Pi, fk, D);
                last_io = io;
            }
            o[0] = D[pc * 3 + qc].re; o[1] = D[pc * 3 + qc].im;
        }
    }
}

/* ------------------------------------------------------------------------- */
/* a3: Incident_Field_single_element, FP64 (src/Compute_EFields_MoM.f90:529-598) */
/* V is 3n x 2*ntr, column-major.                                             */
/* ------------------------------------------------------------------------- */
void or_mom_rhs(int n, const double *x, const double *y, const double *z, double k0,
                int ntr, const double *th, const double *ph, double *V)
{
    const double Pi = ref_pi();
#pragma omp parallel for schedule(static)
    for (int kk = 0; kk < 2 * ntr; ++kk) {
        int vh = kk < ntr ? 0 : 1;
        int t = vh ? kk - ntr : kk;
        double tr = th[t] * Pi / 180., pr = ph[t] * Pi / 180.;
        double kx = k0 * cos(tr), ky = k0 * sin(tr) * cos(pr), kz = k0 * sin(tr) * sin(pr);
        double st = sin(tr), ct = cos(tr), sp = sin(pr), cp = cos(pr);
        for (int c = 0; c < n; ++c) {
            zc8 e = z8mul(z8mul(z8(cos(kx * x[c]), sin(kx * x[c])), z8(cos(ky * y[c]), sin(ky * y[c]))),
                          z8(cos(kz * z[c]), sin(kz * z[c])));
            zc8 o[3];
            if (!vh) {
                o[0] = z8(-(e.re * st), -(e.im * st));            /* - e*sin(theta) */
                o[1] = z8((e.re * ct) * cp, (e.im * ct) * cp);    /* e*cos(theta)*cos(phi) */
                o[2] = z8((e.re * ct) * sp, (e.im * ct) * sp);    /* e*cos(theta)*sin(phi) */
            } else {
                o[0] = z8(0, 0);
                o[1] = z8(-(e.re * sp), -(e.im * sp));            /* - e*sin(phi) */
                o[2] = z8(e.re * cp, e.im * cp);                  /* e*cos(phi) */
            }
            double *w = V + 2 * ((size_t)kk * 3 * n + 3 * c);
            for (int p = 0; p < 3; ++p) { w[2 * p] = o[p].re; w[2 * p + 1] = o[p].im; }
        }
    }
}

/* ------------------------------------------------------------------------- */
/* a8: Incident_Field with complex(4) locals (src/Incident_Field.f90:1-63)    */
/* Cells are idx[0..n) (or 0..n-1 when idx is NULL); transmitters tr0..tr1-1.*/
/* E is 3n x 2*(tr1-tr0) column-major: V block then H block.                  */
/* ------------------------------------------------------------------------- */
void or_incident_c4(int n, const int *idx, const double *x, const double *y, const double *z,
                    double k0, const double *th, const double *ph, int tr0, int tr1, double *E)
{
    const double Pi = ref_pi();
    int nt = tr1 - tr0;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nt; ++t) {
        double tr = th[tr0 + t] * Pi / 180., pr = ph[tr0 + t] * Pi / 180.;
        float kx = (float)(k0 * cos(tr));
        float ky = (float)(k0 * sin(tr) * cos(pr));
        float kz = (float)(k0 * sin(tr) * sin(pr));
        double st = sin(tr), ct = cos(tr), sp = sin(pr), cp = cos(pr);
        for (int c = 0; c < n; ++c) {
            int g = idx ? idx[c] : c;
            double ax = (double)kx * x[g], ay = (double)ky * y[g], az = (double)kz * z[g];
            zc8 e = z8mul(z8mul(z8(cos(ax), sin(ax)), z8(cos(ay), sin(ay))), z8(cos(az), sin(az)));
            double *ov = E + 2 * ((size_t)t * 3 * n + 3 * c);
            double *oh = E + 2 * ((size_t)(t + nt) * 3 * n + 3 * c);
            /* V: Ex = -e*sin(th), Ey = e*cos(th)*cos(ph), Ez = e*cos(th)*sin(ph) */
            zc4 ex = z4of8(z8(-(e.re * st), -(e.im * st)));
            zc4 ey = z4of8(z8((e.re * ct) * cp, (e.im * ct) * cp));
            zc4 ez = z4of8(z8((e.re * ct) * sp, (e.im * ct) * sp));
            ov[0] = ex.re; ov[1] = ex.im; ov[2] = ey.re; ov[3] = ey.im; ov[4] = ez.re; ov[5] = ez.im;
            /* H: Ex = 0, Ey = -e*sin(ph), Ez = e*cos(ph) */
            zc4 hy = z4of8(z8(-(e.re * sp), -(e.im * sp)));
            zc4 hz = z4of8(z8(e.re * cp, e.im * cp));
            oh[0] = 0; oh[1] = 0; oh[2] = hy.re; oh[3] = hy.im; oh[4] = hz.re; oh[5] = hz.im;
        }
    }
}

/* ------------------------------------------------------------------------- */
/* a8: Incident_Field_Spherical (src/Incident_Field.f90:65-166), the CBF      */
/* excitation of type_iws = 2/3 (src/Compute_EFields_CBFME.f90:365-368).      */
/* Cells are idx[0..n) in the order of Cells_in; transmitters tr0..tr1-1.     */
/* Centre Cbl = the cells' mean centroid (sum in cell order, :91-93), Rbl the */
/* largest centroid distance (:94), Rsource = 10 max(Rbl, 2 Pi / k0) (:97).   */
/* Per cell: the complex(4) local phase = exp(i k0 R) / R rounded to float    */
/* (:139), local angles acos(ux), atan2(uz, uy) in FP64 (:142-143), and the   */
/* complex(4) field components from complex(4) x real(8) products evaluated   */
/* left to right in FP64 and rounded at assignment (:146-157).                */
/* E is 3n x 2*(tr1-tr0) column-major: V block then H block.                  */
/* ------------------------------------------------------------------------- */
void or_incident_sph(int n, const int *idx, const double *x, const double *y, const double *z,
                     double k0, const double *th, const double *ph, int tr0, int tr1, double *E)
{
    const double Pi = ref_pi();
    double cx = 0, cy = 0, cz = 0;
    for (int c = 0; c < n; ++c) {
        int g = idx ? idx[c] : c;
        cx += x[g];
        cy += y[g];
        cz += z[g];
    }
    cx /= n;
    cy /= n;
    cz /= n;
    double m2 = 0;
    for (int c = 0; c < n; ++c) {
        int g = idx ? idx[c] : c;
        double dx = x[g] - cx, dy = y[g] - cy, dz = z[g] - cz;
        double d2 = dx * dx + dy * dy + dz * dz;
        if (d2 > m2) m2 = d2;
    }
    const double rbl = sqrt(m2);
    const double lam = 2.0 * Pi / k0;
    const double rsrc = 10.0 * (rbl > lam ? rbl : lam);
    int nt = tr1 - tr0;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nt; ++t) {
        double tr = th[tr0 + t] * Pi / 180., pr = ph[tr0 + t] * Pi / 180.;
        double xs = cx + rsrc * cos(tr);
        double ys = cy + rsrc * sin(tr) * cos(pr);
        double zs = cz + rsrc * sin(tr) * sin(pr);
        for (int c = 0; c < n; ++c) {
            int g = idx ? idx[c] : c;
            double dx = x[g] - xs, dy = y[g] - ys, dz = z[g] - zs;
            double R = sqrt(dx * dx + dy * dy + dz * dz);
            double ux = dx / R, uy = dy / R, uz = dz / R;
            double a = k0 * R;
            zc4 phs = z4of8(z8(cos(a) / R, sin(a) / R));
            double the = acos(ux), phi = atan2(uz, uy);
            double st = sin(the), ct = cos(the), sp = sin(phi), cp = cos(phi);
            double pre = phs.re, pim = phs.im;
            double *ov = E + 2 * ((size_t)t * 3 * n + 3 * c);
            double *oh = E + 2 * ((size_t)(t + nt) * 3 * n + 3 * c);
            /* V: Ex = -phase*sin(theta), Ey = phase*cos(theta)*cos(phi), Ez = phase*cos(theta)*sin(phi) */
            zc4 ex = z4of8(z8(-pre * st, -pim * st));
            zc4 ey = z4of8(z8((pre * ct) * cp, (pim * ct) * cp));
            zc4 ez = z4of8(z8((pre * ct) * sp, (pim * ct) * sp));
            ov[0] = ex.re; ov[1] = ex.im; ov[2] = ey.re; ov[3] = ey.im; ov[4] = ez.re; ov[5] = ez.im;
            /* H: Ex = 0, Ey = -phase*sin(phi), Ez = phase*cos(phi) */
            zc4 hy = z4of8(z8(-pre * sp, -pim * sp));
            zc4 hz = z4of8(z8(pre * cp, pim * cp));
            oh[0] = 0; oh[1] = 0; oh[2] = hy.re; oh[3] = hy.im; oh[4] = hz.re; oh[5] = hz.im;
        }
    }
}

/* ------------------------------------------------------------------------- */
/* a4: Green_s_tr_partial (src/Green_functions.f90:96-173)                    */
/* Z is 3n1 x 3n2 column-major.  Cells are identified by global index; equal  */
/* global indices give the self term 1 - Znnpp (the n_cell test, :125-127).   */
/* ------------------------------------------------------------------------- */
void or_green_partial(int n1, const int *idx1, int n2, const int *idx2,
                      const double *x, const double *y, const double *z,
                      const double *kappa, const double *che, const double *znnpp, double k0,
                      double *Z)
{
    const double Pi = ref_pi();
    size_t ld = 3 * (size_t)n1;
#pragma omp parallel for schedule(dynamic, 2)
    for (int js = 0; js < n2; ++js) {
        int s = idx2[js];
        zc4 fk = fk4_of(kappa, che, s);
        zc8 D[9];
        for (int io = 0; io < n1; ++io) {
            int o = idx1[io];
            if (o == s) {
                for (int p = 0; p < 3; ++p)
                    for (int q = 0; q < 3; ++q) {
                        double *w = Z + 2 * ((size_t)(3 * js + q) * ld + 3 * io + p);
                        if (p == q) { w[0] = 1 - znnpp[2 * s]; w[1] = -znnpp[2 * s + 1]; }
                        else { w[0] = 0; w[1] = 0; }
                    }
                continue;
            }
            dyad4(x[o] - x[s], y[o] - y[s], z[o] - z[s], k0, Pi, fk, D);
            for (int p = 0; p < 3; ++p)
                for (int q = 0; q < 3; ++q) {
                    double *w = Z + 2 * ((size_t)(3 * js + q) * ld + 3 * io + p);
                    w[0] = D[p * 3 + q].re; w[1] = D[p * 3 + q].im;
                }
        }
    }
}

/* Green_s_tr_partial_FN (src/Green_functions.f90:176-287): Frobenius norm of  */
/* the block without storing it.  homog = 1 scans Io >= Is only (:242-282).   */
/* Note the reference weights the off-diagonal dyad terms by 2 (:236-237).    */
double or_green_partial_fn(int n1, const int *idx1, int n2, const int *idx2, int homog,
                           const double *x, const double *y, const double *z,
                           const double *kappa, const double *che, const double *znnpp, double k0)
{
    const double Pi = ref_pi();
    double val = 0;
#pragma omp parallel for schedule(dynamic, 2) reduction(+ : val)
    for (int js = 0; js < n2; ++js) {
        int s = idx2[js];
        zc4 fk = fk4_of(kappa, che, s);
        float afk = absf4(fk.re, fk.im);
        int io0 = homog ? js : 0;
        double part = 0;
        for (int io = io0; io < n1; ++io) {
            int o = idx1[io];
            if (o == s) {
                double a = hypot(1 - znnpp[2 * s], -znnpp[2 * s + 1]);
                part += 3. * (a * a);
                continue;
            }
            /* the reference forms |F| from the complex(4) F, not from -F*f_kapChe */
            double rx = x[o] - x[s], ry = y[o] - y[s], rz = z[o] - z[s];
            double r = sqrt(rx * rx + ry * ry + rz * rz), kr = k0 * r, den = 4 * Pi * (r * r);
            zc4 Gr4 = z4of8(z8(cos(kr) / den, sin(kr) / den));
            zc4 Tau4 = z4of8(z8(-(1 / r), k0));
            zc8 Gr = z8of4(Gr4), Tau = z8of4(Tau4);
            double k2 = k0 * k0, d[3] = {rx, ry, rz};
            float aF[6];
            for (int p = 0; p < 3; ++p) {
                double sv = 3. * (d[p] * d[p]) / (r * r);
                zc4 f = z4of8(z8mul(Gr, z8((Tau.re + k2 * (r - d[p] * d[p] / r)) - sv * Tau.re, Tau.im - sv * Tau.im)));
                aF[p] = absf4(f.re, f.im);
            }
            float t3r = 3.0f * Tau4.re, t3i = 3.0f * Tau4.im;
            zc8 w = z8(-k2 - (double)t3r / r, -((double)t3i / r));
            int pq[3][2] = {{0, 1}, {1, 2}, {0, 2}};
            for (int t = 0; t < 3; ++t) {
                double rr = d[pq[t][0]] * d[pq[t][1]];
                zc4 f = z4of8(z8mul(z8((Gr.re / r) * rr, (Gr.im / r) * rr), w));
                aF[3 + t] = absf4(f.re, f.im);
            }
            /* (|Fxx|**2+2.*|Fxy|**2+2.*|Fxz|**2+|Fyy|**2+2.*|Fyz|**2+|Fzz|**2)*|f_kapChe|**2.: abs() of
             * a complex(4) is real(4), so the whole term is a single-precision expression (:236-237). */
            float t = aF[0] * aF[0] + 2.f * (aF[3] * aF[3]);
            t = t + 2.f * (aF[5] * aF[5]);
            t = t + aF[1] * aF[1];
            t = t + 2.f * (aF[4] * aF[4]);
            t = t + aF[2] * aF[2];
            part += (double)(t * (afk * afk));
        }
        val += part;
    }
    return sqrt(val);
}

/* ------------------------------------------------------------------------- */
/* a6: SR_Green_s_tr_partial (src/Green_functions.f90:290-562) as the dense   */
/* equivalent of the CSR matrix handed to PARDISO: entries with |g| above     */
/* threshold = |1 - Znnpp(first cell)| / fSR are kept, the rest are zero; the */
/* self 3x3 keeps only its diagonal.  homog = 1 stores only Is > Io and       */
/* PARDISO (mtype 6, complex symmetric) mirrors it; the mirror is applied.    */
/* Z (3s x 3s, column-major) may be NULL to count only.                       */
/* Returns nnz and (optionally) the Frobenius norm of the kept entries as     */
/* SR_Green_s_tr_partial_FN does (:564-806).                                  */
/* ------------------------------------------------------------------------- */
long or_sr_dense(int s_n, const int *idx, double fsr, int homog,
                 const double *x, const double *y, const double *z,
                 const double *kappa, const double *che, const double *znnpp, double k0,
                 double *Z, double *fn_out)
{
    const double Pi = ref_pi();
    size_t ld = 3 * (size_t)s_n;
    int c0 = idx[0];
    double vmax = hypot(1 - znnpp[2 * c0], -znnpp[2 * c0 + 1]);
    double thr = vmax / fsr;
    long nnz = 0;
    double g2 = 0;
    if (Z) memset(Z, 0, sizeof(double) * 2 * ld * ld);
#pragma omp parallel for schedule(dynamic, 2) reduction(+ : nnz, g2)
    for (int io = 0; io < s_n; ++io) {
        int o = idx[io];
        zc8 D[9];
        int is0 = homog ? io : 0;
        for (int is = is0; is < s_n; ++is) {
            int s = idx[is];
            if (is == io) {
                double a = hypot(1 - znnpp[2 * s], -znnpp[2 * s + 1]);
                for (int p = 0; p < 3; ++p) {
                    nnz += 1; g2 += a * a;
                    if (Z) {
                        double *w = Z + 2 * ((size_t)(3 * is + p) * ld + 3 * io + p);
                        w[0] = 1 - znnpp[2 * s]; w[1] = -znnpp[2 * s + 1];
                    }
                }
                continue;
            }
            dyad4(x[o] - x[s], y[o] - y[s], z[o] - z[s], k0, Pi, fk4_of(kappa, che, s), D);
            for (int p = 0; p < 3; ++p)
                for (int q = 0; q < 3; ++q) {
                    zc8 g = D[p * 3 + q];
                    /* abs(g) of a complex(4) value */
                    float af = absf4((float)g.re, (float)g.im);
                    double a = (double)af;
                    if (a > thr) {
                        nnz += 1; g2 += (double)(af * af);
                        if (Z) {
                            double *w = Z + 2 * ((size_t)(3 * is + q) * ld + 3 * io + p);
                            w[0] = g.re; w[1] = g.im;
                            if (homog) {
                                double *m = Z + 2 * ((size_t)(3 * io + p) * ld + 3 * is + q);
                                m[0] = g.re; m[1] = g.im;
                            }
                        }
                    }
                }
        }
    }
    if (fn_out) *fn_out = sqrt(g2);
    return nnz;
}

/* setfSR (src/getParameters_CBFM.f90:113-168): walk the fSR ladder until the */
/* relative Frobenius-norm change of the thresholded block is <= res_SR (%).  */
double or_set_fsr(int s_n, const int *idx, int homog, double res_sr,
                  const double *x, const double *y, const double *z,
                  const double *kappa, const double *che, const double *znnpp, double k0,
                  long *nnz_out)
{
    static const double ladder[11] = {1e2f, 1e3f, 2e3f, 3e3f, 4e3f, 5e3f, 6e3f, 7e3f, 8e3f, 9e3f, 1e4f};
    double norm_z = or_green_partial_fn(s_n, idx, s_n, idx, homog, x, y, z, kappa, che, znnpp, k0);
    int jj = 0;
    double res = 1e3, fsr = ladder[0];
    long nnz = 0;
    while (jj < 11 && res > res_sr) {
        double fn;
        fsr = ladder[jj];
        nnz = or_sr_dense(s_n, idx, fsr, homog, x, y, z, kappa, che, znnpp, k0, NULL, &fn);
        res = fabs(norm_z - fn) / norm_z * 100.;
        jj++;
    }
    if (nnz_out) *nnz_out = nnz;
    return fsr;
}

/* ------------------------------------------------------------------------- */
/* a9: getTransmitters_CBFM, 'un' distribution (src/getParameters_CBFM.f90:34-75) */
/* Returns NTr_CBFM; th/ph must hold at least 2*niws + 64 entries.            */
/* ------------------------------------------------------------------------- */
int or_transmitters_un(int niws, double *th, double *ph)
{
    const double Pi = ref_pi();
    /* delta = (360+180)**2.+4*(Niws-1)*(360*180): a real(4) expression */
    float df = 291600.0f + (float)(4 * (niws - 1) * (360 * 180));
    double delta = (double)df;
    double step = ((360. + 180.) + sqrt(delta)) / (2. * (niws - 1));
    int nth = (int)lround(180. / step) + 1;   /* nint() rounds halves away from zero */
    int nph = (int)lround(360. / step) + 1;
    int ntr = nth * nph;
    double step_ph = (360. - 0.) / (nph - 1);
    double margin_th = cos(180. * Pi / 180.) - cos(0. * Pi / 180.);
    double step_th = margin_th / (nth - 1);
    double c0 = cos(0. * Pi / 180.);
    int ind = 0;
    for (int i = 0; i < nph; ++i) {
        double phd = i * step_ph;
        for (int k = 0; k < nth; ++k) {
            double v = 1. * k * step_th + c0;
            if (v < -1.0) v = -1.0;   /* acos domain guard: only rounding can push below -1 */
            th[ind] = acos(v) * 180. / Pi;
            ph[ind] = phd;
            ind++;
        }
    }
    return ntr;
}

/* initializeNipws tables (src/Initialization.f90:58-62,
 * src/getParameters_CBFM.f90:294-348): Niws from r/lambda. */
int or_init_nipws(double r_lambda, int distr, int niws_input)
{
    static const int un[8] = {91, 190, 190, 231, 325, 496, 703, 861};
    static const int sd[8] = {94, 108, 108, 120, 144, 156, 180, 204};
    static const int lb[8] = {86, 110, 110, 146, 170, 194, 230, 266};
    const int *tab = distr == 2 ? sd : (distr == 3 ? lb : un);
    int niws = -1;
    for (int rr = 1; rr <= 8; ++rr)
        if (r_lambda <= rr) { niws = tab[rr - 1]; break; }
    if (niws < 0) niws = un[3];   /* :339-340 (the second assignment wins) */
    return niws_input > niws ? niws_input : niws;
}

/* ------------------------------------------------------------------------- */
/* a12: computeBlockRow / computeBlockCol (src/Green_functions.f90:905-1012,  */
/* 1119-1225) and Calcul_MatrixZij_ACA (src/Calcul_ACA_matrices.f90:6-219).   */
/* Global unknown indices are 0-based here.                                  */
/* ------------------------------------------------------------------------- */
static void block_row(int grow, int col0, int ncols, const double *x, const double *y, const double *z,
                      const double *kappa, const double *che, double k0, double Pi, zc8 *out)
{
    int io = grow / 3, pc = grow % 3;
    zc8 D[9];
    for (int j = 0; j < ncols / 3; ++j) {
        int s = col0 / 3 + j;
        dyad4(x[io] - x[s], y[io] - y[s], z[io] - z[s], k0, Pi, fk4_of(kappa, che, s), D);
        for (int q = 0; q < 3; ++q) out[3 * j + q] = D[pc * 3 + q];
    }
}
static void block_col(int row0, int nrows, int gcol, const double *x, const double *y, const double *z,
                      const double *kappa, const double *che, double k0, double Pi, zc8 *out)
{
    int s = gcol / 3, qc = gcol % 3;
    zc4 fk = fk4_of(kappa, che, s);
    zc8 D[9];
    for (int i = 0; i < nrows / 3; ++i) {
        int io = row0 / 3 + i;
        dyad4(x[io] - x[s], y[io] - y[s], z[io] - z[s], k0, Pi, fk, D);
        for (int p = 0; p < 3; ++p) out[3 * i + p] = D[p * 3 + qc];
    }
}

void or_block_row(int grow, int col0, int ncols, const double *x, const double *y, const double *z,
                  const double *kappa, const double *che, double k0, double *out)
{
    block_row(grow, col0, ncols, x, y, z, kappa, che, k0, ref_pi(), (zc8 *)out);
}
void or_block_col(int row0, int nrows, int gcol, const double *x, const double *y, const double *z,
                  const double *kappa, const double *che, double k0, double *out)
{
    block_col(row0, nrows, gcol, x, y, z, kappa, che, k0, ref_pi(), (zc8 *)out);
}

/* |z| as sqrt(re^2 + im^2) with every operation rounded: the pivot searches and
 * threshold tests compare magnitudes, and this form evaluates bit-identically in
 * the oracle (no FMA contraction) and on the GPU.  (The reference's Fortran ABS
 * of a complex is a compiler intrinsic whose last-bit behaviour is unpinned.) */
static inline double zabs(zc8 a) { return sqrt(a.re * a.re + a.im * a.im); }
static inline zc8 zdiv(zc8 a, zc8 b)
{
    double d = b.re * b.re + b.im * b.im;
    return z8((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}

/* U is nrows x itmax (column-major), V is itmax x ncols (column-major).      */
/* Returns nb_iter_out exactly as the reference does (k at exit; itmax+1 when */
/* the tolerance was never met).                                              */
int or_aca(int row0, int nrows, int col0, int ncols, double eps, int itmax,
           const double *x, const double *y, const double *z,
           const double *kappa, const double *che, double k0, double *Uo, double *Vo)
{
    const double Pi = ref_pi();
    zc8 *U = (zc8 *)Uo, *V = (zc8 *)Vo;
    memset(U, 0, sizeof(zc8) * (size_t)nrows * itmax);
    memset(V, 0, sizeof(zc8) * (size_t)itmax * ncols);
    int *Ir = (int *)calloc(itmax + 2, sizeof(int)), *Jc = (int *)calloc(itmax + 2, sizeof(int));
    zc8 *R = (zc8 *)calloc((size_t)nrows * ncols, sizeof(zc8)); /* Appro_R, column-major */
    double *nf = (double *)calloc(itmax + 2, sizeof(double));
    zc8 *row = (zc8 *)malloc(sizeof(zc8) * ncols), *col = (zc8 *)malloc(sizeof(zc8) * nrows);
#define RR(i, j) R[(size_t)(j) * nrows + (i)]
#define UU(i, k) U[(size_t)(k) * nrows + (i)]
#define VV(k, j) V[(size_t)(j) * itmax + (k)]
    Ir[0] = 0;
    block_row(row0 + Ir[0], col0, ncols, x, y, z, kappa, che, k0, Pi, row);
    for (int j = 0; j < ncols; ++j) RR(Ir[0], j) = row[j];
    int best = 0; double bv = -1;
    for (int j = 0; j < ncols; ++j) { double a = zabs(RR(Ir[0], j)); if (a > bv) { bv = a; best = j; } }
    Jc[0] = best;
    zc8 piv = RR(Ir[0], Jc[0]);
    for (int j = 0; j < ncols; ++j) VV(0, j) = zdiv(RR(Ir[0], j), piv);
    block_col(row0, nrows, col0 + Jc[0], x, y, z, kappa, che, k0, Pi, col);
    for (int i = 0; i < nrows; ++i) RR(i, Jc[0]) = col[i];
    for (int i = 0; i < nrows; ++i) UU(i, 0) = RR(i, Jc[0]);
    double v2 = 0;
    for (int i = 0; i < nrows; ++i) { double a = zabs(UU(i, 0)); v2 += a * a; }
    double nu = sqrt(v2);
    v2 = 0;
    for (int j = 0; j < ncols; ++j) { double a = zabs(VV(0, j)); v2 += a * a; }
    double nv = sqrt(v2);
    nf[0] = sqrt(0. + nu * nu * (nv * nv));
    best = 0; bv = -1;
    for (int i = 0; i < nrows; ++i) {
        double a = (i == Ir[0]) ? 0. : zabs(RR(i, Jc[0]));
        if (a > bv) { bv = a; best = i; }
    }
    Ir[1] = best;
    int k = 2;   /* 1-based iteration counter, as in the reference */
    int go = 1;
    while (go && k <= itmax) {
        int kk = k - 1;   /* 0-based slot */
        int ik = Ir[kk];
        block_row(row0 + ik, col0, ncols, x, y, z, kappa, che, k0, Pi, row);
        for (int j = 0; j < ncols; ++j) {
            zc8 acc = z8(0, 0);
            for (int l = 0; l < kk; ++l) { zc8 p = z8mul(UU(ik, l), VV(l, j)); acc.re += p.re; acc.im += p.im; }
            RR(ik, j) = z8(row[j].re - acc.re, row[j].im - acc.im);
        }
        best = 0; bv = -1;
        for (int j = 0; j < ncols; ++j) {
            int used = 0;
            for (int l = 0; l < kk; ++l) if (Jc[l] == j) { used = 1; break; }
            double a = used ? 0. : zabs(RR(ik, j));
            if (a > bv) { bv = a; best = j; }
        }
        Jc[kk] = best;
        int jk = best;
        piv = RR(ik, jk);
        for (int j = 0; j < ncols; ++j) VV(kk, j) = zdiv(RR(ik, j), piv);
        block_col(row0, nrows, col0 + jk, x, y, z, kappa, che, k0, Pi, col);
        for (int i = 0; i < nrows; ++i) {
            zc8 acc = z8(0, 0);
            for (int l = 0; l < kk; ++l) { zc8 p = z8mul(VV(l, jk), UU(i, l)); acc.re += p.re; acc.im += p.im; }
            RR(i, jk) = z8(col[i].re - acc.re, col[i].im - acc.im);
        }
        for (int i = 0; i < nrows; ++i) UU(i, kk) = RR(i, jk);
        double prev = nf[kk - 1];
        v2 = 0;
        for (int i = 0; i < nrows; ++i) { double a = zabs(UU(i, kk)); v2 += a * a; }
        nu = sqrt(v2);
        v2 = 0;
        for (int j = 0; j < ncols; ++j) { double a = zabs(VV(kk, j)); v2 += a * a; }
        nv = sqrt(v2);
        double suv = 0;
        for (int nj = 0; nj < kk; ++nj) {
            zc8 su = z8(0, 0), sv = z8(0, 0);
            for (int i = 0; i < nrows; ++i) { zc8 p = z8mul(UU(i, nj), UU(i, kk)); su.re += p.re; su.im += p.im; }
            for (int j = 0; j < ncols; ++j) { zc8 p = z8mul(VV(kk, j), VV(nj, j)); sv.re += p.re; sv.im += p.im; }
            suv += zabs(su) * zabs(sv);
        }
        nf[kk] = sqrt(prev * prev + 2 * suv + nu * nu * (nv * nv));
        double res = (nu * nv) / nf[kk];
        if (res <= eps) {
            go = 0;
        } else {
            best = 0; bv = -1;
            for (int i = 0; i < nrows; ++i) {
                int used = 0;
                for (int l = 0; l <= kk; ++l) if (Ir[l] == i) { used = 1; break; }
                double a = used ? 0. : zabs(RR(i, Jc[kk]));
                if (a > bv) { bv = a; best = i; }
            }
            Ir[kk + 1] = best;
            k++;
        }
    }
#undef RR
#undef UU
#undef VV
    free(Ir); free(Jc); free(R); free(nf); free(row); free(col);
    return k;
}

/* ------------------------------------------------------------------------- */
/* 8(f)1: GetFFieldCoeff (src/Green_functions.f90:1399-1438) and the S-matrix  */
/* projection of Compute_EFields_MoM (src/Compute_EFields_MoM.f90:306-369).    */
/* S is nrx x 4*ntr column-major: columns 4tr..4tr+3 = Vv, Vh, Hv, Hh.         */
/* ------------------------------------------------------------------------- */
void or_smatrix(int n, const double *x, const double *y, const double *z,
                const double *kappa, const double *che, double k0,
                int nrx, const double *rth, const double *rph, int ntr, const double *E, double *S)
{
    const double Pi = ref_pi();
    const zc8 *Ez = (const zc8 *)E;
    zc8 *Sz = (zc8 *)S;
#pragma omp parallel for schedule(dynamic, 1)
    for (int r = 0; r < nrx; ++r) {
        double tr = rth[r] * Pi / 180., pr = rph[r] * Pi / 180.;
        double xc = cos(tr), yc = sin(tr) * cos(pr), zcp = sin(tr) * sin(pr);
        zc8 *ff = (zc8 *)malloc(sizeof(zc8) * n);
        for (int c = 0; c < n; ++c) {
            double ph = -k0 * (xc * x[c] + yc * y[c] + zcp * z[c]);
            zc8 ffc = z8(cos(ph), sin(ph));                      /* exp(-J*k_0*(...)) */
            zc8 fk = fk8_of(kappa, che, c);
            zc8 t = z8(ffc.re * (k0 * k0), ffc.im * (k0 * k0));  /* ffc*k_0**2. */
            t = z8mul(t, fk);                                     /* *f_kapChe */
            t = z8(t.re / (4 * Pi), t.im / (4 * Pi));             /* /(4*Pi) */
            ff[c] = z8(t.re * k0, t.im * k0);                     /* *k_0 */
        }
        for (int t = 0; t < ntr; ++t) {
            zc8 ev[3] = {{0, 0}, {0, 0}, {0, 0}}, eh[3] = {{0, 0}, {0, 0}, {0, 0}};
            for (int c = 0; c < n; ++c)
                for (int p = 0; p < 3; ++p) {
                    zc8 a = z8mul(ff[c], Ez[(size_t)t * 3 * n + 3 * c + p]);
                    zc8 b = z8mul(ff[c], Ez[(size_t)(t + ntr) * 3 * n + 3 * c + p]);
                    ev[p].re += a.re; ev[p].im += a.im;
                    eh[p].re += b.re; eh[p].im += b.im;
                }
            double st = sin(tr), ct = cos(tr), sp = sin(pr), cp = cos(pr);
            zc8 vv = z8(-ev[0].re * st + ev[1].re * ct * cp + ev[2].re * ct * sp,
                        -ev[0].im * st + ev[1].im * ct * cp + ev[2].im * ct * sp);
            zc8 vh = z8(-ev[1].re * sp + ev[2].re * cp, -ev[1].im * sp + ev[2].im * cp);
            zc8 hv = z8(-eh[0].re * st + eh[1].re * ct * cp + eh[2].re * ct * sp,
                        -eh[0].im * st + eh[1].im * ct * cp + eh[2].im * ct * sp);
            zc8 hh = z8(-eh[1].re * sp + eh[2].re * cp, -eh[1].im * sp + eh[2].im * cp);
            Sz[(size_t)(4 * t + 0) * nrx + r] = vv;
            Sz[(size_t)(4 * t + 1) * nrx + r] = vh;
            Sz[(size_t)(4 * t + 2) * nrx + r] = hv;
            Sz[(size_t)(4 * t + 3) * nrx + r] = hh;
        }
        free(ff);
    }
}

/* ------------------------------------------------------------------------- */
/* 8(f)1: Compute_ExtAbsCsec_fromIntField (src/Compute_ExtAbsCsec_fromIntField.f90:45-64) */
/* Sums the field components before |.|^2 and before the product with the   */
/* conjugated complex(4) incident field, as the reference does.             */
/* ------------------------------------------------------------------------- */
void or_cext_cabs(int n, const double *x, const double *y, const double *z, const double *sc,
                  const double *che, double k0, int ntr, const double *th, const double *ph,
                  const double *E, double *cext, double *cabs)
{
    const zc8 *Ez = (const zc8 *)E;
    double *Einc = (double *)malloc(sizeof(double) * 2 * 3 * (size_t)n * 2);
    for (int t = 0; t < ntr; ++t) {
        or_incident_c4(n, NULL, x, y, z, k0, th, ph, t, t + 1, Einc);
        const zc8 *Ei = (const zc8 *)Einc;
        double ev = 0, eh = 0, av = 0, ah = 0;
        for (int c = 0; c < n; ++c) {
            zc8 sv = z8(0, 0), sh = z8(0, 0), iv = z8(0, 0), ih = z8(0, 0);
            for (int p = 0; p < 3; ++p) {
                zc8 a = Ez[(size_t)t * 3 * n + 3 * c + p], b = Ez[(size_t)(t + ntr) * 3 * n + 3 * c + p];
                sv.re += a.re; sv.im += a.im; sh.re += b.re; sh.im += b.im;
                zc8 u = Ei[3 * c + p], v = Ei[3 * (size_t)n + 3 * c + p];
                iv.re += u.re; iv.im += u.im; ih.re += v.re; ih.im += v.im;
            }
            double s3 = pow(sc[c], 3.0);
            double cim = che[2 * c + 1];
            double asv = zabs(sv), ash = zabs(sh);
            av += cim * (asv * asv) * s3;
            ah += cim * (ash * ash) * s3;
            zc8 ch = z8(che[2 * c], che[2 * c + 1]);
            zc8 pv = z8mul(z8mul(ch, sv), z8(iv.re, -iv.im));
            zc8 phh = z8mul(z8mul(ch, sh), z8(ih.re, -ih.im));
            ev += pv.im * s3;
            eh += phh.im * s3;
        }
        cext[t] = k0 * (ev + eh) / 2.;
        cabs[t] = k0 * (av + ah) / 2.;
    }
    free(Einc);
}

/* ------------------------------------------------------------------------- */
/* Sphere voxeliser (src/Discretization.f90:246-310): an inscribed cube plus  */
/* six slabs, each cell centre kept when its radius is below ap.  Returns the */
/* number of cells (written to xyz when it fits in cap).                       */
/* ------------------------------------------------------------------------- */
int or_sphere_cells(double dm, double sc, double *xyz, int cap)
{
    double ap = dm / 2.;
    int nd = (int)floor(dm / sc + 0.5);                       /* nint(dm/Sc) */
    /* ceiling((ap - (0.8*ap/sqrt(3.)))/Sc), 0.8 and sqrt(3.) in single precision */
    double q = (double)0.8f * ap / (double)sqrtf(3.0f);
    int next = (int)ceil((ap - q) / sc);
    int nint_ = nd - 2 * next;
    double api = (nint_ * sc) / 2.;
    double sx[7] = {-api, -ap, -ap, api, -api, -api, -ap};
    int nx[7] = {nint_, nd, next, next, nint_, nint_, nd};
    double sy[7] = {-api, -ap, -ap, -ap, -ap, api, -ap};
    int ny[7] = {nint_, nd, nd, nd, next, next, nd};
    double sz[7] = {-api, -ap, -api, -api, -api, -api, api};
    int nz[7] = {nint_, next, nint_, nint_, nint_, nint_, next};
    int cnt = 0;
    for (int d = 0; d < 7; ++d)
        for (int iz = 1; iz <= nz[d]; ++iz)
            for (int iy = 1; iy <= ny[d]; ++iy)
                for (int ix = 1; ix <= nx[d]; ++ix) {
                    double px = sx[d] + (ix - 0.5) * sc, py = sy[d] + (iy - 0.5) * sc, pz = sz[d] + (iz - 0.5) * sc;
                    if (d > 0 && !(sqrt(px * px + py * py + pz * pz) < ap)) continue;
                    if (cnt < cap && xyz) { xyz[3 * cnt] = px; xyz[3 * cnt + 1] = py; xyz[3 * cnt + 2] = pz; }
                    cnt++;
                }
    return cnt;
}

int or_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
