// scatq.cu -- efficiencies per incident direction and their orientation averages.
//
//   Compute_Scattering_Quantities_1 (src/Compute_Scattering_Quantities.f90:1-589):
//     grid transmitters ('un' adaptive quadrature, 'tr' trapezoid, 'gl' weights);
//   Compute_Scattering_Quantities_2 (src/Compute_Scattering_Quantities.f90:593-1012):
//     transmitter lists ('sd', 'rf' means, 'lb' weights);
//   receivers: the same rules, plus 'sd' / 'lb' lists.
//   The adaptive rule is QUADPACK's QAG with the 61-point Gauss-Kronrod pair
//   (src/quadpack.f90:1-890) as the reference modified it: the integrand is a
//   sampled column read at the nearest grid index, and everything runs in
//   single precision (src/Numerical_Integration.f90:213-245).
//
// Work split.  The host builds the O(NRx + NTr) direction tables (propagation
// vectors, sin(theta) weights, forward/backward target angles, the distinct
// grid angles of Unique1DArray_D); the GPU does everything that scales with
// NTr x NRx:
//   k_q_dir      one CTA per transmitter: |S|^2 integrands (Q_sca, g) over the
//                receivers, forward/backward receiver search (getTxRxIndex),
//                Q_ext, Q_bks and the internal-field Q_ext / Q_abs;
//   k_q_rx       one thread per quadrature: a QAG per (transmitter, integrand,
//                phi column) for 'un', else one serial weighted sum per
//                (transmitter, integrand);
//   k_q_rx_fin   one thread per transmitter: the phi QAG ('un') and the
//                Q_sca / g formulas;
//   k_q_avg      one CTA: the averages over the transmitters.
// Every floating-point operation is an explicitly rounded intrinsic (no FMA
// contraction) in the reference's order, so the results are bit-identical to
// a strict IEEE evaluation of the same formulas on the host.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <unordered_set>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace midas {
namespace {

constexpr int QAG_LIMIT = 500;
// QAG work lists per running quadrature: alist, blist, rlist, elist (float) and iord (int).
constexpr size_t QAG_WS = (size_t)QAG_LIMIT * 5 * 4;
// Where the receiver quadratures keep their work lists.  Every bisection reads
// and rewrites them through dependent loads: from shared memory that is ~30
// cycles a step, from global memory (10 KB per quadrature, beyond L1 for a
// block) an L2 round trip.  Shared memory holds 20 lists per SM, registers
// allow 256 quadratures per SM: a call with few quadratures (one incident
// direction: tens) runs them from shared memory, a call with many (an
// orientation average: tens of thousands) from global memory at 6x the
// concurrency.  Measured on GB300: 50 quadratures 14.2 -> 6.8 ms in shared
// memory; 35k quadratures 56 ms in global memory, 84 ms in shared memory.
constexpr int QAG_SM_TPB = 20;                         // quadratures per block (one block per SM)
constexpr int QAG_SMEM = QAG_SM_TPB * (int)QAG_WS;     // 200,000 bytes of dynamic shared memory
constexpr int Q_TPB = 128;                             // threads per block otherwise

// Gauss-Kronrod 30/61 rule on [-1, 1] (QUADPACK qk61): Kronrod abscissae in
// decreasing order (odd indices are the 30-point Gauss abscissae), their
// Kronrod weights, the Gauss weights.  Single precision as in the reference.
__constant__ float c_gk_x[31] = {
    0.9994844100504906f, 0.9968934840746495f, 0.9916309968704046f, 0.9836681232797472f,
    0.9731163225011263f, 0.9600218649683075f, 0.9443744447485600f, 0.9262000474292743f,
    0.9055733076999078f, 0.8825605357920527f, 0.8572052335460611f, 0.8295657623827684f,
    0.7997278358218391f, 0.7677774321048262f, 0.7337900624532268f, 0.6978504947933158f,
    0.6600610641266270f, 0.6205261829892429f, 0.5793452358263617f, 0.5366241481420199f,
    0.4924804678617786f, 0.4470337695380892f, 0.4004012548303944f, 0.3527047255308781f,
    0.3040732022736251f, 0.2546369261678898f, 0.2045251166823099f, 0.1538699136085835f,
    0.1028069379667370f, 0.05147184255531770f, 0.0f};
__constant__ float c_gk_wk[31] = {
    0.001389013698677008f, 0.003890461127099884f, 0.006630703915931292f, 0.009273279659517763f,
    0.01182301525349634f, 0.01436972950704580f, 0.01692088918905327f, 0.01941414119394238f,
    0.02182803582160919f, 0.02419116207808060f, 0.02650995488233310f, 0.02875404876504129f,
    0.03090725756238776f, 0.03298144705748373f, 0.03497933802806002f, 0.03688236465182123f,
    0.03867894562472759f, 0.04037453895153596f, 0.04196981021516425f, 0.04345253970135607f,
    0.04481480013316266f, 0.04605923827100699f, 0.04718554656929915f, 0.04818586175708713f,
    0.04905543455502978f, 0.04979568342707421f, 0.05040592140278235f, 0.05088179589874961f,
    0.05122154784925877f, 0.05142612853745903f, 0.05149472942945157f};
__constant__ float c_gk_wg[15] = {
    0.007968192496166606f, 0.01846646831109096f, 0.02878470788332337f, 0.03879919256962705f,
    0.04840267283059405f, 0.05749315621761907f, 0.06597422988218050f, 0.07375597473770521f,
    0.08075589522942022f, 0.08689978720108298f, 0.09212252223778613f, 0.09636873717464426f,
    0.09959342058679527f, 0.1017623897484055f, 0.1028526528935588f};

// rounded arithmetic (never contracted)
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fdv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dmu(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddv(double a, double b) { return __ddiv_rn(a, b); }

// |z|**2. as the reference evaluates it: (sqrt(re*re + im*im))**2
__device__ __forceinline__ double abs2(double2 z)
{
    const double a = __dsqrt_rn(da(dmu(z.x, z.x), dmu(z.y, z.y)));
    return dmu(a, a);
}

// Status words: [0] a transmitter without a forward receiver (t+1),
// [1] without a backward receiver (t+1), [2] a sample index outside its grid.
enum { QST_FWD = 0, QST_BKW = 1, QST_INDEX = 2, QST_N = 4 };

// f(nint(x*(n-1)/(b0-a0))+1) of a sampled column (src/quadpack.f90:621-627);
// an index outside the column is flagged in `bad` and read at the nearest end.
// Branch-free, so the 61 loads of a rule evaluation issue back to back.
__device__ __forceinline__ float q_sample(const double *f, int n, float span, float x, bool &bad)
{
    const float t = fdv(fm(x, (float)(n - 1)), span);
    const bool finite = t > -1e9f && t < 1e9f;
    const int i = finite ? (int)roundf(t) + 1 : 1;
    bad |= !finite || i < 1 || i > n;
    return __double2float_rn(f[min(max(i, 1), n) - 1]);
}

// qk61 (src/quadpack.f90:486-728) over a sampled column spanning [a0, b0].
__device__ void q_qk61(const double *f, int n, float span, float a, float b, float &result, float &abserr,
                       float &resabs, float &resasc, bool &bad)
{
    const float centr = fm(0.5f, fa(b, a)), hlgth = fm(0.5f, fs(b, a)), dhlgth = fabsf(hlgth);
    float fv1[30], fv2[30];
    const float fc = q_sample(f, n, span, centr, bad);
    float resg = 0.0f, resk = fm(c_gk_wk[30], fc), ra = fabsf(resk);
#pragma unroll
    for (int j = 1; j <= 15; ++j) {   // Gauss abscissae
        const int k = 2 * j - 1;
        const float absc = fm(hlgth, c_gk_x[k]);
        const float f1 = q_sample(f, n, span, fs(centr, absc), bad);
        const float f2 = q_sample(f, n, span, fa(centr, absc), bad);
        fv1[k] = f1;
        fv2[k] = f2;
        const float fsum = fa(f1, f2);
        resg = fa(resg, fm(c_gk_wg[j - 1], fsum));
        resk = fa(resk, fm(c_gk_wk[k], fsum));
        ra = fa(ra, fm(c_gk_wk[k], fa(fabsf(f1), fabsf(f2))));
    }
#pragma unroll
    for (int j = 1; j <= 15; ++j) {   // Kronrod-only abscissae
        const int k = 2 * j - 2;
        const float absc = fm(hlgth, c_gk_x[k]);
        const float f1 = q_sample(f, n, span, fs(centr, absc), bad);
        const float f2 = q_sample(f, n, span, fa(centr, absc), bad);
        fv1[k] = f1;
        fv2[k] = f2;
        const float fsum = fa(f1, f2);
        resk = fa(resk, fm(c_gk_wk[k], fsum));
        ra = fa(ra, fm(c_gk_wk[k], fa(fabsf(f1), fabsf(f2))));
    }
    const float reskh = fm(resk, 0.5f);
    float rasc = fm(c_gk_wk[30], fabsf(fs(fc, reskh)));
#pragma unroll
    for (int k = 0; k < 30; ++k) rasc = fa(rasc, fm(c_gk_wk[k], fa(fabsf(fs(fv1[k], reskh)), fabsf(fs(fv2[k], reskh)))));
    result = fm(resk, hlgth);
    ra = fm(ra, dhlgth);
    rasc = fm(rasc, dhlgth);
    float err = fabsf(fm(fs(resk, resg), hlgth));
    if (rasc != 0.0f && err != 0.0f) {
        float t = fdv(fm(200.0f, err), rasc);
        t = fm(t, __fsqrt_rn(t));
        err = fm(rasc, t < 1.0f ? t : 1.0f);
    }
    if (ra > fdv(FLT_MIN, fm(50.0f, FLT_EPSILON))) {
        const float e2 = fm(fm(FLT_EPSILON, 50.0f), ra);
        err = e2 > err ? e2 : err;
    }
    abserr = err;
    resabs = ra;
    resasc = rasc;
}

// QUADPACK qpsrt (src/quadpack.f90:730-890): keeps iord (1-based interval
// numbers) in decreasing order of elist and picks the next interval to bisect.
// The reference scans iord[ibeg..jbnd] linearly, twice; that segment is kept
// non-increasing in elist, so the first entry <= errmax and the last entry >
// errmin are found here by binary search and the entries in between moved as a
// block: the same iord, maxerr and ermax for every input without NaNs (whose
// quadratures are NaN either way), at O(log n) dependent loads instead of O(n).
// qage calls it with nrmax = 1, where the reference's first loop runs no trips.
__device__ void q_qpsrt(int limit, int last, int &maxerr, float &ermax, const float *elist, int *iord, int &nrmax)
{
#define EL(i) elist[(i) - 1]
#define IO(i) iord[(i) - 1]
    if (last <= 2) {
        IO(1) = 1;
        IO(2) = 2;
    } else {
        const float errmax = EL(maxerr);
        const int trips = nrmax - 1;
        for (int t = 0; t < trips; ++t) {
            const int isucc = IO(nrmax - 1);
            if (errmax <= EL(isucc)) break;
            IO(nrmax) = isucc;
            nrmax -= 1;
        }
        int jupbn = last;
        if (limit / 2 + 2 < last) jupbn = limit + 3 - last;
        const float errmin = EL(last);
        const int jbnd = jupbn - 1, ibeg = nrmax + 1;
        int lo = ibeg, hi = jbnd + 1;   // first i with EL(IO(i)) <= errmax
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (EL(IO(mid)) <= errmax) hi = mid;
            else lo = mid + 1;
        }
        const int i = lo;
        for (int q = ibeg; q < i; ++q) IO(q - 1) = IO(q);
        if (i > jbnd) {
            IO(jbnd) = maxerr;
            IO(jupbn) = last;
        } else {
            IO(i - 1) = maxerr;
            int l2 = i, h2 = jbnd + 1;   // first k with !(errmin < EL(IO(k)))
            while (l2 < h2) {
                const int mid = (l2 + h2) >> 1;
                if (errmin < EL(IO(mid))) l2 = mid + 1;
                else h2 = mid;
            }
            const int k = l2 - 1;
            for (int q = jbnd; q > k; --q) IO(q + 1) = IO(q);
            IO(k + 1) = last;
        }
    }
    maxerr = IO(nrmax);
    ermax = EL(maxerr);
#undef EL
#undef IO
}

// getAdaptiveQuadPts2 -> qag -> qage, key 6, epsabs 0, epsrel 1e-3, limit 500
// (src/Numerical_Integration.f90:213-245, src/quadpack.f90:1-484).  ws holds
// QAG_WS bytes of work lists.
__device__ float q_qag(const double *f, int n, float a, float b, char *ws, int *st)
{
    float *alist = (float *)ws, *blist = alist + QAG_LIMIT, *rlist = blist + QAG_LIMIT, *elist = rlist + QAG_LIMIT;
    int *iord = (int *)(elist + QAG_LIMIT);
    const float epsabs = 0.0f, epsrel = 0.001f, c = 6.0f;
    const float span = fs(b, a);
    float result, abserr, defabs, resabs;
    int ier = 0;
    bool bad = false;
    alist[0] = a;
    blist[0] = b;
    q_qk61(f, n, span, a, b, result, abserr, defabs, resabs, bad);
    rlist[0] = result;
    elist[0] = abserr;
    iord[0] = 1;
    float errbnd = fm(epsrel, fabsf(result));
    if (epsabs > errbnd) errbnd = epsabs;
    if (abserr <= fm(fm(50.0f, FLT_EPSILON), defabs) && errbnd < abserr) ier = 2;
    if (ier != 0 || (abserr <= errbnd && abserr != resabs) || abserr == 0.0f) {
        if (bad) atomicOr(st + QST_INDEX, 1);
        return result;
    }
    float errmax = abserr, area = result, errsum = abserr;
    int maxerr = 1, nrmax = 1, iroff1 = 0, iroff2 = 0, last = 2;
    for (; last <= QAG_LIMIT; ++last) {
        const float a1 = alist[maxerr - 1];
        const float b1 = fm(0.5f, fa(alist[maxerr - 1], blist[maxerr - 1]));
        const float a2 = b1, b2 = blist[maxerr - 1];
        float area1, error1, defab1, area2, error2, defab2, ra;
        q_qk61(f, n, span, a1, b1, area1, error1, ra, defab1, bad);
        q_qk61(f, n, span, a2, b2, area2, error2, ra, defab2, bad);
        const float area12 = fa(area1, area2), erro12 = fa(error1, error2);
        errsum = fs(fa(errsum, erro12), errmax);
        area = fs(fa(area, area12), rlist[maxerr - 1]);
        if (defab1 != error1 && defab2 != error2) {
            if (fabsf(fs(rlist[maxerr - 1], area12)) <= fm(1.0e-5f, fabsf(area12)) && fm(0.99f, errmax) <= erro12)
                iroff1++;
            if (10 < last && errmax < erro12) iroff2++;
        }
        rlist[maxerr - 1] = area1;
        rlist[last - 1] = area2;
        errbnd = fm(epsrel, fabsf(area));
        if (epsabs > errbnd) errbnd = epsabs;
        if (errbnd < errsum) {
            if (6 <= iroff1 || 20 <= iroff2) ier = 2;
            if (last == QAG_LIMIT) ier = 1;
            const float m = fabsf(a1) > fabsf(b2) ? fabsf(a1) : fabsf(b2);
            if (m <= fm(fa(1.0f, fm(fm(c, 1.0e3f), FLT_EPSILON)), fa(fabsf(a2), fm(1.0e4f, FLT_MIN)))) ier = 3;
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
        q_qpsrt(QAG_LIMIT, last, maxerr, errmax, elist, iord, nrmax);
        if (ier != 0 || errsum <= errbnd) break;
    }
    if (last > QAG_LIMIT) last = QAG_LIMIT;
    if (bad) atomicOr(st + QST_INDEX, 1);
    float s = 0.0f;
    for (int k = 0; k < last; ++k) s = fa(s, rlist[k]);
    return s;
}

// trap_2Dc (src/Numerical_Integration.f90:251-305), f nx x ny column-major.
__device__ double q_trap2d(const double *f, double a, double b, double c, double d, int nx, int ny)
{
    const double hx = ddv(b - a, (double)(nx - 1)), hy = ddv(d - c, (double)(ny - 1));
#define F(i, j) f[(size_t)((j) - 1) * nx + ((i) - 1)]
    double s = da(da(da(F(1, 1), F(1, ny)), F(nx, 1)), F(nx, ny));
    for (int i = 2; i <= nx - 1; ++i) s = da(s, dmu(2.0, da(F(i, 1), F(i, ny))));
    for (int j = 2; j <= ny - 1; ++j) s = da(s, dmu(2.0, da(F(1, j), F(nx, j))));
    for (int i = 2; i <= nx - 1; ++i)
        for (int j = 2; j <= ny - 1; ++j) s = da(s, dmu(4.0, F(i, j)));
#undef F
    return dmu(dmu(dmu(0.25, hx), hy), s);
}

// sum_i sum_j (wph[j] * wth[i]) * f(i, j), the reference's Gauss-Legendre loop
__device__ double q_gl2d(const double *f, const double *wth, const double *wph, int nx, int ny)
{
    double q = 0;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j) q = da(q, dmu(dmu(wph[j], wth[i]), f[(size_t)j * nx + i]));
    return q;
}

struct Dir4 {   // a direction table row: x, y, z and a weight
    double x, y, z, w;
};

struct QParams {
    int quad_tr, quad_rx, ntr, ntr_theta, ntr_phi, nrx, nrx_theta, nrx_phi, nrx_tot;
    int list_tr, list_rx, search, cext_intfields;
    double X, ap, k0, Pi, Sn, th0, th1, ph0, ph1;        // receiver grid limits (radians)
    double Snt, tth0, tth1, tph0, tph1;                  // transmitter grid limits (radians)
};

// Per transmitter: integrands over the receivers, the forward / backward
// receivers and the point quantities (Compute_Scattering_Quantities.f90:170-210,
// 360-420, 756-768, 862-872).  qp (8 per transmitter): Q_ext(far field),
// Q_ext(internal field), Q_abs(internal field), Q_bks.
__global__ void k_q_dir(QParams p, const double2 *__restrict__ S, const Dir4 *__restrict__ drx,
                        const Dir4 *__restrict__ dtr, const Dir4 *__restrict__ tgt,
                        const double *__restrict__ rth, const double *__restrict__ rph,
                        const double *__restrict__ w_rx, const double *__restrict__ cext,
                        const double *__restrict__ cabs, double *__restrict__ F, double *__restrict__ qp, int *st)
{
    __shared__ int s_fw, s_bk;
    const int t = blockIdx.x;
    const size_t ld = p.nrx_tot;
    const double2 *Sv = S + (size_t)(4 * t + 0) * ld, *Svh = S + (size_t)(4 * t + 1) * ld;
    const double2 *Shv = S + (size_t)(4 * t + 2) * ld, *Sh = S + (size_t)(4 * t + 3) * ld;
    const Dir4 ki = dtr[t];
    double *fx = F + (size_t)(2 * t) * p.nrx, *fg = fx + p.nrx;
    for (int r = threadIdx.x; r < p.nrx; r += blockDim.x) {
        const double sit = da(da(da(abs2(Sh[r]), abs2(Sv[r])), abs2(Svh[r])), abs2(Shv[r]));
        const Dir4 d = drx[r];
        const double cg = da(da(dmu(ki.x, d.x), dmu(ki.y, d.y)), dmu(ki.z, d.z));
        double v;
        if (p.list_rx) v = p.quad_rx == MIDAS_QUAD_LB ? dmu(w_rx[r], sit) : sit;
        else v = dmu(sit, d.w);
        fx[r] = v;
        fg[r] = dmu(v, cg);
    }
    if (threadIdx.x == 0) {
        s_fw = INT_MAX;
        s_bk = INT_MAX;
    }
    __syncthreads();
    if (p.search) {   // getTxRxIndex (src/get_trans_Receiv.f90:690-713): first match
        const double eps = (double)1e-2f;
        const Dir4 g = tgt[t];
        int fw = INT_MAX, bk = INT_MAX;
        for (int r = threadIdx.x; r < p.nrx_tot; r += blockDim.x) {
            const double a = rth[r], b = rph[r];
            if (fw == INT_MAX && fabs(a - g.x) <= eps && fabs(b - g.y) <= eps) fw = r;
            if (bk == INT_MAX && fabs(a - g.z) <= eps && fabs(b - g.w) <= eps) bk = r;
        }
        if (fw != INT_MAX) atomicMin(&s_fw, fw);
        if (bk != INT_MAX) atomicMin(&s_bk, bk);
    } else if (threadIdx.x == 0) {   // positional (Compute_Scattering_Quantities.f90:760-764, 866-870)
        const bool same = p.ntr == p.nrx;
        const int fw = (same && (p.quad_rx == MIDAS_QUAD_LB || p.quad_rx == MIDAS_QUAD_SD)) ? t : p.nrx + t;
        const int bk = (same && p.list_rx) ? p.nrx + t : p.nrx + p.ntr + t;
        if (fw < p.nrx_tot) s_fw = fw;
        if (bk < p.nrx_tot) s_bk = bk;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int fw = s_fw, bk = s_bk;
        if (fw == INT_MAX) atomicCAS(st + QST_FWD, 0, t + 1);
        if (bk == INT_MAX) atomicCAS(st + QST_BKW, 0, t + 1);
        const double pa2 = dmu(p.Pi, dmu(p.ap, p.ap));
        double *q = qp + 8 * (size_t)t;
        q[0] = fw == INT_MAX ? 0.0
                             : dmu(ddv(2.0, dmu(p.X, p.X)), da(fabs(Sh[fw].y), fabs(Sv[fw].y)));
        q[1] = ddv(cext[t], pa2);
        q[2] = ddv(cabs[t], pa2);
        q[3] = bk == INT_MAX ? 0.0
                             : dmu(ddv(1.0, dmu(dmu(dmu(2.0, p.Pi), p.X), p.X)),
                                   da(da(da(abs2(Sv[bk]), abs2(Sh[bk])), abs2(Svh[bk])), abs2(Shv[bk])));
    }
}

// Receiver quadratures.  'un': one QAG per (transmitter, integrand, phi column)
// over theta, result in fy; other rules: one serial sum per (transmitter,
// integrand), result in qr.
__global__ void __launch_bounds__(Q_TPB) k_q_rx(QParams p, const double *__restrict__ F, const double *__restrict__ w_rx,
                                                double *fy, double *qr, char *ws, int lists_in_smem, int *st)
{
    extern __shared__ __align__(16) char qsm[];   // QAG work lists when lists_in_smem
    const int gid = blockIdx.x * blockDim.x + threadIdx.x, nthr = gridDim.x * blockDim.x;
    char *mine = lists_in_smem ? qsm + (size_t)threadIdx.x * QAG_WS : ws + (size_t)gid * QAG_WS;
    if (p.quad_rx == MIDAS_QUAD_UN) {
        const long long inst = 2LL * p.ntr * p.nrx_phi;
        for (long long i = gid; i < inst; i += nthr) {
            const long long tk = i / p.nrx_phi;
            const int j = (int)(i % p.nrx_phi);
            const double *col = F + (size_t)tk * p.nrx + (size_t)j * p.nrx_theta;
            fy[i] = (double)q_qag(col, p.nrx_theta, (float)p.th0, (float)p.th1, mine, st);
        }
        return;
    }
    for (long long i = gid; i < 2LL * p.ntr; i += nthr) {
        const double *f = F + (size_t)i * p.nrx;
        double q = 0;
        if (p.quad_rx == MIDAS_QUAD_TR) q = q_trap2d(f, p.th0, p.th1, p.ph0, p.ph1, p.nrx_theta, p.nrx_phi);
        else if (p.quad_rx == MIDAS_QUAD_GL) q = q_gl2d(f, w_rx, w_rx + p.nrx_theta, p.nrx_theta, p.nrx_phi);
        else
            for (int r = 0; r < p.nrx; ++r) q = da(q, f[r]);
        qr[i] = q;
    }
}

// Per transmitter: the phi quadrature ('un') and Q_sca, g
// (Compute_Scattering_Quantities.f90:214-355, 768-860); q_dir row = Q_ext,
// Q_abs, Q_sca, Q_bks, g (the Qidtable columns, :383-392).
__global__ void __launch_bounds__(Q_TPB) k_q_rx_fin(QParams p, const double *fy, const double *qr, const double *qp,
                                                    double *q_dir, char *ws, int lists_in_smem, int *st)
{
    extern __shared__ __align__(16) char qsm[];   // QAG work lists when lists_in_smem
    const int gid = blockIdx.x * blockDim.x + threadIdx.x, nthr = gridDim.x * blockDim.x;
    char *mine = lists_in_smem ? qsm + (size_t)threadIdx.x * QAG_WS : ws + (size_t)gid * QAG_WS;
    for (int t = gid; t < p.ntr; t += nthr) {
        double q[2];
        for (int k = 0; k < 2; ++k) {
            if (p.quad_rx == MIDAS_QUAD_UN) {
                const double *y = fy + (size_t)(2 * t + k) * p.nrx_phi;
                q[k] = p.nrx_phi > 1 ? (double)q_qag(y, p.nrx_phi, (float)p.ph0, (float)p.ph1, mine, st)
                                     : y[0];
            } else {
                q[k] = qr[2 * t + k];
            }
        }
        const double c2 = dmu(2.0, dmu(p.k0, p.k0));
        double qs, g;
        if (p.quad_rx == MIDAS_QUAD_LB) {
            const double csca = dmu(ddv(1.0, c2), q[0]);
            qs = dmu(ddv(dmu(4.0, p.Pi), dmu(dmu(dmu(2.0, p.Pi), p.X), p.X)), q[0]);
            g = dmu(ddv(1.0, dmu(c2, csca)), q[1]);
        } else if (p.quad_rx == MIDAS_QUAD_SD || p.quad_rx == MIDAS_QUAD_RF) {
            const double w = ddv(dmu(4.0, p.Pi), (double)p.nrx);
            const double qsd = dmu(w, q[0]);
            const double csca = dmu(ddv(1.0, c2), qsd);
            qs = dmu(ddv(1.0, dmu(dmu(dmu(2.0, p.Pi), p.X), p.X)), qsd);
            g = dmu(dmu(ddv(1.0, dmu(c2, csca)), w), q[1]);
        } else {
            const double csca = dmu(ddv(1.0, c2), q[0]);
            qs = dmu(ddv(2.0, dmu(dmu(p.Sn, p.X), p.X)), q[0]);
            g = dmu(ddv(1.0, dmu(c2, csca)), q[1]);
        }
        const double *pp = qp + 8 * (size_t)t;
        double *o = q_dir + 5 * (size_t)t;
        o[0] = p.cext_intfields == 1 ? pp[1] : pp[0];
        o[1] = pp[2];
        o[2] = qs;
        o[3] = pp[3];
        o[4] = g;
    }
}

// Averages over the transmitters (Compute_Scattering_Quantities.f90:436-526, 937-968).
// One CTA; G holds 5 ntr doubles, gy 5 ntr_phi, ws blockDim.x work lists.
__global__ void __launch_bounds__(256) k_q_avg(QParams p, const double *q_dir, const double *s_tr, const double *w_tr, double *G,
                        double *gy, double *q_avg, char *ws, int *st)
{
    const int tid = threadIdx.x;
    if (p.ntr == 1) {
        if (tid < 5) q_avg[tid] = q_dir[tid];
        return;
    }
    if (p.list_tr) {
        if (tid < 5) {
            double s = 0;
            if (p.quad_tr == MIDAS_QUAD_LB)
                for (int t = 0; t < p.ntr; ++t) s = da(s, dmu(w_tr[t], q_dir[5 * (size_t)t + tid]));
            else {
                for (int t = 0; t < p.ntr; ++t) s = da(s, q_dir[5 * (size_t)t + tid]);
                s = ddv(s, (double)p.ntr);
            }
            q_avg[tid] = s;
        }
        return;
    }
    for (int i = tid; i < 5 * p.ntr; i += blockDim.x) {
        const int k = i / p.ntr, t = i % p.ntr;
        G[i] = dmu(q_dir[5 * (size_t)t + k], s_tr[t % p.ntr_theta]);
    }
    __syncthreads();
    if (p.quad_tr == MIDAS_QUAD_UN) {
        for (int i = tid; i < 5 * p.ntr_phi; i += blockDim.x) {
            const int k = i / p.ntr_phi, j = i % p.ntr_phi;
            gy[i] = (double)q_qag(G + (size_t)k * p.ntr + (size_t)j * p.ntr_theta, p.ntr_theta, (float)p.tth0,
                                  (float)p.tth1, ws + (size_t)tid * QAG_WS, st);
        }
        __syncthreads();
    }
    if (tid < 5) {
        const double *g = G + (size_t)tid * p.ntr;
        double q;
        if (p.quad_tr == MIDAS_QUAD_UN)
            q = p.ntr_phi > 1 ? (double)q_qag(gy + (size_t)tid * p.ntr_phi, p.ntr_phi, (float)p.tph0, (float)p.tph1,
                                              ws + (size_t)tid * QAG_WS, st)
                              : gy[(size_t)tid * p.ntr_phi];
        else if (p.quad_tr == MIDAS_QUAD_TR)   // 'tr' passes TrPh_min as both phi limits (:509-513)
            q = q_trap2d(g, p.tth0, p.tth1, p.tph0, p.tph0, p.ntr_theta, p.ntr_phi);
        else
            q = q_gl2d(g, w_tr, w_tr + p.ntr_theta, p.ntr_theta, p.ntr_phi);
        q_avg[tid] = dmu(ddv(1.0, p.Snt), q);
    }
}

// Unique1DArray_D (src/Compute_Scattering_Quantities.f90:1014-1042): distinct
// values in order of first appearance.
std::vector<double> unique_first(const double *v, int n)
{
    std::vector<double> out;
    std::unordered_set<double> seen;
    for (int i = 0; i < n; ++i) {
        const double x = v[i];
        if (x != x) { out.push_back(x); continue; }   // NaN never compares equal
        if (seen.insert(x == 0.0 ? 0.0 : x).second) out.push_back(x);
    }
    return out;
}

int host_copy(midas_gpu_ctx *c, const double *p, size_t n, std::vector<double> &out)
{
    out.resize(n);
    MIDAS_CUDA(c, cudaMemcpyAsync(out.data(), p, sizeof(double) * n, cudaMemcpyDefault, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    return MIDAS_OK;
}

}  // namespace

int scattering_quantities(midas_gpu_ctx *c, int quad_tr, int quad_rx, int ntr_theta, int ntr_phi,
                          const double *tr_theta, const double *tr_phi, int nrx_theta, int nrx_phi, int nrx_tot,
                          const double *rx_theta, const double *rx_phi, const double *S, const double *cext,
                          const double *cabs, double dm, double k0, int cext_intfields, const double *w_tr,
                          const double *w_rx, double *q_dir, double *q_avg)
{
    auto bad = [&](const char *m) { return c->err.set(MIDAS_ERR_ARG, std::string("scattering_quantities: ") + m); };
    if (quad_tr < MIDAS_QUAD_UN || quad_tr > MIDAS_QUAD_RF || quad_rx < MIDAS_QUAD_UN || quad_rx > MIDAS_QUAD_RF)
        return bad("unknown integration rule");
    if (ntr_theta < 1 || ntr_phi < 1 || nrx_theta < 1 || nrx_phi < 1) return bad("empty direction set");
    const long long ntr_ll = (long long)ntr_theta * ntr_phi, nrx_ll = (long long)nrx_theta * nrx_phi;
    if (ntr_ll > (1 << 24) || nrx_ll > (1 << 24) || nrx_tot < nrx_ll) return bad("direction counts");
    if (!tr_theta || !tr_phi || !rx_theta || !rx_phi || !S || !cext || !cabs || !q_dir || !q_avg)
        return bad("null pointer");
    if (!(dm > 0) || !(k0 > 0)) return bad("dm and k0 must be positive");
    QParams p{};
    p.quad_tr = quad_tr;
    p.quad_rx = quad_rx;
    p.ntr_theta = ntr_theta;
    p.ntr_phi = ntr_phi;
    p.ntr = (int)ntr_ll;
    p.nrx_theta = nrx_theta;
    p.nrx_phi = nrx_phi;
    p.nrx = (int)nrx_ll;
    p.nrx_tot = nrx_tot;
    p.list_tr = quad_tr >= MIDAS_QUAD_SD;
    p.list_rx = quad_rx >= MIDAS_QUAD_SD;
    p.search = !p.list_tr;
    p.cext_intfields = cext_intfields;
    // Compute_Scattering_Quantities_2 reads receiver lists only (its grid branch
    // leaves Q_sca and g unset); _1 has no 'rf' receiver rule.
    if (p.list_tr && !p.list_rx) return bad("list transmitters need 'sd', 'rf' or 'lb' receivers");
    if (!p.list_tr && quad_rx == MIDAS_QUAD_RF) return bad("'rf' receivers need list transmitters");
    if ((quad_rx == MIDAS_QUAD_LB || quad_rx == MIDAS_QUAD_GL) && !w_rx) return bad("receiver weights required");
    if ((quad_tr == MIDAS_QUAD_LB || quad_tr == MIDAS_QUAD_GL) && !w_tr && p.ntr > 1)
        return bad("transmitter weights required");
    const double Pi = c->pi;
    p.Pi = Pi;
    p.X = k0 * dm / 2.;
    p.ap = dm / 2.;
    p.k0 = k0;

    // host direction tables
    std::vector<double> tth, tph, rth, rph;
    MIDAS_TRY(host_copy(c, tr_theta, p.ntr, tth));
    MIDAS_TRY(host_copy(c, tr_phi, p.ntr, tph));
    MIDAS_TRY(host_copy(c, rx_theta, nrx_tot, rth));
    MIDAS_TRY(host_copy(c, rx_phi, nrx_tot, rph));
    std::vector<double> rtv, rpv;
    if (!p.list_rx) {   // :144-166
        rtv = unique_first(rth.data(), p.nrx);
        rpv = unique_first(rph.data(), p.nrx);
        if ((int)rtv.size() != nrx_theta || (int)rpv.size() != nrx_phi)
            return bad("receiver grid: distinct theta / phi counts differ from nrx_theta / nrx_phi");
        p.th0 = rtv.front() * Pi / 180.;
        p.th1 = rtv.back() * Pi / 180.;
        p.ph0 = rpv.front() * Pi / 180.;
        p.ph1 = rpv.back() * Pi / 180.;
        p.Sn = std::fmax(p.ph1 - p.ph0, 1.) * (std::cos(p.th0) - std::cos(p.th1));
    }
    if (!p.list_tr) {   // :81-96, :440
        const std::vector<double> tv = unique_first(tth.data(), p.ntr), pv = unique_first(tph.data(), p.ntr);
        p.tth0 = tv.front() * Pi / 180.;
        p.tth1 = tv.back() * Pi / 180.;
        p.tph0 = pv.front() * Pi / 180.;
        p.tph1 = pv.back() * Pi / 180.;
        p.Snt = std::fmax(p.tph1 - p.tph0, 1.) * (std::cos(p.tth0) - std::cos(p.tth1));
    }
    const size_t n_w_rx = quad_rx == MIDAS_QUAD_GL ? (size_t)nrx_theta + nrx_phi : quad_rx == MIDAS_QUAD_LB ? p.nrx : 0;
    const size_t n_w_tr = quad_tr == MIDAS_QUAD_GL ? (size_t)ntr_theta + ntr_phi : quad_tr == MIDAS_QUAD_LB ? p.ntr : 0;
    // packed host block: drx (4 nrx), dtr (4 ntr), tgt (4 ntr), rth, rph (nrx_tot each),
    // s_tr (ntr_theta), w_rx, w_tr, cext, cabs (ntr each)
    const size_t o_drx = 0, o_dtr = o_drx + 4 * (size_t)p.nrx, o_tgt = o_dtr + 4 * (size_t)p.ntr,
                 o_rth = o_tgt + 4 * (size_t)p.ntr, o_rph = o_rth + nrx_tot, o_str = o_rph + nrx_tot,
                 o_wrx = o_str + ntr_theta, o_wtr = o_wrx + n_w_rx, o_cex = o_wtr + n_w_tr, o_cab = o_cex + p.ntr,
                 n_tab = o_cab + p.ntr;
    std::vector<double> h(n_tab, 0.0);
    auto ang = [&](double deg) { return deg * Pi / 180.; };
    for (int r = 0; r < p.nrx; ++r) {   // propagation vectors of the receivers (:190-199, :262-270)
        double ths, phs, s = 1.0;
        if (p.list_rx) { ths = rth[r]; phs = rph[r]; }
        else { ths = rtv[r % nrx_theta]; phs = rpv[r / nrx_theta]; s = std::sin(ang(ths)); }
        double *d = &h[o_drx + 4 * (size_t)r];
        d[0] = -std::sin(ang(ths)) * std::cos(ang(phs));
        d[1] = -std::sin(ang(ths)) * std::sin(ang(phs));
        d[2] = -std::cos(ang(ths));
        d[3] = s;
    }
    for (int t = 0; t < p.ntr; ++t) {   // incident vectors (:173-176) and the fwd / bkw directions (:203, :411)
        double *d = &h[o_dtr + 4 * (size_t)t];
        d[0] = -std::sin(ang(tth[t])) * std::cos(ang(tph[t]));
        d[1] = -std::sin(ang(tth[t])) * std::sin(ang(tph[t]));
        d[2] = -std::cos(ang(tth[t]));
        double *g = &h[o_tgt + 4 * (size_t)t];
        g[0] = tth[t];
        g[1] = tph[t];
        g[2] = 180. - tth[t];
        g[3] = std::fmod(tph[t] + 180., 360.);
    }
    std::copy(rth.begin(), rth.end(), h.begin() + o_rth);
    std::copy(rph.begin(), rph.end(), h.begin() + o_rph);
    for (int i = 0; i < ntr_theta; ++i) h[o_str + i] = std::sin(ang(tth[i]));   // :442-443
    std::vector<double> tmp;
    if (n_w_rx) {
        MIDAS_TRY(host_copy(c, w_rx, n_w_rx, tmp));
        std::copy(tmp.begin(), tmp.end(), h.begin() + o_wrx);
    }
    if (n_w_tr && w_tr) {
        MIDAS_TRY(host_copy(c, w_tr, n_w_tr, tmp));
        std::copy(tmp.begin(), tmp.end(), h.begin() + o_wtr);
    }
    MIDAS_TRY(host_copy(c, cext, p.ntr, tmp));
    std::copy(tmp.begin(), tmp.end(), h.begin() + o_cex);
    MIDAS_TRY(host_copy(c, cabs, p.ntr, tmp));
    std::copy(tmp.begin(), tmp.end(), h.begin() + o_cab);

    // device buffers
    const void *dS;
    MIDAS_TRY(to_device(c, S, sizeof(double2) * (size_t)nrx_tot * 4 * p.ntr, S_IN0, &dS));
    const long long inst_rx = quad_rx == MIDAS_QUAD_UN ? 2LL * p.ntr * nrx_phi : 2LL * p.ntr;
    const int sms = device_sms(c), avg_threads = 256;
    // launch shapes (grid-stride loops): quadratures with shared-memory lists (one
    // block of 20 per SM) while they fit in two such rounds, else 128-thread blocks
    // with global lists (one block per SM for quadratures, 8 for plain sums)
    size_t ws_slots = 0;
    auto shape = [&](long long inst, bool qag, int &grid, int &tpb, int &smem) {
        const bool in_smem = qag && inst <= 2LL * sms * QAG_SM_TPB;
        tpb = in_smem ? QAG_SM_TPB : Q_TPB;
        smem = in_smem ? QAG_SMEM : 0;
        const long long want = (inst + tpb - 1) / tpb;
        grid = (int)std::max<long long>(1, std::min<long long>(want, qag ? sms : 8LL * sms));
        if (qag && !in_smem) ws_slots = std::max(ws_slots, (size_t)grid * tpb);
    };
    int g_rx, t_rx, m_rx, g_fin, t_fin, m_fin;
    shape(inst_rx, quad_rx == MIDAS_QUAD_UN, g_rx, t_rx, m_rx);
    shape(p.ntr, quad_rx == MIDAS_QUAD_UN && nrx_phi > 1, g_fin, t_fin, m_fin);
    static PerDeviceOnce attr_once;
    MIDAS_CUDA(c, attr_once.run(c->device, [] {
        cudaError_t e = cudaFuncSetAttribute(k_q_rx, cudaFuncAttributeMaxDynamicSharedMemorySize, QAG_SMEM);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_q_rx_fin, cudaFuncAttributeMaxDynamicSharedMemorySize, QAG_SMEM);
        return e;
    }));
    const size_t nF = 2 * (size_t)p.ntr * p.nrx, nfy = 2 * (size_t)p.ntr * nrx_phi, nqr = 2 * (size_t)p.ntr,
                 nqp = 8 * (size_t)p.ntr, nqd = 5 * (size_t)p.ntr, nG = 5 * (size_t)p.ntr, ngy = 5 * (size_t)ntr_phi;
    const size_t dbl = n_tab + nF + nfy + nqr + nqp + nqd + nG + ngy + 8;
    const size_t ws_bytes = std::max(ws_slots, (size_t)avg_threads) * QAG_WS;   // global work lists
    void *base;
    MIDAS_TRY(ensure(c, S_QWS, sizeof(double) * dbl + ws_bytes + 64, &base));
    double *d_tab = (double *)base;
    double *dF = d_tab + n_tab, *dfy = dF + nF, *dqr = dfy + nfy, *dqp = dqr + nqr, *dqd = dqp + nqp, *dG = dqd + nqd,
           *dgy = dG + nG, *dqa = dgy + ngy;
    int *dst = (int *)(dqa + 5);   // QST_N ints inside the last 8-double tail
    char *ws = (char *)(d_tab + dbl);
    MIDAS_CUDA(c, cudaMemcpyAsync(d_tab, h.data(), sizeof(double) * n_tab, cudaMemcpyHostToDevice, c->stream));
    MIDAS_CUDA(c, cudaMemsetAsync(dst, 0, sizeof(int) * QST_N, c->stream));

    const int e0 = kp_begin(c);
    k_q_dir<<<p.ntr, 256, 0, c->stream>>>(p, (const double2 *)dS, (const Dir4 *)(d_tab + o_drx),
                                          (const Dir4 *)(d_tab + o_dtr), (const Dir4 *)(d_tab + o_tgt),
                                          d_tab + o_rth, d_tab + o_rph, d_tab + o_wrx, d_tab + o_cex, d_tab + o_cab,
                                          dF, dqp, dst);
    MIDAS_CUDA(c, cudaGetLastError());
    k_q_rx<<<g_rx, t_rx, m_rx, c->stream>>>(p, dF, d_tab + o_wrx, dfy, dqr, ws, m_rx > 0, dst);
    MIDAS_CUDA(c, cudaGetLastError());
    k_q_rx_fin<<<g_fin, t_fin, m_fin, c->stream>>>(p, dfy, dqr, dqp, dqd, ws, m_fin > 0, dst);
    MIDAS_CUDA(c, cudaGetLastError());
    k_q_avg<<<1, avg_threads, 0, c->stream>>>(p, dqd, d_tab + o_str, d_tab + o_wtr, dG, dgy, dqa, ws, dst);
    MIDAS_CUDA(c, cudaGetLastError());
    c->launches += 4;
    kp_end(c, e0, MIDAS_KC_OTHER, 0.0, (double)sizeof(double2) * nrx_tot * 4 * p.ntr);

    int hst[QST_N];
    MIDAS_CUDA(c, cudaMemcpyAsync(hst, dst, sizeof hst, cudaMemcpyDeviceToHost, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    MIDAS_TRY(kp_flush(c));
    char m[160];
    if (hst[QST_FWD]) {
        snprintf(m, sizeof m, "forward scattering direction of transmitter %d not among the receivers", hst[QST_FWD] - 1);
        return bad(m);
    }
    if (hst[QST_BKW]) {
        snprintf(m, sizeof m, "backward scattering direction of transmitter %d not among the receivers", hst[QST_BKW] - 1);
        return bad(m);
    }
    if (hst[QST_INDEX])
        return bad("adaptive quadrature sampled outside its grid (the 'un' rule needs theta and phi ranges starting at 0)");
    MIDAS_CUDA(c, cudaMemcpyAsync(q_dir, dqd, sizeof(double) * nqd, cudaMemcpyDefault, c->stream));
    MIDAS_CUDA(c, cudaMemcpyAsync(q_avg, dqa, sizeof(double) * 5, cudaMemcpyDefault, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    return MIDAS_OK;
}

}  // namespace midas
