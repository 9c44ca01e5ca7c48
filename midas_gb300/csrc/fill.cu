// fill.cu -- impedance fills and incident fields of the MIDAS VIE-MoM (sm_103a).
//
// The element arithmetic follows the reference routines cited at each kernel.
// Two arithmetic families:
//   * FP64 (MoM path): compute_Green_s_tr_single_element,
//     Incident_Field_single_element (src/Compute_EFields_MoM.f90:433-598);
//   * "complex(4) locals" (CBFM path): Green_s_tr_partial, SR_Green_s_tr_partial,
//     computeBlockRow/Col (src/Green_functions.f90:96-1225) and Incident_Field
//     (src/Incident_Field.f90:1-63): FP64 intermediates rounded to float exactly
//     where the Fortran assigns to a Complex (kind 4) local, single-precision
//     3.*Tau and complex(4) products evaluated without FMA (the reference's
//     ifort -O3 x86-64 build has no FMA).
//
// When the cells sit on one uniform lattice (every configuration built by a
// voxeliser does), the dyad F depends only on the integer lattice offset
// between observation and source cell.  The "lattice" kernels evaluate F once
// per offset into a table (FP64 and complex(4)-rounded) and the fills become a
// gather plus one complex product per element, which turns the fill from
// FP64/SFU-bound into HBM-bound on GB300.
#include <cuda_fp16.h>
#include <algorithm>
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "green.cuh"
#include "kernels.cuh"

namespace midas {

// ---------------------------------------------------------------------------
// a1: SetCellsParams (src/SetCellsParams.f90:31-49)
// ---------------------------------------------------------------------------
__global__ void k_set_cells(int n, const double *sc, const double2 *eps, double k0, double Pi, double *an,
                            double2 *che, double2 *znnpp, double *kappa, double2 *fk8, float2 *fk4)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double third = (double)(1.0f / 3.0f);
    const double two3 = (double)(2.0f / 3.0f);
    double a = sc[c] * pow(0.75 / Pi, third);
    double2 ch = make_double2(eps[c].x - 1.0, eps[c].y);
    double ka = k0 * a;
    double s, co;
    sincos(ka, &s, &co);
    double2 t = make_double2(two3 * co, two3 * s);
    t = zmul8(t, make_double2(1.0, -ka));
    t.x -= 1.0;
    double2 zn = zmul8(t, ch);
    double kap = 4 * Pi * (s - ka * co) / pow(k0, 3.0);
    an[c] = a;
    che[c] = ch;
    znnpp[c] = zn;
    kappa[c] = kap;
    double2 f = make_double2(kap * ch.x, kap * ch.y);   // f_kapChe = Kappa_n*Che_n
    fk8[c] = f;
    fk4[c] = make_float2((float)f.x, (float)f.y);
}

// Table of F per lattice offset: tab8 (FP64) and tab4 (complex(4)-rounded).
__global__ void k_lat_table(int dim0, int dim1, int dim2, int sp0, int sp1, int sp2, double d, double k0,
                            double Pi, double2 *tab8, float2 *tab4)
{
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    size_t tot = (size_t)dim0 * dim1 * dim2;
    if (t >= tot) return;
    int di = (int)(t % dim0) - sp0;
    int dj = (int)((t / dim0) % dim1) - sp1;
    int dk = (int)(t / ((size_t)dim0 * dim1)) - sp2;
    if (di == 0 && dj == 0 && dk == 0) {
        for (int c = 0; c < 6; ++c) { tab8[6 * t + c] = make_double2(0, 0); tab4[6 * t + c] = make_float2(0, 0); }
        return;
    }
    double rx = di * d, ry = dj * d, rz = dk * d;
    double2 F8[6];
    float2 F4[6];
    dyadF8(rx, ry, rz, k0, Pi, F8);
    dyadF4(rx, ry, rz, k0, Pi, F4);
    for (int c = 0; c < 6; ++c) { tab8[6 * t + c] = F8[c]; tab4[6 * t + c] = F4[c]; }
}

// ---------------------------------------------------------------------------
// a2: FP64 MoM fill.  Writes the nine entries of each cell pair (io, is) that
// fall inside rows [r0,r0+nr) x cols [c0,c0+nc) to out[(row-r0)*rs + (col-c0)*cs];
// out32 (optional) receives the same values rounded to complex64.
// Threads run along the source cell so row-major outputs are coalesced.
// ---------------------------------------------------------------------------
template <bool LAT>
__global__ void k_mom_fill(int r0, int nr, int c0, int nc, const double *x, const double *y, const double *z,
                           const double2 *znnpp, const double2 *fk8, double k0, double Pi, Lat lat,
                           const double2 *tab8, double2 *out, float2 *out32, size_t rs, size_t cs)
{
    int is = c0 / 3 + blockIdx.x * blockDim.x + threadIdx.x;
    int io = r0 / 3 + blockIdx.y * blockDim.y + threadIdx.y;
    if (3 * is >= c0 + nc || 3 * io >= r0 + nr) return;
    double2 D[9];
    if (io == is) {
        double2 dg = make_double2(1 - znnpp[is].x, -znnpp[is].y);
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int q = 0; q < 3; ++q) D[p * 3 + q] = (p == q) ? dg : make_double2(0, 0);
    } else {
        double2 F[6];
        if (LAT) {
            size_t sl = lat.slot(io, is);
#pragma unroll
            for (int c = 0; c < 6; ++c) F[c] = tab8[6 * sl + c];
        } else {
            dyadF8(x[io] - x[is], y[io] - y[is], z[io] - z[is], k0, Pi, F);
        }
        double2 fk = fk8[is];
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                double2 v = zmul8(F[comp6(p, q)], fk);
                D[p * 3 + q] = make_double2(-v.x, -v.y);
            }
    }
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        int row = 3 * io + p;
        if (row < r0 || row >= r0 + nr) continue;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            int col = 3 * is + q;
            if (col < c0 || col >= c0 + nc) continue;
            size_t o = (size_t)(row - r0) * rs + (size_t)(col - c0) * cs;
            if (out) out[o] = D[p * 3 + q];
            if (out32) out32[o] = make_float2((float)D[p * 3 + q].x, (float)D[p * 3 + q].y);
        }
    }
}

// ---------------------------------------------------------------------------
// a3: FP64 incident field (Incident_Field_single_element).  V[(3c+p)*rs + col*cs]
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T mkz(double re, double im);
template <>
__device__ __forceinline__ double2 mkz<double2>(double re, double im) { return make_double2(re, im); }
template <>
__device__ __forceinline__ float2 mkz<float2>(double re, double im) { return make_float2((float)re, (float)im); }

template <typename T>
__global__ void k_mom_rhs(int n, const double *x, const double *y, const double *z, double k0, double Pi, int ntr,
                          const double *th, const double *ph, T *V, size_t rs, size_t cs)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    int col = blockIdx.y;
    if (c >= n) return;
    int vh = col >= ntr;
    int t = vh ? col - ntr : col;
    double tr = th[t] * Pi / 180., pr = ph[t] * Pi / 180.;
    double st, ct, sp, cp;
    sincos(tr, &st, &ct);
    sincos(pr, &sp, &cp);
    double kx = k0 * ct, ky = k0 * st * cp, kz = k0 * st * sp;
    double s1, c1, s2, c2, s3, c3;
    sincos(kx * x[c], &s1, &c1);
    sincos(ky * y[c], &s2, &c2);
    sincos(kz * z[c], &s3, &c3);
    double2 e = zmul8(zmul8(make_double2(c1, s1), make_double2(c2, s2)), make_double2(c3, s3));
    double2 o[3];
    if (!vh) {
        o[0] = make_double2(-(e.x * st), -(e.y * st));
        o[1] = make_double2((e.x * ct) * cp, (e.y * ct) * cp);
        o[2] = make_double2((e.x * ct) * sp, (e.y * ct) * sp);
    } else {
        o[0] = make_double2(0, 0);
        o[1] = make_double2(-(e.x * sp), -(e.y * sp));
        o[2] = make_double2(e.x * cp, e.y * cp);
    }
    for (int p = 0; p < 3; ++p) V[(size_t)(3 * c + p) * rs + (size_t)col * cs] = mkz<T>(o[p].x, o[p].y);
}

// ---------------------------------------------------------------------------
// a8: Incident_Field with complex(4) locals, on cells idx[0..ncell).
// E[(3c+p)*rs + col*cs]; column t = V, t + ntr = H.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_incident4(int ncell, const int *idx, const double *x, const double *y, const double *z, double k0,
                            double Pi, int ntr, const double *th, const double *ph, T *E, size_t rs, size_t cs)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    int t = blockIdx.y;
    if (c >= ncell) return;
    int g = idx ? idx[c] : c;
    double tr = th[t] * Pi / 180., pr = ph[t] * Pi / 180.;
    double st = sin(tr), ct = cos(tr), sp = sin(pr), cp = cos(pr);
    float kx = (float)(k0 * ct);
    float ky = (float)((k0 * st) * cp);
    float kz = (float)((k0 * st) * sp);
    double s1, c1, s2, c2, s3, c3;
    sincos((double)kx * x[g], &s1, &c1);
    sincos((double)ky * y[g], &s2, &c2);
    sincos((double)kz * z[g], &s3, &c3);
    double2 e = zmul8_rn(zmul8_rn(make_double2(c1, s1), make_double2(c2, s2)), make_double2(c3, s3));
    float2 ex = make_float2((float)(-__dmul_rn(e.x, st)), (float)(-__dmul_rn(e.y, st)));
    float2 ey = make_float2((float)__dmul_rn(__dmul_rn(e.x, ct), cp), (float)__dmul_rn(__dmul_rn(e.y, ct), cp));
    float2 ez = make_float2((float)__dmul_rn(__dmul_rn(e.x, ct), sp), (float)__dmul_rn(__dmul_rn(e.y, ct), sp));
    float2 hy = make_float2((float)(-__dmul_rn(e.x, sp)), (float)(-__dmul_rn(e.y, sp)));
    float2 hz = make_float2((float)__dmul_rn(e.x, cp), (float)__dmul_rn(e.y, cp));
    size_t rv = (size_t)t * cs, rh = (size_t)(t + ntr) * cs;
    E[(size_t)(3 * c) * rs + rv] = mkz<T>(ex.x, ex.y);
    E[(size_t)(3 * c + 1) * rs + rv] = mkz<T>(ey.x, ey.y);
    E[(size_t)(3 * c + 2) * rs + rv] = mkz<T>(ez.x, ez.y);
    E[(size_t)(3 * c) * rs + rh] = mkz<T>(0, 0);
    E[(size_t)(3 * c + 1) * rs + rh] = mkz<T>(hy.x, hy.y);
    E[(size_t)(3 * c + 2) * rs + rh] = mkz<T>(hz.x, hz.y);
}

// ---------------------------------------------------------------------------
// a8: Incident_Field_Spherical (src/Incident_Field.f90:65-166), the CBF
// excitations of type_iws = 2/3.  k_sph_centre (one CTA) forms the block
// centre -- the mean centroid, summed in cell order by one thread as the
// reference's sum() is read -- and the source radius Rsource = 10 max(Rbl,
// 2 Pi / k0) from the largest centroid distance (a max: any order).
// geo = (Xc, Yc, Zc, Rsource).  Every FP64 operation is an explicitly rounded
// intrinsic, so no product is fused into a sum.
// ---------------------------------------------------------------------------
__global__ void k_sph_centre(int ncell, const int *idx, const double *x, const double *y, const double *z,
                             double k0, double Pi, double *geo)
{
    __shared__ double cen[3];
    __shared__ double red[256];
    if (threadIdx.x == 0) {
        double sx = 0, sy = 0, sz = 0;
        for (int c = 0; c < ncell; ++c) {
            const int g = idx ? idx[c] : c;
            sx = __dadd_rn(sx, x[g]);
            sy = __dadd_rn(sy, y[g]);
            sz = __dadd_rn(sz, z[g]);
        }
        cen[0] = __ddiv_rn(sx, (double)ncell);
        cen[1] = __ddiv_rn(sy, (double)ncell);
        cen[2] = __ddiv_rn(sz, (double)ncell);
    }
    __syncthreads();
    double m2 = 0;
    for (int c = threadIdx.x; c < ncell; c += blockDim.x) {
        const int g = idx ? idx[c] : c;
        const double dx = __dsub_rn(x[g], cen[0]), dy = __dsub_rn(y[g], cen[1]), dz = __dsub_rn(z[g], cen[2]);
        m2 = fmax(m2, __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
    }
    red[threadIdx.x] = m2;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double rbl = __dsqrt_rn(red[0]);
        const double lam = __ddiv_rn(__dmul_rn(2.0, Pi), k0);
        geo[0] = cen[0];
        geo[1] = cen[1];
        geo[2] = cen[2];
        geo[3] = __dmul_rn(10.0, fmax(rbl, lam));
    }
}

// E[(3c+p)*rs + col*cs]; column t = V, t + ntr = H.  Per cell: the complex(4)
// phase exp(i k0 R) / R (:139), the local angles acos(ux), atan2(uz, uy)
// (:142-143), and complex(4) x real(8) products evaluated left to right in FP64
// and rounded to float at the assignment (:146-157).
template <typename T>
__global__ void k_incident_sph(int ncell, const int *idx, const double *x, const double *y, const double *z,
                               double k0, double Pi, int ntr, const double *th, const double *ph, const double *geo,
                               T *E, size_t rs, size_t cs)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    int t = blockIdx.y;
    if (c >= ncell) return;
    const int g = idx ? idx[c] : c;
    const double rsrc = geo[3];
    const double tr = th[t] * Pi / 180., pr = ph[t] * Pi / 180.;
    const double str = sin(tr), ctr = cos(tr), spr = sin(pr), cpr = cos(pr);
    const double xs = __dadd_rn(geo[0], __dmul_rn(rsrc, ctr));
    const double ys = __dadd_rn(geo[1], __dmul_rn(__dmul_rn(rsrc, str), cpr));
    const double zs = __dadd_rn(geo[2], __dmul_rn(__dmul_rn(rsrc, str), spr));
    const double dx = __dsub_rn(x[g], xs), dy = __dsub_rn(y[g], ys), dz = __dsub_rn(z[g], zs);
    const double R = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
    const double ux = __ddiv_rn(dx, R), uy = __ddiv_rn(dy, R), uz = __ddiv_rn(dz, R);
    double sa, ca;
    sincos(__dmul_rn(k0, R), &sa, &ca);
    const double pre = (double)(float)__ddiv_rn(ca, R), pim = (double)(float)__ddiv_rn(sa, R);
    const double the = acos(ux), phi = atan2(uz, uy);
    double st, ct, sp, cp;
    sincos(the, &st, &ct);
    sincos(phi, &sp, &cp);
    const float2 ex = make_float2((float)__dmul_rn(-pre, st), (float)__dmul_rn(-pim, st));
    const float2 ey = make_float2((float)__dmul_rn(__dmul_rn(pre, ct), cp), (float)__dmul_rn(__dmul_rn(pim, ct), cp));
    const float2 ez = make_float2((float)__dmul_rn(__dmul_rn(pre, ct), sp), (float)__dmul_rn(__dmul_rn(pim, ct), sp));
    const float2 hy = make_float2((float)__dmul_rn(-pre, sp), (float)__dmul_rn(-pim, sp));
    const float2 hz = make_float2((float)__dmul_rn(pre, cp), (float)__dmul_rn(pim, cp));
    const size_t rv = (size_t)t * cs, rh = (size_t)(t + ntr) * cs;
    E[(size_t)(3 * c) * rs + rv] = mkz<T>(ex.x, ex.y);
    E[(size_t)(3 * c + 1) * rs + rv] = mkz<T>(ey.x, ey.y);
    E[(size_t)(3 * c + 2) * rs + rv] = mkz<T>(ez.x, ez.y);
    E[(size_t)(3 * c) * rs + rh] = mkz<T>(0, 0);
    E[(size_t)(3 * c + 1) * rs + rh] = mkz<T>(hy.x, hy.y);
    E[(size_t)(3 * c + 2) * rs + rh] = mkz<T>(hz.x, hz.y);
}

// ---------------------------------------------------------------------------
// a4/a6: complex(4)-local block fill over cell lists idx1 (rows) x idx2 (cols).
//   mode 0: Green_s_tr_partial (all entries; self 3x3 = diag(1 - Znnpp)).
//   mode 1: SR_Green_s_tr_partial dense form: keep |g| > thr (float abs), self
//           3x3 keeps its diagonal; homog mirrors the upper triangle (PARDISO
//           mtype 6 reads only Is > Io).  idx1 == idx2 (extended block).
// out[(3 io + p) * rs + (3 is + q) * cs].
// ---------------------------------------------------------------------------
template <bool LAT, typename T>
__global__ void k_block_fill4(int n1, const int *idx1, int n2, const int *idx2, const double *x, const double *y,
                              const double *z, const double2 *znnpp, const float2 *fk4, double k0, double Pi,
                              Lat lat, const float2 *tab4, int mode, double thr, int homog, T *out, size_t rs,
                              size_t cs)
{
    int js = blockIdx.x * blockDim.x + threadIdx.x;
    int io = blockIdx.y * blockDim.y + threadIdx.y;
    if (js >= n2 || io >= n1) return;
    int o = idx1[io], s = idx2[js];
    T V[9];
    if (o == s) {
        T dg = mkz<T>(1 - znnpp[s].x, -znnpp[s].y);
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int q = 0; q < 3; ++q) V[p * 3 + q] = (p == q) ? dg : mkz<T>(0, 0);
    } else {
        // homog SR: the lower triangle is the transposed mirror of the pair (s -> o)
        bool mirror = (mode == 1 && homog && js < io);
        int oo = mirror ? s : o, ss = mirror ? o : s;
        float2 F[6];
        if (LAT) {
            size_t sl = lat.slot(oo, ss);
#pragma unroll
            for (int c = 0; c < 6; ++c) F[c] = tab4[6 * sl + c];
        } else {
            dyadF4(x[oo] - x[ss], y[oo] - y[ss], z[oo] - z[ss], k0, Pi, F);
        }
        float2 fk = fk4[ss];
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                float2 g = zmul4_rn(F[comp6(p, q)], fk);
                g = make_float2(-g.x, -g.y);
                if (mode == 1) {
                    float a = absf4(g);
                    if (!((double)a > thr)) g = make_float2(0.f, 0.f);
                }
                // the mirror transposes the 3x3: entry (p,q) of (o,s) is (q,p) of (s,o); F is symmetric
                V[p * 3 + q] = mkz<T>(g.x, g.y);
            }
    }
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q) out[(size_t)(3 * io + p) * rs + (size_t)(3 * js + q) * cs] = V[p * 3 + q];
}

// ---------------------------------------------------------------------------
// a4 fill straight into the split-TF32 A operand of the reduced-matrix product:
// row r of A3 holds (hi | hi | lo) of the complex(4) entries Z(r, 0..K), hi =
// TF32(z), lo = TF32(z - hi) (the layout zgemm_x3 builds), so the complex(4)
// block is never stored on its own.  Entries are those of mode 0 of
// k_block_fill4; the padding columns 6K..lda3 of each row are zeroed.  With A3h
// the row is the fp16 [hi | lo] operand of the fp16 split product (pieces of
// h16_piece(K) complex entries, their tails zeroed).
// ---------------------------------------------------------------------------
template <bool LAT>
__global__ void k_block_fill4_a3(int n1, const int *idx1, int n2, const int *idx2, const double *x, const double *y,
                                 const double *z, const double2 *znnpp, const float2 *fk4, double k0, double Pi,
                                 Lat lat, const float2 *tab4, float *A3, long long lda3, __half *A3h,
                                 float hscale)
{
    int js = blockIdx.x * blockDim.x + threadIdx.x;
    int io = blockIdx.y * blockDim.y + threadIdx.y;
    const long long K = 3LL * n2;
    float2 V[9];
    const bool live = js < n2 && io < n1;   // every thread reaches the staging barrier
    const int o = live ? idx1[io] : 0, s = live ? idx2[js] : 0;
    if (!live) {
#pragma unroll
        for (int e = 0; e < 9; ++e) V[e] = make_float2(0.f, 0.f);
    } else if (o == s) {
        float2 dg = make_float2((float)(1 - znnpp[s].x), (float)(-znnpp[s].y));
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int q = 0; q < 3; ++q) V[p * 3 + q] = (p == q) ? dg : make_float2(0.f, 0.f);
    } else {
        float2 F[6];
        if (LAT) {
            size_t sl = lat.slot(o, s);
#pragma unroll
            for (int cc = 0; cc < 6; ++cc) F[cc] = tab4[6 * sl + cc];
        } else {
            dyadF4(x[o] - x[s], y[o] - y[s], z[o] - z[s], k0, Pi, F);
        }
        const float2 fk = fk4[s];
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                float2 g = zmul4_rn(F[comp6(p, q)], fk);
                V[p * 3 + q] = make_float2(-g.x, -g.y);
            }
    }
    // stage the CTA's 6 rows x (64 cells x 3) complex entries (hi and lo) in shared
    // memory, then write each row segment as one contiguous run
    // (with A3h: fp16 pieces of the entries scaled by hscale, a power of two)
    __shared__ float2 sh[6][192], sl[6][192];
    const int tr = threadIdx.y, tc = threadIdx.x;
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float2 v = V[p * 3 + q];
            if (A3h) {
                const float xr = v.x * hscale, xi = v.y * hscale;
                const float hr = __half2float(__float2half_rn(xr)), hi = __half2float(__float2half_rn(xi));
                sh[3 * tr + p][3 * tc + q] = make_float2(hr, hi);
                sl[3 * tr + p][3 * tc + q] = make_float2(xr - hr, xi - hi);
            } else {
                const float hr = tf32_rna(v.x), hi = tf32_rna(v.y);
                sh[3 * tr + p][3 * tc + q] = make_float2(hr, hi);
                sl[3 * tr + p][3 * tc + q] = make_float2(tf32_rna(v.x - hr), tf32_rna(v.y - hi));
            }
        }
    __syncthreads();
    const int js0 = blockIdx.x * blockDim.x, io0 = blockIdx.y * blockDim.y;
    const int ncol = 3 * min(64, n2 - js0);                       // complex columns of this CTA
    const int nrow = 3 * min((int)blockDim.y, n1 - io0);
    const long long kc0 = 3LL * js0;
    for (int t = threadIdx.y * blockDim.x + threadIdx.x; t < nrow * ncol; t += blockDim.x * blockDim.y) {
        const int rr = t / ncol, cc = t % ncol;
        const float2 h = sh[rr][cc];
        if (A3h) {
            __half2 *row = (__half2 *)(A3h + (3LL * io0 + rr) * lda3);
            row[kc0 + cc] = __floats2half2_rn(h.x, h.y);
            row[h16_piece(K) + kc0 + cc] = __floats2half2_rn(sl[rr][cc].x, sl[rr][cc].y);
        } else {
            float2 *row = (float2 *)(A3 + (3LL * io0 + rr) * lda3);
            row[kc0 + cc] = h;
            row[K + kc0 + cc] = h;
            row[2 * K + kc0 + cc] = sl[rr][cc];
        }
    }
    if (js0 + 64 >= n2)   // the CTA holding the last columns zeroes the row padding
        for (int t = threadIdx.y * blockDim.x + threadIdx.x; t < nrow; t += blockDim.x * blockDim.y) {
            if (A3h) {
                __half2 *row = (__half2 *)(A3h + (3LL * io0 + t) * lda3);
                const long long P = h16_piece(K);
                for (long long pad = K; pad < P; ++pad) {
                    row[pad] = __floats2half2_rn(0.f, 0.f);
                    row[P + pad] = __floats2half2_rn(0.f, 0.f);
                }
            } else {
                float *row = A3 + (3LL * io0 + t) * lda3;
                for (long long pad = 6 * K; pad < lda3; ++pad) row[pad] = 0.f;
            }
        }
}

// ---------------------------------------------------------------------------
// setfSR scan: one pass over the extended block computes
//   fnz   -- Green_s_tr_partial_FN (src/Green_functions.f90:176-287), and
//   for each fSR of the ladder j: nnz_j and sum |g|^2 of SR_Green_s_tr_partial_FN
//   (:564-806).  Per-CTA partials: part[cta * (1 + 2 * NL) + ...].
// ---------------------------------------------------------------------------
constexpr int NLAD = 11;
// The ladder's threshold tests run on the FP32 pipe: an entry's magnitude a is a
// float, and (double)a > thr exactly when a > thr_f, thr_f = the largest float
// <= thr (no float lies strictly between the two).  Counts are integers and the
// squared magnitudes (floats) are summed in double float (TwoSum), which holds
// the FP64 sum of the same terms to ~2^-48; only the per-thread totals and the
// block reduction are FP64.  The FP64 form (a double compare and two FP64 adds
// per entry and threshold) made this scan FP64-bound.
__device__ __forceinline__ void df_add(float &hi, float &lo, float v)
{
    float s, e;
    ef_two_sum(hi, v, s, e);
    hi = s;
    lo = __fadd_rn(lo, e);
}

template <bool LAT>
__global__ void k_sr_scan(int s_n, const int *idx, const double *x, const double *y, const double *z,
                          const double2 *znnpp, const float2 *fk4, double k0, double Pi, Lat lat, const float2 *tab4,
                          int homog, const float *thr_f, double *part)
{
    __shared__ double sh[32][1 + 2 * NLAD];
    float tf[NLAD];
#pragma unroll
    for (int j = 0; j < NLAD; ++j) tf[j] = thr_f[j];
    double acc0 = 0, self_sq = 0;
    int cnt[NLAD];
    float qh[NLAD], ql[NLAD];
#pragma unroll
    for (int j = 0; j < NLAD; ++j) { cnt[j] = 0; qh[j] = ql[j] = 0.f; }
    size_t npair = (size_t)s_n * s_n;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < npair; t += (size_t)gridDim.x * blockDim.x) {
        int io = (int)(t / s_n), is = (int)(t % s_n);
        int o = idx[io], s = idx[is];
        if (io == is) {
            double a = hypot(1 - znnpp[s].x, -znnpp[s].y);
            acc0 += 3. * (a * a);                       // FN of Z (self term)
            self_sq += 3. * (a * a);
#pragma unroll
            for (int j = 0; j < NLAD; ++j) cnt[j] += 3;
            continue;
        }
        float2 F[6];
        if (LAT) {
            size_t sl = lat.slot(o, s);
            for (int c = 0; c < 6; ++c) F[c] = tab4[6 * sl + c];
        } else {
            dyadF4(x[o] - x[s], y[o] - y[s], z[o] - z[s], k0, Pi, F);
        }
        float2 fk = fk4[s];
        // Green_s_tr_partial_FN: homog scans Io >= Is; term is a real(4) expression
        if (!homog || io >= is) {
            float aF[6];
            for (int c = 0; c < 6; ++c) aF[c] = absf4(F[c]);
            float afk = absf4(fk);
            float tt = __fadd_rn(__fmul_rn(aF[0], aF[0]), __fmul_rn(2.f, __fmul_rn(aF[3], aF[3])));
            tt = __fadd_rn(tt, __fmul_rn(2.f, __fmul_rn(aF[5], aF[5])));
            tt = __fadd_rn(tt, __fmul_rn(aF[1], aF[1]));
            tt = __fadd_rn(tt, __fmul_rn(2.f, __fmul_rn(aF[4], aF[4])));
            tt = __fadd_rn(tt, __fmul_rn(aF[2], aF[2]));
            acc0 += (double)__fmul_rn(tt, __fmul_rn(afk, afk));
        }
        // SR: homog keeps only Is > Io
        if (!homog || is > io) {
            for (int p = 0; p < 3; ++p)
                for (int q = 0; q < 3; ++q) {
                    float2 g = zmul4_rn(F[comp6(p, q)], fk);
                    float a = absf4(g);
                    float a2 = __fmul_rn(a, a);
#pragma unroll
                    for (int j = 0; j < NLAD; ++j)
                        if (a > tf[j]) { cnt[j] += 1; df_add(qh[j], ql[j], a2); }
                }
        }
    }
    // block reduction (fixed order)
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int j = 0; j < 1 + 2 * NLAD; ++j) {
        double v;
        if (j == 0) v = acc0;
        else if (j <= NLAD) v = (double)cnt[j - 1];
        else v = (double)qh[j - 1 - NLAD] + (double)ql[j - 1 - NLAD] + self_sq;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sh[wid][j] = v;
    }
    __syncthreads();
    if (threadIdx.x < 1 + 2 * NLAD) {
        double v = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += sh[w][threadIdx.x];
        part[(size_t)blockIdx.x * (1 + 2 * NLAD) + threadIdx.x] = v;
    }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
static Lat make_lat(const midas_gpu_ctx *c)
{
    Lat l;
    l.ijk = c->lat_ijk;
    l.dim0 = c->lat_dim[0]; l.dim1 = c->lat_dim[1]; l.dim2 = c->lat_dim[2];
    l.sp0 = (c->lat_dim[0] - 1) / 2; l.sp1 = (c->lat_dim[1] - 1) / 2; l.sp2 = (c->lat_dim[2] - 1) / 2;
    return l;
}

static bool use_lat(const midas_gpu_ctx *c) { return c->lattice && c->lat_tab4 != nullptr; }

int launch_set_cells(midas_gpu_ctx *c)
{
    int n = c->n;
    ++c->launches;
    k_set_cells<<<(n + 127) / 128, 128, 0, c->stream>>>(n, c->sc, c->eps, c->k0, c->pi, c->an, c->che, c->znnpp,
                                                        c->kappa, c->fk8, c->fk4);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

int launch_lat_table(midas_gpu_ctx *c)
{
    size_t tot = (size_t)c->lat_dim[0] * c->lat_dim[1] * c->lat_dim[2];
    ++c->launches;
    k_lat_table<<<(unsigned)((tot + 127) / 128), 128, 0, c->stream>>>(
        c->lat_dim[0], c->lat_dim[1], c->lat_dim[2], (c->lat_dim[0] - 1) / 2, (c->lat_dim[1] - 1) / 2,
        (c->lat_dim[2] - 1) / 2, c->lat_d, c->k0, c->pi, c->lat_tab8, c->lat_tab4);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

int launch_mom_fill(midas_gpu_ctx *c, int r0, int nr, int c0, int nc, double2 *out, float2 *out32, size_t rs,
                    size_t cs)
{
    int ci0 = c0 / 3, ci1 = (c0 + nc - 1) / 3, ri0 = r0 / 3, ri1 = (r0 + nr - 1) / 3;
    dim3 blk(64, 4);
    dim3 grd((ci1 - ci0 + 1 + 63) / 64, (ri1 - ri0 + 1 + 3) / 4);
    // the fill kernel indexes cells from r0/3, c0/3: pass the aligned starts
    Lat l = make_lat(c);
    ++c->launches;
    int kp = kp_begin(c);
    if (c->opts.fill_mode == MIDAS_FILL_FAST && c->lattice && c->lat_tab8)
        k_mom_fill<true><<<grd, blk, 0, c->stream>>>(r0, nr, c0, nc, c->x, c->y, c->z, c->znnpp, c->fk8, c->k0, c->pi,
                                                     l, c->lat_tab8, out, out32, rs, cs);
    else
        k_mom_fill<false><<<grd, blk, 0, c->stream>>>(r0, nr, c0, nc, c->x, c->y, c->z, c->znnpp, c->fk8, c->k0,
                                                      c->pi, l, nullptr, out, out32, rs, cs);
    kp_end(c, kp, MIDAS_KC_FILL, 0.0, (double)nr * nc * ((out ? 16 : 0) + (out32 ? 8 : 0)));
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

template <typename T>
int launch_mom_rhs(midas_gpu_ctx *c, int ntr, const double *th, const double *ph, T *V, size_t rs, size_t cs)
{
    dim3 grd((c->n + 127) / 128, 2 * ntr);
    ++c->launches;
    k_mom_rhs<T><<<grd, 128, 0, c->stream>>>(c->n, c->x, c->y, c->z, c->k0, c->pi, ntr, th, ph, V, rs, cs);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}
template int launch_mom_rhs<double2>(midas_gpu_ctx *, int, const double *, const double *, double2 *, size_t, size_t);

template <typename T>
int launch_incident_sph(midas_gpu_ctx *c, int ncell, const int *idx, int ntr, const double *th, const double *ph,
                        T *E, size_t rs, size_t cs)
{
    if (ncell <= 0 || ntr <= 0) return MIDAS_OK;
    void *p;
    MIDAS_TRY(ensure(c, S_SPH, sizeof(double) * 4, &p));
    double *geo = (double *)p;
    c->launches += 2;
    k_sph_centre<<<1, 256, 0, c->stream>>>(ncell, idx, c->x, c->y, c->z, c->k0, c->pi, geo);
    dim3 grd((ncell + 127) / 128, ntr);
    k_incident_sph<T><<<grd, 128, 0, c->stream>>>(ncell, idx, c->x, c->y, c->z, c->k0, c->pi, ntr, th, ph, geo, E, rs,
                                                   cs);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}
template int launch_incident_sph<double2>(midas_gpu_ctx *, int, const int *, int, const double *, const double *,
                                          double2 *, size_t, size_t);
template int launch_incident_sph<float2>(midas_gpu_ctx *, int, const int *, int, const double *, const double *,
                                         float2 *, size_t, size_t);

template <typename T>
int launch_incident4(midas_gpu_ctx *c, int ncell, const int *idx, int ntr, const double *th, const double *ph, T *E,
                     size_t rs, size_t cs)
{
    dim3 grd((ncell + 127) / 128, ntr);
    ++c->launches;
    k_incident4<T><<<grd, 128, 0, c->stream>>>(ncell, idx, c->x, c->y, c->z, c->k0, c->pi, ntr, th, ph, E, rs, cs);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}
template int launch_incident4<double2>(midas_gpu_ctx *, int, const int *, int, const double *, const double *,
                                       double2 *, size_t, size_t);
template int launch_incident4<float2>(midas_gpu_ctx *, int, const int *, int, const double *, const double *,
                                      float2 *, size_t, size_t);

template <typename T>
int launch_block_fill4(midas_gpu_ctx *c, int n1, const int *idx1, int n2, const int *idx2, int mode, double thr,
                       int homog, T *out, size_t rs, size_t cs)
{
    dim3 blk(64, 2);
    dim3 grd((n2 + 63) / 64, (n1 + 1) / 2);
    Lat l = make_lat(c);
    ++c->launches;
    int kp = kp_begin(c);
    if (c->opts.fill_mode == MIDAS_FILL_FAST && use_lat(c))
        k_block_fill4<true, T><<<grd, blk, 0, c->stream>>>(n1, idx1, n2, idx2, c->x, c->y, c->z, c->znnpp, c->fk4,
                                                           c->k0, c->pi, l, c->lat_tab4, mode, thr, homog, out, rs, cs);
    else
        k_block_fill4<false, T><<<grd, blk, 0, c->stream>>>(n1, idx1, n2, idx2, c->x, c->y, c->z, c->znnpp, c->fk4,
                                                            c->k0, c->pi, l, nullptr, mode, thr, homog, out, rs, cs);
    kp_end(c, kp, MIDAS_KC_FILL, 0.0, 9.0 * n1 * n2 * sizeof(T));
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}
int launch_block_fill4_a3(midas_gpu_ctx *c, int n1, const int *idx1, int n2, const int *idx2, float *A3,
                          long long lda3, __half *A3h, float hscale)
{
    if (A3h && lda3 != h16_arow(3LL * n2)) return c->err.set(MIDAS_ERR_ARG, "block fill: bad fp16 operand stride");
    dim3 blk(64, 2);
    dim3 grd((n2 + 63) / 64, (n1 + 1) / 2);
    Lat l = make_lat(c);
    ++c->launches;
    int kp = kp_begin(c);
    if (c->opts.fill_mode == MIDAS_FILL_FAST && use_lat(c))
        k_block_fill4_a3<true><<<grd, blk, 0, c->stream>>>(n1, idx1, n2, idx2, c->x, c->y, c->z, c->znnpp, c->fk4,
                                                           c->k0, c->pi, l, c->lat_tab4, A3, lda3, A3h, hscale);
    else
        k_block_fill4_a3<false><<<grd, blk, 0, c->stream>>>(n1, idx1, n2, idx2, c->x, c->y, c->z, c->znnpp, c->fk4,
                                                            c->k0, c->pi, l, nullptr, A3, lda3, A3h, hscale);
    kp_end(c, kp, MIDAS_KC_FILL, 0.0, (A3h ? 2.0 : 4.0) * 3 * n1 * (double)lda3);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}
template int launch_block_fill4<double2>(midas_gpu_ctx *, int, const int *, int, const int *, int, double, int,
                                         double2 *, size_t, size_t);
template int launch_block_fill4<float2>(midas_gpu_ctx *, int, const int *, int, const int *, int, double, int,
                                        float2 *, size_t, size_t);

// An upper bound of |Z_os| over every cell pair of the lattice-table fill (mode 0):
// max(max |1 - Znnpp|, max over the table of |F| times max |f_kapChe|) -- the
// scale of the fp16 operand pieces of the reduced-matrix products.  0 when the
// fill does not come from the table.
__global__ void k_fill_bound(long long ntab, const float2 *tab4, int n, const double2 *znnpp, const float2 *fk4,
                             unsigned *out)
{
    float mt = 0.f, mf = 0.f, md = 0.f;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < ntab; e += (long long)gridDim.x * blockDim.x)
        mt = fmaxf(mt, absf4(tab4[e]));
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        mf = fmaxf(mf, absf4(fk4[e]));
        md = fmaxf(md, (float)hypot(1.0 - znnpp[e].x, -znnpp[e].y));
    }
    for (int o = 16; o > 0; o >>= 1) {
        mt = fmaxf(mt, __shfl_down_sync(0xffffffffu, mt, o));
        mf = fmaxf(mf, __shfl_down_sync(0xffffffffu, mf, o));
        md = fmaxf(md, __shfl_down_sync(0xffffffffu, md, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, __float_as_uint(mt));
        atomicMax(out + 1, __float_as_uint(mf));
        atomicMax(out + 2, __float_as_uint(md));
    }
}

int fill4_bound(midas_gpu_ctx *c, double *bound)
{
    *bound = 0.0;
    if (!(c->opts.fill_mode == MIDAS_FILL_FAST && use_lat(c))) return MIDAS_OK;
    void *p;
    MIDAS_TRY(ensure(c, S_RED, 64, &p));
    unsigned *d = (unsigned *)p;
    MIDAS_CUDA(c, cudaMemsetAsync(d, 0, 3 * sizeof(unsigned), c->stream));
    const long long ntab = 6LL * c->lat_dim[0] * c->lat_dim[1] * c->lat_dim[2];
    ++c->launches;
    k_fill_bound<<<1024, 256, 0, c->stream>>>(ntab, c->lat_tab4, c->n, c->znnpp, c->fk4, d);
    MIDAS_CUDA(c, cudaGetLastError());
    unsigned h[3];
    MIDAS_CUDA(c, cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    float f[3];
    memcpy(f, h, sizeof(f));
    // the complex(4) products round: a 1 % margin covers them
    *bound = 1.01 * std::max((double)f[0] * (double)f[1], (double)f[2]);
    return MIDAS_OK;
}

// setfSR ladder (src/getParameters_CBFM.f90:140-162).  vmax = |1 - Znnpp(first cell)|.
int sr_ladder(midas_gpu_ctx *c, int s_n, const int *d_idx, int first_cell, int homog, double res_sr, double *fsr_out,
              long long *nnz_out, int want_all, double *all_nnz, double *all_fn, double *fnz_out)
{
    static const double ladder[NLAD] = {1e2, 1e3, 2e3, 3e3, 4e3, 5e3, 6e3, 7e3, 8e3, 9e3, 1e4};
    double2 zn;
    MIDAS_CUDA(c, cudaMemcpyAsync(&zn, c->znnpp + first_cell, sizeof(double2), cudaMemcpyDeviceToHost, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    double vmax = hypot(1 - zn.x, -zn.y);
    float thr[NLAD];   // vmax / ladder rounded down to float (see k_sr_scan)
    for (int j = 0; j < NLAD; ++j) {
        const double t = vmax / ladder[j];
        float f = (float)t;
        if ((double)f > t) f = std::nextafter(f, -INFINITY);
        thr[j] = f;
    }
    const int nblk = 2 * 152, nv = 1 + 2 * NLAD;
    void *buf;
    MIDAS_TRY(ensure(c, S_RED, sizeof(double) * (nblk * nv + NLAD), &buf));
    double *part = (double *)buf;
    float *dthr = (float *)(part + nblk * nv);
    MIDAS_CUDA(c, cudaMemcpyAsync(dthr, thr, sizeof(thr), cudaMemcpyHostToDevice, c->stream));
    Lat l = make_lat(c);
    ++c->launches;
    int kp = kp_begin(c);
    if (c->opts.fill_mode == MIDAS_FILL_FAST && use_lat(c))
        k_sr_scan<true><<<nblk, 256, 0, c->stream>>>(s_n, d_idx, c->x, c->y, c->z, c->znnpp, c->fk4, c->k0, c->pi, l,
                                                     c->lat_tab4, homog, dthr, part);
    else
        k_sr_scan<false><<<nblk, 256, 0, c->stream>>>(s_n, d_idx, c->x, c->y, c->z, c->znnpp, c->fk4, c->k0, c->pi,
                                                      l, nullptr, homog, dthr, part);
    kp_end(c, kp, MIDAS_KC_SR_SCAN, 0.0, 0.0);
    MIDAS_CUDA(c, cudaGetLastError());
    std::vector<double> h((size_t)nblk * nv);
    MIDAS_CUDA(c, cudaMemcpyAsync(h.data(), part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    double tot[1 + 2 * NLAD] = {0};
    for (int b = 0; b < nblk; ++b)
        for (int j = 0; j < nv; ++j) tot[j] += h[(size_t)b * nv + j];
    double norm_z = sqrt(tot[0]);
    if (fnz_out) *fnz_out = norm_z;
    if (want_all) {
        for (int j = 0; j < NLAD; ++j) { all_nnz[j] = tot[1 + j]; all_fn[j] = sqrt(tot[1 + NLAD + j]); }
    }
    int jj = 0;
    double res = 1e3, fsr = ladder[0];
    long long nnz = 0;
    while (jj < NLAD && res > res_sr) {
        fsr = ladder[jj];
        nnz = (long long)tot[1 + jj];
        double fn = sqrt(tot[1 + NLAD + jj]);
        res = fabs(norm_z - fn) / norm_z * 100.;
        jj++;
    }
    if (fsr_out) *fsr_out = fsr;
    if (nnz_out) *nnz_out = nnz;
    return MIDAS_OK;
}

}  // namespace midas
