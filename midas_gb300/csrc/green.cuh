// green.cuh -- device arithmetic of the dyadic Green's function shared by the
// fill kernels (fill.cu) and the ACA row/column kernels (aca.cu).
#pragma once
#include <cuda_runtime.h>

namespace midas {

// ---------------------------------------------------------------------------
// complex helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 zmul8(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// complex(8) product with every operation separately rounded (no FMA)
__device__ __forceinline__ double2 zmul8_rn(double2 a, double2 b)
{
    return make_double2(__dsub_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)),
                        __dadd_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x)));
}
// |z| as sqrt(re^2 + im^2) with every operation rounded: threshold tests and
// pivot searches compare magnitudes, and this form is bit-identical to the
// oracle's evaluation of the same expression
__device__ __forceinline__ float absf4(float2 a)
{
    return __fsqrt_rn(__fadd_rn(__fmul_rn(a.x, a.x), __fmul_rn(a.y, a.y)));
}
__device__ __forceinline__ double absd8(double2 a)
{
    return __dsqrt_rn(__dadd_rn(__dmul_rn(a.x, a.x), __dmul_rn(a.y, a.y)));
}
// complex(4) product with every float operation separately rounded (no FMA)
__device__ __forceinline__ float2 zmul4_rn(float2 a, float2 b)
{
    return make_float2(__fsub_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)),
                       __fadd_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}

// ---------------------------------------------------------------------------
// dyads.  Component order of the six unique entries: xx, yy, zz, xy, yz, xz.
// ---------------------------------------------------------------------------
// FP64 F (before the -f_kapChe factor): src/Compute_EFields_MoM.f90:474-519.
__device__ __forceinline__ void dyadF8(double rx, double ry, double rz, double k0, double Pi, double2 F[6])
{
    double r = sqrt(rx * rx + ry * ry + rz * rz);
    double s, co;
    sincos(k0 * r, &s, &co);
    double den = 4 * Pi * (r * r);
    double2 Gr = make_double2(co / den, s / den);
    double2 Tau = make_double2(-(1 / r), k0);
    double k2 = k0 * k0;
    double d[3] = {rx, ry, rz};
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        double sv = 3. * (d[p] * d[p]) / (r * r);
        double2 in = make_double2((Tau.x + k2 * (r - d[p] * d[p] / r)) - sv * Tau.x, Tau.y - sv * Tau.y);
        F[p] = zmul8(Gr, in);
    }
    double2 w = make_double2(-k2 - (3. * Tau.x) / r, -((3. * Tau.y) / r));
    double2 g;
    g = make_double2((Gr.x / r) * (rx * ry), (Gr.y / r) * (rx * ry)); F[3] = zmul8(g, w);
    g = make_double2((Gr.x / r) * (ry * rz), (Gr.y / r) * (ry * rz)); F[4] = zmul8(g, w);
    g = make_double2((Gr.x / r) * (rx * rz), (Gr.y / r) * (rx * rz)); F[5] = zmul8(g, w);
}

// complex(4)-rounded F: Green_s_tr_partial (src/Green_functions.f90:139-157).
__device__ __forceinline__ void dyadF4(double rx, double ry, double rz, double k0, double Pi, float2 F[6])
{
    double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz)));
    double s, co;
    sincos(__dmul_rn(k0, r), &s, &co);
    double den = __dmul_rn(__dmul_rn(4.0, Pi), __dmul_rn(r, r));
    float2 Gr4 = make_float2((float)__ddiv_rn(co, den), (float)__ddiv_rn(s, den));
    float2 Tau4 = make_float2((float)(-__ddiv_rn(1.0, r)), (float)k0);
    double2 Gr = make_double2(Gr4.x, Gr4.y), Tau = make_double2(Tau4.x, Tau4.y);
    double k2 = __dmul_rn(k0, k0);
    double r2 = __dmul_rn(r, r);
    double d[3] = {rx, ry, rz};
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        double dd = __dmul_rn(d[p], d[p]);
        double sv = __ddiv_rn(__dmul_rn(3., dd), r2);
        double re = __dsub_rn(__dadd_rn(Tau.x, __dmul_rn(k2, __dsub_rn(r, __ddiv_rn(dd, r)))), __dmul_rn(sv, Tau.x));
        double im = __dsub_rn(Tau.y, __dmul_rn(sv, Tau.y));
        double2 f = zmul8_rn(Gr, make_double2(re, im));
        F[p] = make_float2((float)f.x, (float)f.y);
    }
    // 3.*Tau_mn is a single-precision complex(4) product
    float t3r = __fmul_rn(3.0f, Tau4.x), t3i = __fmul_rn(3.0f, Tau4.y);
    double2 w = make_double2(__dsub_rn(-k2, __ddiv_rn((double)t3r, r)), -__ddiv_rn((double)t3i, r));
    double gr = __ddiv_rn(Gr.x, r), gi = __ddiv_rn(Gr.y, r);
    double pr[3] = {__dmul_rn(rx, ry), __dmul_rn(ry, rz), __dmul_rn(rx, rz)};
#pragma unroll
    for (int t = 0; t < 3; ++t) {
        double2 f = zmul8_rn(make_double2(__dmul_rn(gr, pr[t]), __dmul_rn(gi, pr[t])), w);
        F[3 + t] = make_float2((float)f.x, (float)f.y);
    }
}

// index (p,q) -> unique component
__device__ __forceinline__ int comp6(int p, int q)
{
    return p == q ? p : ((p + q == 1) ? 3 : ((p + q == 3) ? 4 : 5));
}

// lattice offset -> table slot (offsets stored for every (di,dj,dk) in range)
struct Lat {
    const int *ijk;
    int dim0, dim1, dim2;     // table extents (2*span+1)
    int sp0, sp1, sp2;        // spans
    __device__ __forceinline__ size_t slot(int o, int s) const
    {
        int di = ijk[3 * o] - ijk[3 * s] + sp0;
        int dj = ijk[3 * o + 1] - ijk[3 * s + 1] + sp1;
        int dk = ijk[3 * o + 2] - ijk[3 * s + 2] + sp2;
        return ((size_t)dk * dim1 + dj) * dim0 + di;
    }
};

}  // namespace midas
