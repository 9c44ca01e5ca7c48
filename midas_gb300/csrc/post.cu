// post.cu -- cross sections and far-field scattering matrix from the internal field.
//
//   Cext / Cabs : Compute_ExtAbsCsec_fromIntField
//                 (src/Compute_ExtAbsCsec_fromIntField.f90:45-64); the field
//                 components of a cell are summed before |.|^2 and before the
//                 product with the conjugated complex(4) incident field, as in
//                 the reference.
//   S-matrix    : GetFFieldCoeff (src/Green_functions.f90:1399-1438) and the
//                 Vv/Vh/Hv/Hh projection (src/Compute_EFields_MoM.f90:306-369).
// Both are FP64 reductions; one CTA per transmitter (Cext/Cabs) or per receiver
// (S), fixed-order block reductions so results are reproducible run to run.
#include "common.cuh"
#include "kernels.cuh"

namespace midas {

__device__ __forceinline__ double2 cm(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

template <int NV>
__device__ void block_sum(double (&v)[NV], double *sh)
{
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int j = 0; j < NV; ++j) {
        double s = v[j];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) sh[w * NV + j] = s;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0;
        for (int k = 0; k < nw; ++k) s += sh[k * NV + threadIdx.x];
        sh[threadIdx.x] = s;   // sh[0..NV) hold the totals after the barrier below
    }
    __syncthreads();
}

// E is 3n x 2ntr column-major (ld = 3n) FP64
__global__ void k_cext_cabs(int n, const double *x, const double *y, const double *z, const double *sc,
                            const double2 *che, double k0, double Pi, int ntr, const double *th, const double *ph,
                            const double2 *E, double *cext, double *cabs)
{
    __shared__ double sh[32 * 4];
    int t = blockIdx.x;
    double tr = th[t] * Pi / 180., pr = ph[t] * Pi / 180.;
    double st = sin(tr), ct = cos(tr), sp = sin(pr), cp = cos(pr);
    float kx = (float)(k0 * ct), ky = (float)((k0 * st) * cp), kz = (float)((k0 * st) * sp);
    double v[4] = {0, 0, 0, 0};   // ext V, ext H, abs V, abs H
    const double2 *Ev = E + (long long)t * 3 * n, *Eh = E + (long long)(t + ntr) * 3 * n;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        // incident field with complex(4) locals (Incident_Field, src/Incident_Field.f90:43-58)
        double s1, c1, s2, c2, s3, c3;
        sincos((double)kx * x[c], &s1, &c1);
        sincos((double)ky * y[c], &s2, &c2);
        sincos((double)kz * z[c], &s3, &c3);
        double2 e = cm(cm(make_double2(c1, s1), make_double2(c2, s2)), make_double2(c3, s3));
        float2 ex = make_float2((float)(-(e.x * st)), (float)(-(e.y * st)));
        float2 ey = make_float2((float)((e.x * ct) * cp), (float)((e.y * ct) * cp));
        float2 ez = make_float2((float)((e.x * ct) * sp), (float)((e.y * ct) * sp));
        float2 hy = make_float2((float)(-(e.x * sp)), (float)(-(e.y * sp)));
        float2 hz = make_float2((float)(e.x * cp), (float)(e.y * cp));
        double2 iv = make_double2(((double)ex.x + ey.x) + ez.x, ((double)ex.y + ey.y) + ez.y);
        double2 ih = make_double2((0.0 + hy.x) + hz.x, (0.0 + hy.y) + hz.y);
        double2 sv = make_double2((Ev[3 * c].x + Ev[3 * c + 1].x) + Ev[3 * c + 2].x,
                                  (Ev[3 * c].y + Ev[3 * c + 1].y) + Ev[3 * c + 2].y);
        double2 sh_ = make_double2((Eh[3 * c].x + Eh[3 * c + 1].x) + Eh[3 * c + 2].x,
                                   (Eh[3 * c].y + Eh[3 * c + 1].y) + Eh[3 * c + 2].y);
        double s3c = pow(sc[c], 3.0);
        double2 ch = che[c];
        double asv = hypot(sv.x, sv.y), ash = hypot(sh_.x, sh_.y);
        v[2] += ch.y * (asv * asv) * s3c;
        v[3] += ch.y * (ash * ash) * s3c;
        v[0] += cm(cm(ch, sv), make_double2(iv.x, -iv.y)).y * s3c;
        v[1] += cm(cm(ch, sh_), make_double2(ih.x, -ih.y)).y * s3c;
    }
    block_sum<4>(v, sh);
    if (threadIdx.x == 0) {
        cext[t] = k0 * (sh[0] + sh[1]) / 2.;
        cabs[t] = k0 * (sh[2] + sh[3]) / 2.;
    }
}

// S is nrx x 4ntr column-major (ld = nrx)
__global__ void k_smatrix(int n, const double *x, const double *y, const double *z, const double *kappa,
                          const double2 *che, double k0, double Pi, int nrx, const double *rth, const double *rph,
                          int ntr, const double2 *E, double2 *S)
{
    extern __shared__ double shd[];
    int r = blockIdx.x;
    int tb = blockIdx.y;   // transmitter
    double tr = rth[r] * Pi / 180., pr = rph[r] * Pi / 180.;
    double xc = cos(tr), yc = sin(tr) * cos(pr), zc = sin(tr) * sin(pr);
    double v[12] = {0};    // (ev re/im x3, eh re/im x3)
    const double2 *Ev = E + (long long)tb * 3 * n, *Eh = E + (long long)(tb + ntr) * 3 * n;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
        double phs = -k0 * (xc * x[c] + yc * y[c] + zc * z[c]);
        double s, co;
        sincos(phs, &s, &co);
        double2 ch = che[c];
        double2 fk = make_double2(kappa[c] * ch.x, kappa[c] * ch.y);
        double2 t = make_double2(co * (k0 * k0), s * (k0 * k0));
        t = cm(t, fk);
        t = make_double2(t.x / (4 * Pi), t.y / (4 * Pi));
        double2 ff = make_double2(t.x * k0, t.y * k0);
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            double2 a = cm(ff, Ev[3 * c + p]), b = cm(ff, Eh[3 * c + p]);
            v[2 * p] += a.x; v[2 * p + 1] += a.y;
            v[6 + 2 * p] += b.x; v[6 + 2 * p + 1] += b.y;
        }
    }
    block_sum<12>(v, shd);
    if (threadIdx.x == 0) {
        double st = sin(tr), ct = cos(tr), sp = sin(pr), cp = cos(pr);
        double2 ev[3], eh[3];
        for (int p = 0; p < 3; ++p) {
            ev[p] = make_double2(shd[2 * p], shd[2 * p + 1]);
            eh[p] = make_double2(shd[6 + 2 * p], shd[6 + 2 * p + 1]);
        }
        double2 vv = make_double2(-ev[0].x * st + ev[1].x * ct * cp + ev[2].x * ct * sp,
                                  -ev[0].y * st + ev[1].y * ct * cp + ev[2].y * ct * sp);
        double2 vh = make_double2(-ev[1].x * sp + ev[2].x * cp, -ev[1].y * sp + ev[2].y * cp);
        double2 hv = make_double2(-eh[0].x * st + eh[1].x * ct * cp + eh[2].x * ct * sp,
                                  -eh[0].y * st + eh[1].y * ct * cp + eh[2].y * ct * sp);
        double2 hh = make_double2(-eh[1].x * sp + eh[2].x * cp, -eh[1].y * sp + eh[2].y * cp);
        S[(long long)(4 * tb + 0) * nrx + r] = vv;
        S[(long long)(4 * tb + 1) * nrx + r] = vh;
        S[(long long)(4 * tb + 2) * nrx + r] = hv;
        S[(long long)(4 * tb + 3) * nrx + r] = hh;
    }
}

int launch_cext_cabs(midas_gpu_ctx *c, int ntr, const double *th, const double *ph, const double2 *E, double *cext,
                     double *cabs)
{
    ++c->launches;
    k_cext_cabs<<<ntr, 256, 0, c->stream>>>(c->n, c->x, c->y, c->z, c->sc, c->che, c->k0, c->pi, ntr, th, ph, E,
                                            cext, cabs);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

int launch_smatrix(midas_gpu_ctx *c, int nrx, const double *rth, const double *rph, int ntr, const double2 *E,
                   double2 *S)
{
    dim3 grd(nrx, ntr);
    ++c->launches;
    k_smatrix<<<grd, 256, sizeof(double) * 8 * 12, c->stream>>>(c->n, c->x, c->y, c->z, c->kappa, c->che, c->k0,
                                                                 c->pi, nrx, rth, rph, ntr, E, S);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

}  // namespace midas
