// fft.cu -- the MoM operator on a voxel lattice as an FFT convolution (sm_103a).
//
// When every cell centroid sits on one uniform lattice, the MoM matrix of
// compute_Green_s_tr_single_element (src/Compute_EFields_MoM.f90:433-523)
// depends on a cell pair only through the lattice offset of the two cells:
//
//   (Z x)_o,p = (1 - Znnpp_o) x_o,p - sum_{s != o} sum_q F_pq(r_o - r_s) kc_s x_s,q
//
// with kc = f_kapChe = kappa Che.  The sum is a 3-D linear convolution of the
// six unique dyad components with w_q = kc x_q, evaluated here with zero-padded
// FFTs in FP64: grids of L_a >= 2 n_a - 1 points per axis (powers of two), the
// dyad spectra computed once per set of cells, and per right-hand side three
// forward transforms, a 3 x 3 pointwise product and three inverse transforms.
// The refinement residuals of the mixed MoM solve and the Krylov solver use it:
// an O(N log N) product instead of the O(N^2) dense residual, with no FP64
// matrix in memory.
//
// The transforms are radix-2 decimation-in-time FFTs along one axis at a time,
// several lines per CTA in shared memory (bit-reversed load, log2 L butterfly
// stages).  Lines that are all zero in the padded input (the padding region of
// the axes not yet transformed) are skipped on the way in, and lines whose
// outputs are never read are skipped on the way out.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "green.cuh"
#include "kernels.cuh"

namespace midas {

constexpr int FFT_THREADS = 256;
constexpr int FFT_TILE = 2048;   // complex points per CTA (lines x length)
constexpr int FFT_LMAX = 512;
constexpr int FFT_L3MAX = 384;   // the largest mixed-radix length 3 * 2^k

// twiddles w_k = exp(-2 pi i k / FFT_LMAX), k < FFT_LMAX / 2, followed by
// exp(-2 pi i j / FFT_L3MAX), j < 2 FFT_L3MAX / 3 (host libm, once per device)
static double2 *g_tw[64];

static int twiddles(midas_gpu_ctx *c, const double2 **out)
{
    static std::atomic<int> ready[64];
    const int dv = c->device & 63;
    if (!ready[dv].load(std::memory_order_acquire)) {
        std::vector<double2> h(FFT_LMAX / 2 + 2 * FFT_L3MAX / 3);
        for (int k = 0; k < FFT_LMAX / 2; ++k) {
            const double a = -2.0 * M_PI * k / FFT_LMAX;
            h[k] = make_double2(cos(a), sin(a));
        }
        for (int j = 0; j < 2 * FFT_L3MAX / 3; ++j) {
            const double a = -2.0 * M_PI * j / FFT_L3MAX;
            h[FFT_LMAX / 2 + j] = make_double2(cos(a), sin(a));
        }
        double2 *d = nullptr;
        MIDAS_CUDA(c, cudaMalloc(&d, sizeof(double2) * h.size()));
        MIDAS_CUDA(c, cudaMemcpy(d, h.data(), sizeof(double2) * h.size(), cudaMemcpyHostToDevice));
        int expect = 0;
        if (ready[dv].compare_exchange_strong(expect, 1, std::memory_order_acq_rel)) {
            g_tw[dv] = d;
        } else {
            cudaFree(d);   // another thread won; its table is the one in use
        }
    }
    *out = g_tw[dv];
    return MIDAS_OK;
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// ---------------------------------------------------------------------------
// The transforms compute in double float on the FP32 pipe (GB300's FP64 rate is
// 1/64 of its FP32 rate): a complex value is (re_hi, im_hi, re_lo, im_lo), each
// part a hi + lo pair of floats, ~2^-48 relative per operation (Dekker's product
// with FMA, Knuth's TwoSum for the sum).  Data stay FP64 in global memory and are
// split on load and rejoined on store.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void df_fast2(float s, float e, float &h, float &l)   // |s| >= |e|
{
    h = __fadd_rn(s, e);
    l = __fsub_rn(e, __fsub_rn(h, s));
}
__device__ __forceinline__ void dfr_add(float ah, float al, float bh, float bl, float &h, float &l)
{
    float s, e;
    ef_two_sum(ah, bh, s, e);
    e = __fadd_rn(e, __fadd_rn(al, bl));
    df_fast2(s, e, h, l);
}
__device__ __forceinline__ void dfr_mul(float ah, float al, float bh, float bl, float &h, float &l)
{
    const float p = __fmul_rn(ah, bh);
    float e = fmaf(ah, bh, -p);
    e = fmaf(ah, bl, e);
    e = fmaf(al, bh, e);
    df_fast2(p, e, h, l);
}
__device__ __forceinline__ float4 dfc_load(double2 v)
{
    const float rh = (float)v.x, ih = (float)v.y;
    return make_float4(rh, ih, (float)(v.x - (double)rh), (float)(v.y - (double)ih));
}
__device__ __forceinline__ double2 dfc_store(float4 v)
{
    return make_double2((double)v.x + (double)v.z, (double)v.y + (double)v.w);
}
__device__ __forceinline__ float4 dfc_add(float4 a, float4 b)
{
    float4 r;
    dfr_add(a.x, a.z, b.x, b.z, r.x, r.z);
    dfr_add(a.y, a.w, b.y, b.w, r.y, r.w);
    return r;
}
__device__ __forceinline__ float4 dfc_sub(float4 a, float4 b)
{
    float4 r;
    dfr_add(a.x, a.z, -b.x, -b.z, r.x, r.z);
    dfr_add(a.y, a.w, -b.y, -b.w, r.y, r.w);
    return r;
}
__device__ __forceinline__ float4 dfc_mul(float4 a, float4 b)
{
    float p1h, p1l, p2h, p2l, p3h, p3l, p4h, p4l;
    dfr_mul(a.x, a.z, b.x, b.z, p1h, p1l);
    dfr_mul(a.y, a.w, b.y, b.w, p2h, p2l);
    dfr_mul(a.x, a.z, b.y, b.w, p3h, p3l);
    dfr_mul(a.y, a.w, b.x, b.z, p4h, p4l);
    float4 r;
    dfr_add(p1h, p1l, -p2h, -p2l, r.x, r.z);
    dfr_add(p3h, p3l, p4h, p4l, r.y, r.w);
    return r;
}

// One radix-2 FFT pass along axis `ax` of a batch of L0 x L1 x L2 grids (x fastest).
// The lines along ax are indexed by (a, b): for ax = 0, a = y and b = z; for
// ax = 1, a = x and b = z; for ax = 2, a = x and b = y.  Only lines with
// a < na and b < nb are transformed.  sign = -1 forward, +1 inverse
// (unnormalised).  blockIdx.y selects the grid of the batch.
template <int LOGL>
__global__ void __launch_bounds__(FFT_THREADS) k_fft_axis(double2 *data, long long gstride, int ax, int L0, int L1,
                                                          int na, int nb, int sign, const double2 *tw)
{
    constexpr int L = 1 << LOGL;
    constexpr int G = FFT_TILE / L;   // lines per CTA
    constexpr int LP = L + 1;         // padded line length in shared memory
    extern __shared__ float4 sm[];
    float4 *stw = sm + G * LP;
    const int tid = threadIdx.x;
    for (int k = tid; k < L / 2; k += FFT_THREADS) {
        const double2 w = tw[k * (FFT_LMAX / L)];
        stw[k] = dfc_load(make_double2(w.x, sign > 0 ? -w.y : w.y));
    }
    const int ntile = (na + G - 1) / G;
    const int a0 = (blockIdx.x % ntile) * G, b = blockIdx.x / ntile;
    if (b >= nb) return;
    long long sa, sb, es;
    if (ax == 0) { sa = L0; sb = (long long)L0 * L1; es = 1; }
    else if (ax == 1) { sa = 1; sb = (long long)L0 * L1; es = L0; }
    else { sa = 1; sb = L0; es = (long long)L0 * L1; }
    double2 *g = data + (long long)blockIdx.y * gstride + (long long)b * sb;
    // load, bit-reversing the position along the line
    for (int idx = tid; idx < G * L; idx += FFT_THREADS) {
        int gl, k;
        if (ax == 0) { gl = idx / L; k = idx % L; } else { gl = idx % G; k = idx / G; }
        const int a = a0 + gl;
        if (a < na) sm[gl * LP + (__brev(k) >> (32 - LOGL))] = dfc_load(g[(long long)a * sa + (long long)k * es]);
    }
    __syncthreads();
#pragma unroll 1
    for (int s = 0; s < LOGL; ++s) {
        const int h = 1 << s;
        for (int j = tid; j < G * (L / 2); j += FFT_THREADS) {
            const int gl = j / (L / 2), bj = j % (L / 2);
            const int grp = bj >> s, pos = bj & (h - 1);
            const int i0 = gl * LP + grp * 2 * h + pos, i1 = i0 + h;
            const float4 t = dfc_mul(stw[pos << (LOGL - 1 - s)], sm[i1]);
            const float4 u = sm[i0];
            sm[i0] = dfc_add(u, t);
            sm[i1] = dfc_sub(u, t);
        }
        __syncthreads();
    }
    for (int idx = tid; idx < G * L; idx += FFT_THREADS) {
        int gl, k;
        if (ax == 0) { gl = idx / L; k = idx % L; } else { gl = idx % G; k = idx / G; }
        const int a = a0 + gl;
        if (a < na) g[(long long)a * sa + (long long)k * es] = dfc_store(sm[gl * LP + k]);
    }
}

// The same pass for lines of L = 3 M points (M = 2^LOGM): three radix-2
// transforms of the sub-sequences x[3n + r] (loaded bit-reversed), then one
// radix-3 step X[k + qM] = Y0[k] + w^q W^k Y1[k] + w^2q W^2k Y2[k], w = W^M,
// W = exp(sign 2 pi i / L).  The 3 x 2^k sizes put grids of odd lattice widths
// closer to 2n - 1 than the next power of two.
template <int LOGM>
__global__ void __launch_bounds__(FFT_THREADS) k_fft_axis3(double2 *data, long long gstride, int ax, int L0, int L1,
                                                           int na, int nb, int sign, const double2 *tw)
{
    constexpr int M = 1 << LOGM, L = 3 * M;
    constexpr int G = FFT_TILE / L;   // lines per CTA
    constexpr int LP = L + 1;
    extern __shared__ float4 sm[];
    float4 *stw = sm + G * LP;   // M / 2 twiddles of the length-M transforms
    float4 *stw3 = stw + M / 2;  // 2M twiddles W^j of the radix-3 step
    const double2 *tw3 = tw + FFT_LMAX / 2;
    const int tid = threadIdx.x;
    for (int k = tid; k < M / 2; k += FFT_THREADS) {
        const double2 w = tw[k * (FFT_LMAX / M)];
        stw[k] = dfc_load(make_double2(w.x, sign > 0 ? -w.y : w.y));
    }
    for (int j = tid; j < 2 * M; j += FFT_THREADS) {
        const double2 w = tw3[j * (FFT_L3MAX / L)];
        stw3[j] = dfc_load(make_double2(w.x, sign > 0 ? -w.y : w.y));
    }
    const int ntile = (na + G - 1) / G;
    const int a0 = (blockIdx.x % ntile) * G, b = blockIdx.x / ntile;
    if (b >= nb) return;
    long long sa, sb, es;
    if (ax == 0) { sa = L0; sb = (long long)L0 * L1; es = 1; }
    else if (ax == 1) { sa = 1; sb = (long long)L0 * L1; es = L0; }
    else { sa = 1; sb = L0; es = (long long)L0 * L1; }
    double2 *g = data + (long long)blockIdx.y * gstride + (long long)b * sb;
    // load: point k goes to sub-line k % 3 at the bit-reversed position of k / 3
    for (int idx = tid; idx < G * L; idx += FFT_THREADS) {
        int gl, k;
        if (ax == 0) { gl = idx / L; k = idx % L; } else { gl = idx % G; k = idx / G; }
        const int a = a0 + gl;
        if (a < na)
            sm[gl * LP + (k % 3) * M + (__brev(k / 3) >> (32 - LOGM))] = dfc_load(g[(long long)a * sa + (long long)k * es]);
    }
    __syncthreads();
#pragma unroll 1
    for (int s = 0; s < LOGM; ++s) {
        const int h = 1 << s;
        for (int j = tid; j < G * 3 * (M / 2); j += FFT_THREADS) {
            const int sub = j / (M / 2), bj = j % (M / 2);
            const int base = (sub / 3) * LP + (sub % 3) * M;
            const int grp = bj >> s, pos = bj & (h - 1);
            const int i0 = base + grp * 2 * h + pos, i1 = i0 + h;
            const float4 t = dfc_mul(stw[pos << (LOGM - 1 - s)], sm[i1]);
            const float4 u = sm[i0];
            sm[i0] = dfc_add(u, t);
            sm[i1] = dfc_sub(u, t);
        }
        __syncthreads();
    }
    // Im w = sign sin(2 pi / 3) as a double float; i Im(w) (y1 - y2) is (-c3 d.im, c3 d.re)
    const double c3d = (sign > 0 ? 1.0 : -1.0) * 0.86602540378443864676;
    const float c3h = (float)c3d, c3l = (float)(c3d - (double)c3h);
    for (int j = tid; j < G * M; j += FFT_THREADS) {
        const int base = (j / M) * LP, k = j % M;
        const float4 y0 = sm[base + k], y1 = dfc_mul(stw3[k], sm[base + M + k]),
                     y2 = dfc_mul(stw3[2 * k], sm[base + 2 * M + k]);
        const float4 sp = dfc_add(y1, y2), dm = dfc_sub(y1, y2);
        const float4 h0 = dfc_sub(y0, make_float4(0.5f * sp.x, 0.5f * sp.y, 0.5f * sp.z, 0.5f * sp.w));
        float4 rot;
        dfr_mul(-c3h, -c3l, dm.y, dm.w, rot.x, rot.z);
        dfr_mul(c3h, c3l, dm.x, dm.z, rot.y, rot.w);
        sm[base + k] = dfc_add(y0, sp);
        sm[base + M + k] = dfc_add(h0, rot);
        sm[base + 2 * M + k] = dfc_sub(h0, rot);
    }
    __syncthreads();
    for (int idx = tid; idx < G * L; idx += FFT_THREADS) {
        int gl, k;
        if (ax == 0) { gl = idx / L; k = idx % L; } else { gl = idx % G; k = idx / G; }
        const int a = a0 + gl;
        if (a < na) g[(long long)a * sa + (long long)k * es] = dfc_store(sm[gl * LP + k]);
    }
}

static int fft_pass(midas_gpu_ctx *c, double2 *data, long long gstride, int ngrids, int ax, const int L[3], int na,
                    int nb, int sign, const double2 *tw)
{
    const int len = L[ax];
    const int G = FFT_TILE / len;
    const int ntile = (na + G - 1) / G;
    const dim3 grd((unsigned)(ntile * nb), (unsigned)ngrids);
    if (len % 3 == 0) {   // 3 x 2^k
        const int m = len / 3, logm = 31 - __builtin_clz(m);
        const size_t smem = sizeof(double2) * ((size_t)G * (len + 1) + m / 2 + 2 * m);
        ++c->launches;
        switch (logm) {
#define FFT3_CASE(LG)                                                                                              \
    case LG:                                                                                                       \
        k_fft_axis3<LG><<<grd, FFT_THREADS, smem, c->stream>>>(data, gstride, ax, L[0], L[1], na, nb, sign, tw); \
        break;
            FFT3_CASE(3) FFT3_CASE(4) FFT3_CASE(5) FFT3_CASE(6) FFT3_CASE(7)
#undef FFT3_CASE
        default: return c->err.set(MIDAS_ERR_UNSUPPORTED, "lattice fft: mixed-radix axis length outside 24..384");
        }
        MIDAS_CUDA(c, cudaGetLastError());
        return MIDAS_OK;
    }
    const int logl = 31 - __builtin_clz(len);
    const size_t smem = sizeof(double2) * ((size_t)G * (len + 1) + len / 2);
    ++c->launches;
    switch (logl) {
#define FFT_CASE(LG)                                                                                              \
    case LG:                                                                                                      \
        k_fft_axis<LG><<<grd, FFT_THREADS, smem, c->stream>>>(data, gstride, ax, L[0], L[1], na, nb, sign, tw); \
        break;
        FFT_CASE(3) FFT_CASE(4) FFT_CASE(5) FFT_CASE(6) FFT_CASE(7) FFT_CASE(8) FFT_CASE(9)
#undef FFT_CASE
    default: return c->err.set(MIDAS_ERR_UNSUPPORTED, "lattice fft: axis length outside 8..512");
    }
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// 3-D transform of `ngrids` grids whose nonzero input occupies [0,n0) x [0,n1) x [0,n2)
// (forward) or whose needed output is that box (inverse).
static int fft3(midas_gpu_ctx *c, double2 *data, long long gstride, int ngrids, const int L[3], const int n[3],
                int sign, const double2 *tw)
{
    if (sign < 0) {
        MIDAS_TRY(fft_pass(c, data, gstride, ngrids, 0, L, n[1], n[2], sign, tw));   // x lines with y < n1, z < n2
        MIDAS_TRY(fft_pass(c, data, gstride, ngrids, 1, L, L[0], n[2], sign, tw));   // y lines with z < n2
        MIDAS_TRY(fft_pass(c, data, gstride, ngrids, 2, L, L[0], L[1], sign, tw));   // every z line
    } else {
        MIDAS_TRY(fft_pass(c, data, gstride, ngrids, 2, L, L[0], L[1], sign, tw));
        MIDAS_TRY(fft_pass(c, data, gstride, ngrids, 1, L, L[0], n[2], sign, tw));
        MIDAS_TRY(fft_pass(c, data, gstride, ngrids, 0, L, n[1], n[2], sign, tw));
    }
    return MIDAS_OK;
}

// dyad components on the circular offset grid: offset (di, dj, dk) at index
// (di mod L0, dj mod L1, dk mod L2) for |d| < n per axis, zero elsewhere and at 0
__global__ void k_dyad_grid(int L0, int L1, int L2, int n0, int n1, int n2, double d, double k0, double Pi,
                            int c4, double2 *G6, long long gstride)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long tot = (long long)L0 * L1 * L2;
    if (t >= tot) return;
    const int i = (int)(t % L0), j = (int)((t / L0) % L1), k = (int)(t / ((long long)L0 * L1));
    const int di = i < L0 / 2 ? i : i - L0, dj = j < L1 / 2 ? j : j - L1, dk = k < L2 / 2 ? k : k - L2;
    double2 F[6];
    if ((di == 0 && dj == 0 && dk == 0) || abs(di) >= n0 || abs(dj) >= n1 || abs(dk) >= n2) {
#pragma unroll
        for (int q = 0; q < 6; ++q) F[q] = make_double2(0, 0);
    } else if (c4) {
        float2 F4[6];
        dyadF4(di * d, dj * d, dk * d, k0, Pi, F4);
#pragma unroll
        for (int q = 0; q < 6; ++q) F[q] = make_double2(F4[q].x, F4[q].y);
    } else {
        dyadF8(di * d, dj * d, dk * d, k0, Pi, F);
    }
#pragma unroll
    for (int q = 0; q < 6; ++q) G6[q * gstride + t] = F[q];
}

// w_q = kc_s x_{3s+q} scattered into three zeroed grids per column
__global__ void k_lat_scatter(int ncell, const int *ijk, const int *lo, int L0, int L1, const double2 *fk8,
                              const float2 *fk4, const double2 *X, long long ldx, int col0, double2 *grids,
                              long long gstride)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ncell) return;
    const int col = col0 + blockIdx.y;
    const long long gi = ((long long)(ijk[3 * s + 2] - lo[2]) * L1 + (ijk[3 * s + 1] - lo[1])) * L0 +
                         (ijk[3 * s] - lo[0]);
    const double2 f = fk4 ? make_double2(fk4[s].x, fk4[s].y) : fk8[s];
    double2 *g = grids + (long long)blockIdx.y * 3 * gstride;
#pragma unroll
    for (int q = 0; q < 3; ++q) g[q * gstride + gi] = cmul(f, X[(long long)col * ldx + 3 * s + q]);
}

// Y_p = sum_q F^_pq W_q at every frequency, for every column of the batch (the
// spectra are read once per point and kept in registers across the columns)
__global__ void k_lat_pointwise(long long npts, const double2 *G6, long long gstride, double2 *grids, int ncol)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= npts) return;
    double2 F[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) F[q] = G6[q * gstride + t];
    for (int col = 0; col < ncol; ++col) {
        double2 *g = grids + (long long)col * 3 * gstride + t;
        const double2 wx = g[0], wy = g[gstride], wz = g[2 * gstride];
        const double2 yx = cmul(F[0], wx), yy = cmul(F[1], wy), yz = cmul(F[2], wz);
        const double2 xy = cmul(F[3], wy), xz = cmul(F[5], wz);
        const double2 yx2 = cmul(F[3], wx), yz2 = cmul(F[4], wz);
        const double2 zx = cmul(F[5], wx), zy = cmul(F[4], wy);
        g[0] = make_double2(yx.x + xy.x + xz.x, yx.y + xy.y + xz.y);
        g[gstride] = make_double2(yx2.x + yy.x + yz2.x, yx2.y + yy.y + yz2.y);
        g[2 * gstride] = make_double2(zx.x + zy.x + yz.x, zx.y + zy.y + yz.y);
    }
}

// Y = (1 - Znnpp) X - conv / Ntot, or, with B given, R = B - that (the residual)
__global__ void k_lat_gather(int ncell, const int *ijk, const int *lo, int L0, int L1, const double2 *znnpp,
                             const double2 *X, long long ldx, const double2 *B, long long ldb, double2 *Y,
                             long long ldy, int col0, const double2 *grids, long long gstride, double scale)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= ncell) return;
    const int col = col0 + blockIdx.y;
    const long long gi = ((long long)(ijk[3 * o + 2] - lo[2]) * L1 + (ijk[3 * o + 1] - lo[1])) * L0 +
                         (ijk[3 * o] - lo[0]);
    const double2 dg = make_double2(1.0 - znnpp[o].x, -znnpp[o].y);
    const double2 *g = grids + (long long)blockIdx.y * 3 * gstride;
#pragma unroll
    for (int p = 0; p < 3; ++p) {
        const double2 cv = g[p * gstride + gi];
        const double2 dx = cmul(dg, X[(long long)col * ldx + 3 * o + p]);
        double2 y = make_double2(dx.x - cv.x * scale, dx.y - cv.y * scale);
        if (B) {
            const double2 bb = B[(long long)col * ldb + 3 * o + p];
            y = make_double2(bb.x - y.x, bb.y - y.y);
        }
        Y[(long long)col * ldy + 3 * o + p] = y;
    }
}

// the smallest transform length >= v: a power of two from 8 or 3 x 2^k (24 .. 384)
static int fft_len(int v)
{
    int p = 8;
    while (p < v) p <<= 1;
    for (int q = 24; q <= FFT_L3MAX; q <<= 1)
        if (q >= v && q < p) return q;
    return p;
}

bool lattice_fft_fits(const midas_gpu_ctx *c)
{
    if (!c->lattice || !c->lat_ijk) return false;
    for (int a = 0; a < 3; ++a)
        if (fft_len(2 * (c->lat_hi[a] - c->lat_lo[a] + 1) - 1) > FFT_LMAX) return false;
    return true;
}

// The MoM solve takes its refinement residuals from the FFT operator when that
// is the cheaper product: per right-hand side the FP64 transforms of a padded
// grid of V points cost ~15 V log2 V double-float-MAC equivalents (six
// transforms of 5 V log2 V flops, ~1.75 of three passes each way, at the part's
// ~1 TFLOP/s FP64 against ~0.67e12 double-float complex MACs/s of the dense
// residual), the dense residual np^2.  Compact scatterers (spheres, cubes) have
// V ~ 8 n and take the FFT; sparse aggregates, whose bounding box pads to grids
// far larger than their cell count, take the dense residual.
bool lattice_fft_preferred(const midas_gpu_ctx *c, long long np)
{
    if (!lattice_fft_fits(c)) return false;
    double V = 1.0;
    for (int a = 0; a < 3; ++a) V *= fft_len(2 * (c->lat_hi[a] - c->lat_lo[a] + 1) - 1);
    return 15.0 * V * std::log2(V) < (double)np * (double)np;
}

// Lattice FFT set-up of the current cells: grid sizes and the dyad spectra (6
// grids) -- FP64 dyads (the MoM element) or, with c4, the complex(4)-rounded
// dyads of Green_s_tr_partial (src/Green_functions.f90:139-157).
int lattice_fft_prepare(midas_gpu_ctx *c, bool c4)
{
    if (!c->lattice || !c->lat_ijk) return c->err.set(MIDAS_ERR_UNSUPPORTED, "lattice fft: cells are not on a lattice");
    LatticeFft &f = c->lfft;
    if (f.version != c->cells_version) {   // new cells: both spectra sets are stale
        if (f.G6) cudaFree(f.G6);
        if (f.G6c4) cudaFree(f.G6c4);
        f.G6 = f.G6c4 = nullptr;
    }
    if (c4 ? f.G6c4 : f.G6) return MIDAS_OK;
    for (int a = 0; a < 3; ++a) {
        f.n[a] = c->lat_hi[a] - c->lat_lo[a] + 1;
        f.L[a] = fft_len(2 * f.n[a] - 1);
        if (f.L[a] > FFT_LMAX) return c->err.set(MIDAS_ERR_UNSUPPORTED, "lattice fft: lattice wider than 256 cells along an axis");
    }
    f.npts = (long long)f.L[0] * f.L[1] * f.L[2];
    if (!f.lo) MIDAS_CUDA(c, cudaMalloc(&f.lo, sizeof(int) * 4));
    MIDAS_CUDA(c, cudaMemcpyAsync(f.lo, c->lat_lo, sizeof(int) * 3, cudaMemcpyHostToDevice, c->stream));
    double2 *&G = c4 ? f.G6c4 : f.G6;
    MIDAS_CUDA(c, cudaMalloc(&G, sizeof(double2) * 6 * (size_t)f.npts));
    const double2 *tw;
    MIDAS_TRY(twiddles(c, &tw));
    ++c->launches;
    k_dyad_grid<<<(unsigned)((f.npts + 255) / 256), 256, 0, c->stream>>>(f.L[0], f.L[1], f.L[2], f.n[0], f.n[1],
                                                                          f.n[2], c->lat_d, c->k0, c->pi, c4 ? 1 : 0,
                                                                          G, f.npts);
    MIDAS_CUDA(c, cudaGetLastError());
    // the dyad grid is nonzero over the whole circular grid: full transforms
    const int full[3] = {f.L[0], f.L[1], f.L[2]};
    MIDAS_TRY(fft3(c, G, f.npts, 6, f.L, full, -1, tw));
    f.version = c->cells_version;
    return MIDAS_OK;
}

void lattice_fft_release(midas_gpu_ctx *c)
{
    if (c->lfft.G6) cudaFree(c->lfft.G6);
    if (c->lfft.G6c4) cudaFree(c->lfft.G6c4);
    if (c->lfft.lo) cudaFree(c->lfft.lo);
    c->lfft = LatticeFft();
}

// Y = Z X (B == nullptr) or Y = B - Z X, for nrhs columns (column-major, FP64;
// rows 3 * ncell of each column are read / written).  Scratch from `slot`.
// c4: the matrix of Green_s_tr_partial (complex(4)-rounded dyads and f_kapChe,
// their products formed in FP64) instead of the FP64 MoM element.
int lattice_matvec(midas_gpu_ctx *c, int nrhs, const double2 *X, long long ldx, const double2 *B, long long ldb,
                   double2 *Y, long long ldy, int slot, bool c4)
{
    MIDAS_TRY(lattice_fft_prepare(c, c4));
    LatticeFft &f = c->lfft;
    const double2 *tw;
    MIDAS_TRY(twiddles(c, &tw));
    // columns per batch: three grids each, batch scratch bounded to ~1 GB
    const size_t per_col = sizeof(double2) * 3 * (size_t)f.npts;
    const int batch = (int)std::max<size_t>(1, std::min<size_t>((size_t)nrhs, ((size_t)1 << 30) / per_col));
    void *p;
    MIDAS_TRY(ensure(c, slot, per_col * batch, &p));
    double2 *grids = (double2 *)p;
    const int ncell = c->n;
    const double scale = 1.0 / (double)f.npts;
    const int kp = kp_begin(c);
    for (int col0 = 0; col0 < nrhs; col0 += batch) {
        const int nb = std::min(batch, nrhs - col0);
        MIDAS_CUDA(c, cudaMemsetAsync(grids, 0, per_col * nb, c->stream));
        const dim3 grd((unsigned)((ncell + 127) / 128), (unsigned)nb);
        ++c->launches;
        k_lat_scatter<<<grd, 128, 0, c->stream>>>(ncell, c->lat_ijk, f.lo, f.L[0], f.L[1], c->fk8,
                                                  c4 ? c->fk4 : nullptr, X, ldx, col0, grids, f.npts);
        MIDAS_CUDA(c, cudaGetLastError());
        MIDAS_TRY(fft3(c, grids, f.npts, 3 * nb, f.L, f.n, -1, tw));
        ++c->launches;
        k_lat_pointwise<<<(unsigned)((f.npts + 127) / 128), 128, 0, c->stream>>>(f.npts, c4 ? f.G6c4 : f.G6, f.npts,
                                                                                  grids, nb);
        MIDAS_CUDA(c, cudaGetLastError());
        MIDAS_TRY(fft3(c, grids, f.npts, 3 * nb, f.L, f.n, +1, tw));
        ++c->launches;
        k_lat_gather<<<grd, 128, 0, c->stream>>>(ncell, c->lat_ijk, f.lo, f.L[0], f.L[1], c->znnpp, X, ldx, B, ldb, Y,
                                                 ldy, col0, grids, f.npts, scale);
        MIDAS_CUDA(c, cudaGetLastError());
    }
    // algorithmic work: 6 complex FFTs (5 N log2 N each) + 9 complex MACs per point, per column;
    // bytes: X, Y (and B) once
    const double lg = log2((double)f.npts);
    kp_end(c, kp, MIDAS_KC_LATTICE, nrhs * (6 * 5.0 * f.npts * lg + 72.0 * f.npts),
           16.0 * 3 * ncell * nrhs * (B ? 3 : 2));
    return MIDAS_OK;
}

}  // namespace midas
