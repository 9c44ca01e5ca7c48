// cbfm.cu -- CBFM-E solve on the GPU: Compute_EFields_CBFME
// (src/Compute_EFields_CBFME.f90:1-1006), optionally with ACA off-diagonal
// reduced blocks (src/Compute_EFields_CBFME_ACA.f90:588-635).
//
// Pipeline (reference line numbers in brackets):
//   1. per block b, extended cells = block cells + extension cells [348-358]
//      a. fSR ladder (setfSR) [221-244]
//      b. thresholded extended-block matrix (SR_Green_s_tr_partial, dense form) [385-397]
//      c. CBF excitations (Incident_Field, complex(4) locals) [361-369]
//      d. solve Z_ext X = E_ref: no-pivot TF32 tensor LU + refinement with a
//         double-float residual (PARDISO with 20 refinement steps in the reference) [396]
//      e. SVD of X by its Gram matrix X^H X (FP64) and a Hermitian eigen-solver; keep
//         sigma_i / sigma_1 >= Threshold_CBFM; C_b = (X V_K Sigma_K^-1)[rows of the
//         non-extended block] [419-445] -- the span of the retained left singular
//         vectors, which is all the reduced system depends on.
//   2. T = Z(:, block j) C_j for every block column (complex(4)-rounded fill, FP32-grade
//      3xTF32 tensor GEMM) and Zc(i, :) = C_i^T T(rows of i) -- plain transpose as
//      ZGEMM('T','N') [630-809].  With ACA, every off-diagonal pair first runs the
//      partial-pivot ACA (one CTA per pair, one launch for all pairs); a pair whose
//      rank stays below Nb_it_max contributes T(rows of i, cols of j) = U (V C_j)
//      instead of its dense fill (src/Compute_EFields_CBFME_ACA.f90:588-635).
//   3. Vc = C^T Einc [829-849], reduced solve (mixed LU + FP64 refinement) [873-943],
//      E = C alpha [990-1006].
#include <algorithm>
#include <cuda_fp16.h>

#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <mutex>
#include <thread>

#include "common.cuh"
#include "kernels.cuh"

namespace midas {

int zgemm64(midas_gpu_ctx *c, int M, int N, int K, const double2 *A, long long ars, long long acs, int conjA,
            const double2 *B, long long brs, long long bcs, double2 *C, long long crs, long long ccs, double2 alpha,
            double2 beta);
template <typename TA, typename TB>
int zgemm_x3(midas_gpu_ctx *c, int M, int N, int K, const TA *A, long long ars, long long acs, int conjA,
             const TB *B, long long brs, long long bcs, float *D, long long ldd, float alpha, float beta);
template <typename TB>
int zgemm_x3_a3(midas_gpu_ctx *c, int M, int N, int K, const float *A3, long long K6, const TB *B, long long brs,
                long long bcs, float *D, long long ldd, float alpha, float beta, int kclass = MIDAS_KC_GEMM_PROD);
int zsplit_a3_h16(midas_gpu_ctx *c, int M, int K, const float2 *A, long long lda, __half *A3, long long K6h,
                  float *sc);
int resid_update_x3(midas_gpu_ctx *c, int n, int m, const __half *A3h, long long K6h, float *sc, const float2 *D,
                    float *P, double2 *R);
template <typename TB>
int zgemm_x3h_a3(midas_gpu_ctx *c, int M, int N, int K, const __half *A3h, long long K6h, float *sc, const TB *B,
                 long long brs, long long bcs, float *D, long long ldd, int kclass, int promote_kb = 2);
int set_h16_scale(midas_gpu_ctx *c, float *sc, float s);
template <typename TA, typename TB>
int zgemm_x3h(midas_gpu_ctx *c, int M, int N, int K, const TA *A, long long ars, long long acs, const TB *B,
              long long brs, long long bcs, float *D, long long ldd, int kclass, int promote_kb = 2);
int residual_df32(midas_gpu_ctx *c, int n, int nrhs, const float2 *Z, long long ldz, const float2 *Xh,
                  const float2 *Xl, const float2 *B, double2 *R);
int heev_dev(midas_gpu_ctx *c, int batch, int m, double2 *A, long long lda, long long sa, double2 *H, double2 *V,
             long long sv, double *W);
size_t gram_df_scratch_bytes(int m);
int zgemm_df(midas_gpu_ctx *c, int M, int N, int K, const double2 *A, long long ars, long long acs,
             const double2 *B, long long brs, long long bcs, double2 *C, long long crs, long long ccs);
int gram_df(midas_gpu_ctx *c, int m, int K, const float2 *Xh, const float2 *Xl, long long rs, long long cs,
            double2 *G, float4 *P);

static inline int pad64(int x) { return (x + 63) / 64 * 64; }

__global__ void k_pad_diag32(float2 *Z, long long ld, int n0, int np)
{
    int i = n0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < np) Z[(long long)i * ld + i] = make_float2(1.f, 0.f);
}

// X64 += d32 ; Xh = fp32(X64) ; Xl = fp32(X64 - Xh)   (n x m column-major, ld n);
// with rm = 1, Xh and Xl are written row-major (n rows of ldx) for the CSR
// residual and the correction d row-major (n x m) into Drm
__global__ void k_ir_update(long long tot, int n, int m, double2 *X64, const float2 *d32, float2 *Xh, float2 *Xl,
                            float2 *Drm, int first, int rm, int ldx)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= tot) return;
    double2 x = first ? make_double2(d32[i].x, d32[i].y) : make_double2(X64[i].x + d32[i].x, X64[i].y + d32[i].y);
    X64[i] = x;
    float2 h = make_float2((float)x.x, (float)x.y);
    const long long o = rm ? (i % n) * ldx + i / n : i;
    Xh[o] = h;
    Xl[o] = make_float2((float)(x.x - h.x), (float)(x.y - h.y));
    if (Drm) Drm[rm ? (i % n) * m + i / n : i] = d32[i];   // the correction, for the FP32 residual update
}

// d = fp32(r) and x += d, for the correction of the reduced solution
__global__ void k_c64_to_c32(long long tot, const double2 *r, float2 *d)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < tot) d[i] = make_float2((float)r[i].x, (float)r[i].y);
}
__global__ void k_add_c32(long long tot, const float2 *d, double2 *x)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < tot) x[i] = make_double2(x[i].x + d[i].x, x[i].y + d[i].y);
}

// R = B (FP64 copy of the FP32 right-hand sides)
__global__ void k_b_to_r64(long long tot, const float2 *B, double2 *R)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < tot) R[i] = make_double2(B[i].x, B[i].y);
}

// d32 = fp32(r); per-column max |r| and max |x| into red (bit patterns of >= 0 doubles)
__global__ void k_r_to32(int n, int m, const double2 *r, float2 *d32, const double2 *X64,
                         unsigned long long *red)
{
    int col = blockIdx.y;
    double mr = 0, mx = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double2 v = r[(long long)col * n + i];
        d32[(long long)col * n + i] = make_float2((float)v.x, (float)v.y);
        mr = fmax(mr, fmax(fabs(v.x), fabs(v.y)));
        double2 x = X64[(long long)col * n + i];
        mx = fmax(mx, fmax(fabs(x.x), fabs(x.y)));
    }
    for (int o = 16; o > 0; o >>= 1) {
        mr = fmax(mr, __shfl_down_sync(0xffffffffu, mr, o));
        mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(red + col, __double_as_longlong(mr));
        atomicMax(red + m + col, __double_as_longlong(mx));
    }
}

// V[:, j] *= 1 / sigma_j  for j < K   (V row-major m x m)
__global__ void k_scale_cols(int m, int K, double2 *V, const double *W)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m * K) return;
    int r = t / K, j = t % K;
    double s = sqrt(fmax(W[j], 0.0));
    double f = s > 0 ? 1.0 / s : 0.0;
    V[(long long)r * m + j].x *= f;
    V[(long long)r * m + j].y *= f;
}

// Zc (fp32 floats, row-major ld ldf) -> Z64/Z32 padded (np x np row-major)
// the reduced system from Zc (compact rows; column j of the system is Zc's column colmap[j])
__global__ void k_zc_to_sys(int K, const float *Zf, long long ldf, const int *colmap, double2 *Z64, float2 *Z32,
                            long long np)
{
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)np * np) return;
    int i = (int)(t / np), j = (int)(t % np);
    float2 v = make_float2(0.f, 0.f);
    if (i < K && j < K) {
        const long long q = (long long)i * ldf + 2LL * colmap[j];
        v = make_float2(Zf[q], Zf[q + 1]);
    }
    else if (i == j) v = make_float2(1.f, 0.f);
    Z64[t] = make_double2(v.x, v.y);
    Z32[t] = v;
}

__global__ void k_iota(int *p, int n, int base)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = base + i;
}

struct Buf {
    midas_gpu_ctx *c;
    size_t off = 0;
    char *base = nullptr;
    template <typename T>
    T *take(size_t count)
    {
        off = (off + 255) & ~(size_t)255;
        T *p = (T *)(base + off);
        off += sizeof(T) * count;
        return p;
    }
};

// Read-only description of the CBF generation shared by the lanes.
struct CbfShared {
    const int *bo, *xo;            // host: block / extended-block offsets
    const int *d_xall;             // device: cell indices of every extended block
    const double *d_cth, *d_cph;   // device: CBF excitation directions
    int ncbf, m;
    bool sr, homog;
    double res_sr, cbf_tol;
    double2 *Xall;                 // device: FP64 block solutions (output)
    const size_t *xoff;
    double2 *Gall;                 // device: Gram matrices (output)
    size_t mm;
    int *srefine;                  // host: refinement steps per block (output)
    bool spherical;                // CBF excitations by Incident_Field_Spherical (type_iws = 2/3)
};

static int cbf_block(midas_gpu_ctx *c, const CbfShared &S, int b)
{
    const int *bo = S.bo, *xo = S.xo, m = S.m, ncbf = S.ncbf;
    const bool sr = S.sr, homog = S.homog;
    const double res_sr = S.res_sr, cbf_tol = S.cbf_tol;
    const int *d_xall = S.d_xall;
    const double *d_cth = S.d_cth, *d_cph = S.d_cph;
    {
        const int s = xo[b + 1] - xo[b];
        const int N3 = 3 * s, sp = pad64(N3);
        const int *idx = d_xall + xo[b];
        double2 *X64 = S.Xall + S.xoff[b];
        // work buffers of this lane (grow-only; the lane takes its blocks largest first)
        const size_t nrm = (size_t)sp * m;
        // row stride of the row-major Xh / Xl the CSR residual reads (its column groups, no tail)
        const int ldx = sr ? csr_resid_ldx(m) : m;
        const size_t nrx = (size_t)sp * ldx;
        void *p1, *p2 = nullptr, *p3, *pred;
        MIDAS_TRY(ensure(c, S_CBF1, sizeof(float2) * (size_t)sp * sp, &p1));
        if (!sr) MIDAS_TRY(ensure(c, S_CBF2, sizeof(float2) * (size_t)sp * sp, &p2));
        MIDAS_TRY(ensure(c, S_CBF3, (sizeof(float2) * 3 + sizeof(double2)) * nrm + sizeof(float2) * 2 * nrx + 8 * 256,
                         &p3));
        MIDAS_TRY(ensure(c, S_RED2, sizeof(unsigned long long) * 2 * m + 64, &pred));
        float2 *Zlu = (float2 *)p1, *Zsr = (float2 *)p2;
        Buf b3{c, 0, (char *)p3};
        float2 *Bm = b3.take<float2>(nrm), *Xh = b3.take<float2>(nrx), *Xl = b3.take<float2>(nrx),
               *d32 = b3.take<float2>(nrm), *Drm = b3.take<float2>(nrm);
        double2 *R64 = b3.take<double2>(nrm);
        unsigned long long *red = (unsigned long long *)pred;
        std::vector<unsigned long long> hred(2 * m);
        double thr_sr = 0.0;
        if (sr) {
            double fsr;
            long long nnz;
            MIDAS_TRY(sr_ladder(c, s, idx, bo[b], homog, res_sr, &fsr, &nnz, 0, nullptr, nullptr, nullptr));
            double2 zn;
            MIDAS_CUDA(c, cudaMemcpyAsync(&zn, c->znnpp + bo[b], sizeof(double2), cudaMemcpyDeviceToHost, c->stream));
            MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
            thr_sr = hypot(1 - zn.x, -zn.y) / fsr;
            if (c->opts.verbose >= 2) fprintf(stderr, "[midas] cbf block %d: fSR=%g nnz=%lld thr=%.17g\n", b, fsr, nnz, thr_sr);
        }
        // the thresholded block goes straight into the LU buffer; with SR its CSR
        // form (about a sixth of the entries) serves the refinement residuals,
        // without SR a dense copy does
        MIDAS_CUDA(c, cudaMemsetAsync(Zlu, 0, sizeof(float2) * (size_t)sp * sp, c->stream));
        MIDAS_TRY(launch_block_fill4<float2>(c, s, idx, s, idx, sr ? 1 : 0, thr_sr, homog, Zlu, (size_t)sp, 1));
        if (sp > N3) {
            ++c->launches;
            k_pad_diag32<<<1, 64, 0, c->stream>>>(Zlu, sp, N3, sp);
        }
        // With SR, the thresholded block is kept twice before the LU overwrites it:
        // in CSR form for the double-float residual (CUDA cores, a sixth of the
        // dense work) and as the split-TF32 operand A3 for the FP32-grade residual
        // updates r -= Z d (dense, on the tensor cores).
        Csr zcsr;
        __half *A3z = nullptr;
        float *A3sc = nullptr;   // the split's scales (4 floats after it)
        const long long K6z = h16_arow(sp);
        if (sr) {
            MIDAS_TRY(csr_from_dense(c, sp, Zlu, sp, S_CSR, &zcsr));
            MIDAS_TRY(ensure(c, S_CBF2, sizeof(__half) * (size_t)sp * (size_t)K6z + 256, &p2));
            A3z = (__half *)p2;
            A3sc = (float *)(A3z + (size_t)sp * (size_t)K6z);
            MIDAS_TRY(zsplit_a3_h16(c, sp, sp, Zlu, sp, A3z, K6z, A3sc));
        } else
            MIDAS_CUDA(c, cudaMemcpyAsync(Zsr, Zlu, sizeof(float2) * (size_t)sp * sp, cudaMemcpyDeviceToDevice,
                                          c->stream));
        MIDAS_CUDA(c, cudaMemsetAsync(Bm, 0, sizeof(float2) * (size_t)sp * m, c->stream));
        // CBF excitations: plane waves (type_iws = 1) or spherical waves (type_iws = 2/3),
        // src/Compute_EFields_CBFME.f90:363-368
        if (S.spherical)
            MIDAS_TRY(launch_incident_sph<float2>(c, s, idx, ncbf, d_cth, d_cph, Bm, 1, (size_t)sp));
        else
            MIDAS_TRY(launch_incident4<float2>(c, s, idx, ncbf, d_cth, d_cph, Bm, 1, (size_t)sp));
        DenseLU lu;
        lu.n = sp;
        lu.A = Zlu;
        lu.lda = sp;
        MIDAS_TRY(lu_factor_nopiv(c, lu));
        // x0 = LU^-1 B, then refinement with the double-float residual
        MIDAS_CUDA(c, cudaMemcpyAsync(d32, Bm, sizeof(float2) * (size_t)sp * m, cudaMemcpyDeviceToDevice, c->stream));
        MIDAS_TRY(lu_solve(c, lu, d32, m));
        long long tot = (long long)sp * m;
        ++c->launches;
        k_ir_update<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(tot, sp, m, X64, d32, Xh, Xl,
                                                                          sr ? Drm : nullptr, 1, sr, ldx);
        // Residuals.  The first, B - Z x0, is needed only to ~1e-3 of itself (x0 from
        // the TF32 factors is ~1e-3.5 off), so it is formed as an FP32-grade
        // split-TF32 product on the tensor cores.  Then double-float B - Z x on the
        // CSR form while the corrections are large; once the relative residual is
        // below 1e-5 every later correction d is ~1e-5 |x| or smaller, and r - Z d
        // as the same split-TF32 product (relative error ~2^-22 of |Z||d|) keeps the
        // computed residual within ~1e-11 |x| of the true one.
        int it;
        bool upd = false;
        for (it = 0; it < 12; ++it) {
            if (sr && it == 0) {
                ++c->launches;
                k_b_to_r64<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(tot, Bm, R64);
                MIDAS_TRY(resid_update_x3(c, sp, m, A3z, K6z, A3sc, Drm, (float *)d32, R64));
            } else if (sr && upd)
                MIDAS_TRY(resid_update_x3(c, sp, m, A3z, K6z, A3sc, Drm, (float *)d32, R64));
            else if (sr)
                MIDAS_TRY(residual_csr_df32(c, zcsr, m, ldx, Xh, Xl, Bm, R64));
            else
                MIDAS_TRY(residual_df32(c, sp, m, Zsr, sp, Xh, Xl, Bm, R64));
            MIDAS_CUDA(c, cudaMemsetAsync(red, 0, sizeof(unsigned long long) * 2 * m, c->stream));
            ++c->launches;
            k_r_to32<<<dim3(32, m), 256, 0, c->stream>>>(sp, m, R64, d32, X64, red);
            MIDAS_CUDA(c, cudaMemcpyAsync(hred.data(), red, sizeof(unsigned long long) * 2 * m,
                                          cudaMemcpyDeviceToHost, c->stream));
            MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
            MIDAS_TRY(check_flag(c, "cbf block solve"));
            double worst = 0;
            for (int k = 0; k < m; ++k) {
                double rn, xn;
                memcpy(&rn, &hred[k], 8);
                memcpy(&xn, &hred[m + k], 8);
                worst = std::max(worst, xn > 0 ? rn / xn : rn);
            }
            if (!(worst == worst)) return c->err.set(MIDAS_ERR_NOT_CONVERGED, "cbf block solve: NaN");
            if (worst <= cbf_tol && !(sr && it == 0)) break;   // the FP32 first residual never ends it
            upd = sr && it > 0 && worst <= 1e-5;
            MIDAS_TRY(lu_solve(c, lu, d32, m));
            ++c->launches;
            k_ir_update<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(tot, sp, m, X64, d32, Xh, Xl,
                                                                              upd ? Drm : nullptr, 0, sr, ldx);
        }
        if (it == 12) return c->err.set(MIDAS_ERR_NOT_CONVERGED, "cbf block solve: refinement did not converge");
        // Gram G = X^H X over the 3s rows of the extended block, in double float from
        // the refinement's hi/lo copies of X (row-major with SR, column-major without)
        void *pg;
        MIDAS_TRY(ensure(c, S_CBF9, gram_df_scratch_bytes(m), &pg));
        MIDAS_TRY(gram_df(c, m, N3, Xh, Xl, sr ? ldx : 1, sr ? 1 : sp, S.Gall + S.mm * b, (float4 *)pg));
        S.srefine[b] = it;
    }
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// Lanes: the extended blocks are independent, so CBF generation runs NLANES
// blocks at once, each lane a host thread driving its own stream and scratch
// pool (the cells and lattice tables are shared read-only).  The latency-bound
// parts of one block (diagonal LUs, small GEMMs, host checks of the
// refinement) then overlap the bandwidth-bound parts of another.  The lanes
// live as long as the context.
// ---------------------------------------------------------------------------
// default lanes; MIDAS_CBFM_LANES (1..16) overrides.  Measured on the 41k-cell scene with the
// eigen-solves streamed (12-step means): 5 lanes 1026 ms, 6 989-1000 ms, 7 962-973 ms, 8 964 ms
constexpr int CBF_LANES = 7;

static int cbf_lanes()
{
    const char *e = getenv("MIDAS_CBFM_LANES");
    int v = e ? atoi(e) : CBF_LANES;
    return v < 1 ? 1 : (v > 16 ? 16 : v);
}

static void lane_sync_cells(midas_gpu_ctx *L, const midas_gpu_ctx *c)
{
    L->opts = c->opts;
    L->device = c->device;
    L->pi = c->pi;
    L->n = c->n; L->k0 = c->k0;
    L->x = c->x; L->y = c->y; L->z = c->z; L->sc = c->sc; L->an = c->an; L->kappa = c->kappa;
    L->eps = c->eps; L->che = c->che; L->znnpp = c->znnpp; L->fk4 = c->fk4; L->fk8 = c->fk8;
    L->lattice = c->lattice; L->lat_d = c->lat_d;
    for (int i = 0; i < 3; ++i) {
        L->lat_o[i] = c->lat_o[i]; L->lat_lo[i] = c->lat_lo[i]; L->lat_hi[i] = c->lat_hi[i];
        L->lat_dim[i] = c->lat_dim[i];
    }
    L->lat_ijk = c->lat_ijk; L->lat_tab4 = c->lat_tab4; L->lat_tab8 = c->lat_tab8;
    L->kprof.on = c->kprof.on;
    L->err = Err();
}

static int get_lanes(midas_gpu_ctx *c, int nl)
{
    while ((int)c->lanes.size() < nl) {
        midas_gpu_ctx *L = new midas_gpu_ctx;
        L->device = c->device;
        L->pool.resize(S_NSLOTS);
        const bool first = c->lanes.empty();
        c->lanes.push_back(L);
        // lane 0 starts with the largest block, the critical path of the step: its
        // stream has the highest priority, so its CTAs are scheduled first when SMs free up
        int least = 0, greatest = 0;
        MIDAS_CUDA(c, cudaDeviceGetStreamPriorityRange(&least, &greatest));
        MIDAS_CUDA(c, cudaStreamCreateWithPriority(&L->stream, cudaStreamNonBlocking, first ? greatest : least));
        MIDAS_CUDA(c, cudaMalloc(&L->d_flag, sizeof(int)));
        MIDAS_CUDA(c, cudaMemset(L->d_flag, 0, sizeof(int)));
    }
    return MIDAS_OK;
}

void free_lanes(midas_gpu_ctx *c)
{
    for (midas_gpu_ctx *L : c->aux) c->lanes.push_back(L);
    c->aux.clear();
    for (midas_gpu_ctx *L : c->lanes) {
        if (L->stream) cudaStreamSynchronize(L->stream);
        for (auto &d : L->pool)
            if (d.p) cudaFree(d.p);
        if (L->d_flag) cudaFree(L->d_flag);
        for (cudaEvent_t e : L->kprof.ev) cudaEventDestroy(e);
        destroy_side(L);
        if (L->stream) cudaStreamDestroy(L->stream);
        delete L;   // the cell arrays belong to the parent context
    }
    c->lanes.clear();
}

// Auxiliary contexts of the streamed CBFM pipeline (own stream and scratch pool, the
// cells aliased): aux[0 .. CBF_FINISHERS) finish blocks (K_b, C_b and the
// reduced-assembly column of block b) at the lowest stream priority (a second stream,
// overlapping one column's fill with another's product, measured no faster: both are
// bandwidth-bound); aux[CBF_FINISHERS + l] runs the eigen-solves of lane l's blocks at
// the highest (one CTA each, on the tail of the step).
constexpr int CBF_FINISHERS = 1;
static int get_aux(midas_gpu_ctx *c, int na)
{
    while ((int)c->aux.size() < na) {
        midas_gpu_ctx *A = new midas_gpu_ctx;
        A->device = c->device;
        A->pool.resize(S_NSLOTS);
        const bool finisher = (int)c->aux.size() < CBF_FINISHERS;
        c->aux.push_back(A);
        int least = 0, greatest = 0;
        MIDAS_CUDA(c, cudaDeviceGetStreamPriorityRange(&least, &greatest));
        MIDAS_CUDA(c, cudaStreamCreateWithPriority(&A->stream, cudaStreamNonBlocking, finisher ? least : greatest));
        MIDAS_CUDA(c, cudaMalloc(&A->d_flag, sizeof(int)));
        MIDAS_CUDA(c, cudaMemset(A->d_flag, 0, sizeof(int)));
    }
    return MIDAS_OK;
}

// on_done(L, l, b), when given, runs on lane l's host thread after block b's
// Gram matrix is enqueued on L's stream; *idle, when given, counts the lanes whose
// work has drained (no block left to take, their stream idle)
static int cbf_generate(midas_gpu_ctx *c, int nb, const CbfShared &S,
                        const std::function<int(midas_gpu_ctx *, int, int)> *on_done = nullptr,
                        std::atomic<int> *idle = nullptr)
{
    // with kernel-class profiling on, one lane: each launch's event interval then
    // covers that kernel alone
    const int nl = c->kprof.on ? 1 : std::min(nb, cbf_lanes());
    MIDAS_TRY(get_lanes(c, nl));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));   // the shared inputs are on the device
    // largest blocks first; lane 0 (highest-priority stream) takes the largest, and
    // every lane then pulls the next block from a shared counter as it finishes one,
    // so the lanes end within about one small block of each other
    std::vector<int> order(nb);
    for (int b = 0; b < nb; ++b) order[b] = b;
    auto sz = [&](int b) { return S.xo[b + 1] - S.xo[b]; };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b2) { return sz(a) > sz(b2); });
    std::atomic<int> next{nl > 1 ? 1 : 0};
    std::vector<std::vector<int>> done_by(nl);
    std::vector<long long> l0(nl);
    for (int l = 0; l < nl; ++l) {
        lane_sync_cells(c->lanes[l], c);
        l0[l] = c->lanes[l]->launches;
    }
    std::atomic<int> fail{0};
    std::vector<int> status(nl, MIDAS_OK);
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<double> lane_ms(nl, 0.0);
    // verbose: the device-side end of every block, by events on the lanes' streams
    const bool timeline = c->opts.verbose >= 1;
    cudaEvent_t ev0 = nullptr;
    std::vector<std::vector<cudaEvent_t>> ev_end(nl);
    if (timeline) {
        cudaEventCreate(&ev0);
        cudaEventRecord(ev0, c->stream);
    }
    auto work = [&](int l) {
        midas_gpu_ctx *L = c->lanes[l];
        cudaSetDevice(L->device);
        for (int q = (l == 0 && nl > 1) ? 0 : next++; q < nb; q = next++) {
            if (fail.load()) break;
            const int b = order[q];
            done_by[l].push_back(b);
            const auto tb = std::chrono::steady_clock::now();
            int st = cbf_block(L, S, b);
            if (st == MIDAS_OK && on_done) st = (*on_done)(L, l, b);
            if (st != MIDAS_OK) { status[l] = st; fail = 1; break; }
            if (timeline) {
                cudaEvent_t ev;
                cudaEventCreate(&ev);
                cudaEventRecord(ev, L->stream);
                ev_end[l].push_back(ev);
            }
            if (c->opts.verbose >= 2) {
                cudaStreamSynchronize(L->stream);
                const auto te = std::chrono::steady_clock::now();
                fprintf(stderr, "[midas] cbf lane %d block %d (s=%d): %.0f -> %.0f ms\n", l, b, sz(b),
                        std::chrono::duration<double, std::milli>(tb - t0).count(),
                        std::chrono::duration<double, std::milli>(te - t0).count());
            }
        }
        const cudaError_t se = cudaStreamSynchronize(L->stream);
        if (idle) ++*idle;
        if (se != cudaSuccess && status[l] == MIDAS_OK) {
            status[l] = L->err.set(MIDAS_ERR_CUDA, "cbf lane: stream failed");
            fail = 1;
        }
        lane_ms[l] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    };
    std::vector<std::thread> th;
    for (int l = 1; l < nl; ++l) th.emplace_back(work, l);
    work(0);
    for (auto &t : th) t.join();
    for (int l = 0; l < nl; ++l) {
        midas_gpu_ctx *L = c->lanes[l];
        c->launches += L->launches - l0[l];
        if (L->kprof.on) {
            kp_flush(L);
            for (int k = 0; k < MIDAS_KC_COUNT; ++k) {
                c->kprof.ms[k] += L->kprof.ms[k]; c->kprof.flops[k] += L->kprof.flops[k];
                c->kprof.bytes[k] += L->kprof.bytes[k]; c->kprof.n[k] += L->kprof.n[k];
                L->kprof.ms[k] = L->kprof.flops[k] = L->kprof.bytes[k] = 0; L->kprof.n[k] = 0;
            }
        }
    }
    if (timeline) {
        for (int l = 0; l < nl; ++l) {
            fprintf(stderr, "[midas] cbf lane %d (block:cells@end ms):", l);
            for (size_t q = 0; q < ev_end[l].size(); ++q) {
                float t = 0;
                cudaEventElapsedTime(&t, ev0, ev_end[l][q]);
                const int b = done_by[l][q];
                fprintf(stderr, " %d:%d@%.0f", b, sz(b), t);
                cudaEventDestroy(ev_end[l][q]);
            }
            fprintf(stderr, "\n");
        }
        cudaEventDestroy(ev0);
    }
    if (c->opts.verbose >= 1) {
        fprintf(stderr, "[midas] cbf lanes (finish ms / blocks):");
        for (int l = 0; l < nl; ++l) fprintf(stderr, " %.0f/%zu", lane_ms[l], done_by[l].size());
        fprintf(stderr, "\n");
    }
    for (int l = 0; l < nl; ++l)
        if (status[l] != MIDAS_OK) return c->err.set(status[l], c->lanes[l]->err.msg);
    return MIDAS_OK;
}

int cbfm_run(midas_gpu_ctx *c, int nb, const int *blk_offsets, const int *ext_offsets, const int *ext_idx, int ncbf,
             const double *cbf_theta, const double *cbf_phi, double thr_cbf, double res_sr, int flags, double eps_aca,
             int aca_itmax, int ntr, const double *theta, const double *phi, double2 *E_user, int *K_user,
             midas_gpu_info *info)
{
    auto tw0 = std::chrono::steady_clock::now();
    if (info) memset(info, 0, sizeof(*info));
    const int base = c->opts.index_base;
    const int n = c->n;
    // ---- host copies of the partition (small) ------------------------------
    std::vector<int> bo(nb + 1), eo(nb + 1);
    MIDAS_CUDA(c, cudaMemcpy(bo.data(), blk_offsets, sizeof(int) * (nb + 1), cudaMemcpyDefault));
    MIDAS_CUDA(c, cudaMemcpy(eo.data(), ext_offsets, sizeof(int) * (nb + 1), cudaMemcpyDefault));
    for (auto &v : bo) v -= base;
    for (auto &v : eo) v -= base;
    if (bo[0] != 0 || bo[nb] != n) return c->err.set(MIDAS_ERR_ARG, "cbfm: block offsets must cover all cells");
    for (int b = 0; b < nb; ++b)
        if (bo[b + 1] <= bo[b] || eo[b + 1] < eo[b]) return c->err.set(MIDAS_ERR_ARG, "cbfm: bad offsets");
    if (eo[0] != 0) return c->err.set(MIDAS_ERR_ARG, "cbfm: ext offsets must start at the index base");
    std::vector<int> ext(std::max(eo[nb], 1));
    if (eo[nb] > 0) {
        if (!ext_idx) return c->err.set(MIDAS_ERR_ARG, "cbfm: ext_idx missing");
        MIDAS_CUDA(c, cudaMemcpy(ext.data(), ext_idx, sizeof(int) * eo[nb], cudaMemcpyDefault));
        for (int i = 0; i < eo[nb]; ++i) {
            ext[i] -= base;
            if (ext[i] < 0 || ext[i] >= n) return c->err.set(MIDAS_ERR_ARG, "cbfm: extension cell out of range");
        }
    }
    const int m = 2 * ncbf;
    const bool sr = flags & MIDAS_CBFM_SR, homog = flags & MIDAS_CBFM_HOMOG;
    const bool use_aca = flags & MIDAS_CBFM_ACA;
    if (!(res_sr > 0)) res_sr = (double)1e-2f;
    if (!(eps_aca > 0)) eps_aca = (double)1e-4f;        // Epsilon_ACA (src/InOut_ReadWrite_Functions.f90:396)
    if (aca_itmax <= 0) aca_itmax = 50;                 // Nb_it_max
    if (use_aca && (aca_itmax < 2 || aca_itmax > ACA_MAX_IT))
        return c->err.set(MIDAS_ERR_ARG, "cbfm: aca_itmax must be in [2, 128]");
    // the ACA driver fixes Threshold_CBFM = 1e-3 (src/Compute_EFields_CBFME_ACA.f90:124)
    if (use_aca && !(thr_cbf > 0)) thr_cbf = (double)1e-3f;
    // ---- Threshold_CBFM from max |m| (src/Compute_EFields_CBFME.f90:286-288) ----
    if (!(thr_cbf > 0)) {
        std::vector<double2> eps(n);
        MIDAS_CUDA(c, cudaMemcpy(eps.data(), c->eps, sizeof(double2) * n, cudaMemcpyDeviceToHost));
        double mmax = 0;
        for (auto &e : eps) mmax = std::max(mmax, sqrt(hypot(e.x, e.y)));
        double rel = ceil(mmax) - 2.0;
        thr_cbf = std::max(pow(10.0, -3.0 - rel), (double)1e-10f);
    }
    // ---- index lists: extended block b = [block cells, extension cells] ------
    std::vector<int> xo(nb + 1, 0), xall;
    int smax = 0, nbmax = 0;
    for (int b = 0; b < nb; ++b) {
        for (int i = bo[b]; i < bo[b + 1]; ++i) xall.push_back(i);
        for (int i = eo[b]; i < eo[b + 1]; ++i) xall.push_back(ext[i]);
        xo[b + 1] = (int)xall.size();
        smax = std::max(smax, xo[b + 1] - xo[b]);
        nbmax = std::max(nbmax, bo[b + 1] - bo[b]);
    }
    // ---- persistent buffers ------------------------------------------------
    void *p0;
    size_t need0 = sizeof(int) * (xall.size() + n + 64) + sizeof(double) * 4 * (ncbf + ntr + 64) + 4096;
    MIDAS_TRY(ensure(c, S_CBF0, need0, &p0));
    Buf b0{c, 0, (char *)p0};
    int *d_xall = b0.take<int>(xall.size());
    int *d_all = b0.take<int>(n);
    double *d_cth = b0.take<double>(ncbf), *d_cph = b0.take<double>(ncbf);
    double *d_th = b0.take<double>(ntr), *d_ph = b0.take<double>(ntr);
    MIDAS_CUDA(c, cudaMemcpyAsync(d_xall, xall.data(), sizeof(int) * xall.size(), cudaMemcpyHostToDevice, c->stream));
    MIDAS_CUDA(c, cudaMemcpyAsync(d_cth, cbf_theta, sizeof(double) * ncbf, cudaMemcpyDefault, c->stream));
    MIDAS_CUDA(c, cudaMemcpyAsync(d_cph, cbf_phi, sizeof(double) * ncbf, cudaMemcpyDefault, c->stream));
    MIDAS_CUDA(c, cudaMemcpyAsync(d_th, theta, sizeof(double) * ntr, cudaMemcpyDefault, c->stream));
    MIDAS_CUDA(c, cudaMemcpyAsync(d_ph, phi, sizeof(double) * ntr, cudaMemcpyDefault, c->stream));
    ++c->launches;
    k_iota<<<(n + 255) / 256, 256, 0, c->stream>>>(d_all, n, 0);
    // CBF storage: block b's C_b (3 n_b x K_b, column-major) at coff[b], with room for K_b = m
    void *pC;
    MIDAS_TRY(ensure(c, S_CBF5, sizeof(double2) * (size_t)3 * n * m, &pC));
    double2 *Call = (double2 *)pC;
    std::vector<size_t> coff(nb + 1, 0);
    for (int b = 0; b < nb; ++b) coff[b + 1] = coff[b] + (size_t)3 * (bo[b + 1] - bo[b]) * m;
    std::vector<int> Kb(nb, 0);
    // FP64 block solutions of every block are kept for the eigen-solves
    void *p3, *p4;
    std::vector<size_t> xoff(nb + 1, 0);
    for (int b = 0; b < nb; ++b) xoff[b + 1] = xoff[b] + (size_t)pad64(3 * (xo[b + 1] - xo[b])) * m;
    MIDAS_TRY(ensure(c, S_CBF3, sizeof(double2) * xoff[nb] + 4096, &p3));
    MIDAS_TRY(ensure(c, S_CBF4, (sizeof(double2) * (size_t)3 * m * m + sizeof(double) * m) * nb + 4096, &p4));
    double2 *Xall = (double2 *)p3;
    Buf b4{c, 0, (char *)p4};
    const size_t mm = (size_t)m * m;
    double2 *Gall = b4.take<double2>(mm * nb), *Vall = b4.take<double2>(mm * nb), *Hall = b4.take<double2>(mm * nb);
    double *Wall = b4.take<double>((size_t)m * nb);
    std::vector<int> srefine(nb, 0);
    const double cbf_tol = (flags & MIDAS_CBFM_FAST_CBF) ? 1e-7 : 1e-11;
    // Reduced assembly T = Z C (3n rows, complex as float pairs): block j's columns start
    // at column j m, since K_j is known only after block j's eigen-solve; the gaps are
    // zero.  Zc = C^T T takes the same padded columns, its rows are compact.
    const int ncolp = nb * m;
    const long long ldT = 2LL * ncolp;   // floats per row of T and Zc
    void *pt;
    MIDAS_TRY(ensure(c, S_CBF7, sizeof(float) * (size_t)3 * n * ldT + sizeof(float) * (size_t)ncolp * ldT +
                                    sizeof(int) * (size_t)ncolp + 256, &pt));
    float *T = (float *)pt, *Zcf = T + (size_t)3 * n * ldT;
    int *d_colmap = (int *)(Zcf + (size_t)ncolp * ldT);
    // With the lattice-table fill the products Z C_j take fp16 operand pieces (kind::f16:
    // twice the rate and half the bytes of TF32), scaled by a power of two from a bound
    // of every entry; otherwise TF32 pieces.
    double zbound = 0.0;
    MIDAS_TRY(fill4_bound(c, &zbound));
    const bool h16 = zbound > 0.0;
    // an FFT reduced residual corrects alpha after the reduced solve (lattice cells, no ACA)
    const bool fft_correction = !use_aca && lattice_fft_fits(c);
    const float hsA = h16 ? ldexpf(1.f, 12 - (int)std::ceil(std::log2(zbound))) : 1.f;
    // ACA of every off-diagonal pair (i, j), pair index i * (nb - 1) + (j < i ? j : j - 1)
    const int npairs = use_aca ? nb * (nb - 1) : 0;
    std::vector<int> rank(npairs, 0);
    std::vector<AcaPair> pairs(npairs);
    double2 *Uaca = nullptr, *Vaca = nullptr, *Waca = nullptr;
    auto pidx = [&](int i, int j) { return i * (nb - 1) + (j < i ? j : j - 1); };
    int n_far = 0;
    auto dense = [&](int i, int j) { return i == j || !use_aca || std::min(rank[pidx(i, j)], aca_itmax) >= aca_itmax; };

    // K_b = #{k : sigma_k / sigma_1 >= Threshold_CBFM} from the eigenvalues of block b's
    // Gram matrix (hW: host copy), then C_b = X_b[0:3 n_b, :] V_K Sigma_K^-1 and the zero
    // gap of block b's columns in T, on X's stream
    auto finish_block = [&](midas_gpu_ctx *X, int b, const double *hW) -> int {
        const int s = xo[b + 1] - xo[b], nbc = bo[b + 1] - bo[b];
        const int N3 = 3 * s, sp = pad64(N3);
        double2 *Vv = Vall + mm * b;
        const double s1 = sqrt(std::max(hW[0], 0.0));
        if (c->opts.verbose >= 2) {
            fprintf(stderr, "[midas] cbf block %d: s=%d refine=%d sigma/sigma1:", b, s, srefine[b]);
            for (int k = 0; k < std::min(N3, m); ++k) fprintf(stderr, " %.6e", sqrt(std::max(hW[k], 0.0)) / s1);
            fprintf(stderr, "\n");
        }
        int K = 0;
        for (int k = 0; k < std::min(N3, m); ++k) {
            const double sk = sqrt(std::max(hW[k], 0.0));
            if (s1 > 0 && sk / s1 >= thr_cbf) K++;
        }
        if (K == 0) return X->err.set(MIDAS_ERR_SINGULAR, "cbf: no singular value above the threshold");
        Kb[b] = K;
        ++X->launches;
        k_scale_cols<<<(m * K + 255) / 256, 256, 0, X->stream>>>(m, K, Vv, Wall + (size_t)m * b);
        MIDAS_TRY(zgemm_df(X, 3 * nbc, K, m, Xall + xoff[b], 1, sp, Vv, m, 1, Call + coff[b], 1, 3 * nbc));
        if (K < m)
            MIDAS_CUDA(X, cudaMemset2DAsync(T + 2LL * ((long long)b * m + K), sizeof(float) * ldT, 0,
                                            sizeof(float2) * (m - K), (size_t)3 * n, X->stream));
        return MIDAS_OK;
    };
    // block j's columns of T = Z C: the dense row runs as split products of the filled
    // rows with C_j (the fill writes the split A operand directly), the low-rank pairs
    // as U (V C_j) in FP64; on X's stream
    auto assemble_column = [&](midas_gpu_ctx *X, int j) -> int {
        const int nj = bo[j + 1] - bo[j];
        const double2 *Cj = Call + coff[j];
        const long long tc = 2LL * j * m;   // first float of block j's columns in a row of T
        for (int i = 0; i < nb;) {
            if (!dense(i, j)) { ++i; continue; }
            int i1 = i;
            while (i1 < nb && dense(i1, j)) ++i1;
            const int r0 = bo[i], nr = bo[i1] - bo[i];
            void *pa;
            if (h16) {
                const long long K6h = h16_arow(3LL * nj);
                MIDAS_TRY(ensure(X, S_CBF8, sizeof(__half) * (size_t)3 * nr * K6h + 256, &pa));
                __half *A3h = (__half *)pa;
                float *sc = (float *)(A3h + (size_t)3 * nr * K6h);
                MIDAS_TRY(launch_block_fill4_a3(X, nr, d_all + r0, nj, d_all + bo[j], nullptr, K6h, A3h, hsA));
                MIDAS_TRY(set_h16_scale(X, sc, hsA));
                MIDAS_TRY(zgemm_x3h_a3<double2>(X, 3 * nr, Kb[j], 3 * nj, A3h, K6h, sc, Cj, 1, 3LL * nj,
                                                T + (size_t)3 * r0 * ldT + tc, ldT, MIDAS_KC_GEMM_PROD,
                                                fft_correction ? 4 : 2));
            } else {
                const long long K6 = (6LL * 3 * nj + 3) / 4 * 4;
                MIDAS_TRY(ensure(X, S_CBF8, sizeof(float) * (size_t)3 * nr * K6, &pa));
                MIDAS_TRY(launch_block_fill4_a3(X, nr, d_all + r0, nj, d_all + bo[j], (float *)pa, K6));
                MIDAS_TRY(zgemm_x3_a3<double2>(X, 3 * nr, Kb[j], 3 * nj, (const float *)pa, K6, Cj, 1, 3LL * nj,
                                               T + (size_t)3 * r0 * ldT + tc, ldT, 1.f, 0.f));
            }
            i = i1;
        }
        for (int i = 0; i < nb && use_aca; ++i) {
            if (dense(i, j)) continue;
            const AcaPair &p = pairs[pidx(i, j)];
            const int k = rank[pidx(i, j)];
            MIDAS_TRY(zgemm64(X, k, Kb[j], 3 * nj, Vaca + p.voff, 3LL * nj, 1, 0, Cj, 1, 3LL * nj, Waca, Kb[j], 1,
                              make_double2(1, 0), make_double2(0, 0)));
            MIDAS_TRY(aca_uw(X, 3 * p.ni, k, Kb[j], Uaca + p.uoff, Waca,
                             (float2 *)T + (size_t)3 * bo[i] * ncolp + (size_t)j * m, ncolp));
        }
        return MIDAS_OK;
    };

    cudaEvent_t e0, e1, e2, e3;
    cudaEventCreate(&e0); cudaEventCreate(&e1); cudaEventCreate(&e2); cudaEventCreate(&e3);
    cudaEventRecord(e0, c->stream);
    int ir_max = 0;
    CbfShared S{bo.data(), xo.data(), d_xall, d_cth, d_cph, ncbf, m, sr, homog, res_sr, cbf_tol, Xall,
                xoff.data(), Gall, mm, srefine.data(), (flags & MIDAS_CBFM_SPHERICAL) != 0};
    // Streamed (the default): as each lane finishes a block, the block's eigen-solve (one
    // CTA, ~50 ms of serial FP64 work at m = 182) starts on the lane's eigen-solve stream,
    // and a finisher thread then builds C_b and block b's columns of T on its own stream,
    // so the eigen-solves run under the CBF generation and the reduced assembly.  With ACA
    // (the pair ranks come first) or per-class kernel timing (one stream at a time) the
    // steps run in sequence.
    const bool streamed = !use_aca && !c->kprof.on && nb > 1 && std::min(nb, cbf_lanes()) > 1;
    cudaEvent_t e_lanes = nullptr;
    if (c->opts.verbose >= 1) {
        cudaEventCreate(&e_lanes);
    }
    if (streamed) {
        const int nl = std::min(nb, cbf_lanes());
        constexpr int NF = CBF_FINISHERS;
        const int na = NF + nl;
        MIDAS_TRY(get_aux(c, na));
        midas_gpu_ctx *F = c->aux[0];   // the finisher thread's error state
        for (int a = 0; a < na; ++a) {
            lane_sync_cells(c->aux[a], c);
            c->aux[a]->allow_side = false;
        }
        std::vector<long long> a0(na);
        for (int a = 0; a < na; ++a) a0[a] = c->aux[a]->launches;
        std::vector<int> fidx(nb, 0);   // the finisher stream of block b (C_b and its column)
        double *hW = nullptr;
        MIDAS_CUDA(c, cudaMallocHost(&hW, sizeof(double) * (size_t)m * nb));
        std::vector<cudaEvent_t> ev_gram(nb), ev_eig(nb);
        for (int b = 0; b < nb; ++b) {
            cudaEventCreateWithFlags(&ev_gram[b], cudaEventDisableTiming);
            cudaEventCreateWithFlags(&ev_eig[b], cudaEventDisableTiming);
        }
        std::mutex qm;
        std::condition_variable qcv;
        std::deque<int> q;
        bool lanes_over = false;
        // the columns of T start once a lane has drained (no block left for it): the tail
        // of the CBF generation then shares the GPU with them (measured over 12 steps:
        // 1013 ms waiting for every lane, 1000 ms from the first drained lane)
        std::atomic<int> lanes_idle{0};
        std::function<int(midas_gpu_ctx *, int, int)> on_done = [&](midas_gpu_ctx *L, int l, int b) -> int {
            midas_gpu_ctx *E = c->aux[NF + l];
            int st = [&]() -> int {
                MIDAS_CUDA(L, cudaEventRecord(ev_gram[b], L->stream));
                MIDAS_CUDA(E, cudaStreamWaitEvent(E->stream, ev_gram[b], 0));
                MIDAS_TRY(heev_dev(E, 1, m, Gall + mm * b, m, (long long)mm, Hall + mm * b, Vall + mm * b,
                                   (long long)mm, Wall + (size_t)m * b));
                MIDAS_CUDA(E, cudaMemcpyAsync(hW + (size_t)m * b, Wall + (size_t)m * b, sizeof(double) * m,
                                              cudaMemcpyDeviceToHost, E->stream));
                MIDAS_CUDA(E, cudaEventRecord(ev_eig[b], E->stream));
                return MIDAS_OK;
            }();
            if (st != MIDAS_OK) {
                if (L->err.msg.empty()) L->err = E->err;
                return st;
            }
            {
                std::lock_guard<std::mutex> g(qm);
                q.push_back(b);
            }
            qcv.notify_one();
            return MIDAS_OK;
        };
        // The finisher builds C_b as each eigen-solve ends (small products); the columns of
        // T (full-GPU fills and products) wait for the tail of the lanes, whose
        // latency-bound chains they would otherwise hold up (started with the first block
        // they made the CBF generation 30 % slower), and then run under the eigen-solves
        // still in flight.
        int fst = MIDAS_OK;
        // verbose: device times of the finisher's steps ('C' C_b built, 'T' column of T done)
        std::vector<std::pair<int, cudaEvent_t>> fin_ev;
        auto fin_mark = [&](midas_gpu_ctx *X, int tag) {
            if (c->opts.verbose < 1) return;
            cudaEvent_t ev;
            cudaEventCreate(&ev);
            cudaEventRecord(ev, X->stream);
            fin_ev.push_back({tag, ev});
        };
        std::thread fin([&]() {
            cudaSetDevice(F->device);
            std::vector<int> ready;
            int nfin = 0;
            auto over = [&] {
                if (lanes_idle.load() > 0) return true;
                std::lock_guard<std::mutex> g(qm);
                return lanes_over;
            };
            auto flush = [&] {
                for (int j : ready) {
                    midas_gpu_ctx *X = c->aux[fidx[j]];
                    if (fst == MIDAS_OK) {
                        fst = assemble_column(X, j);
                        if (fst != MIDAS_OK && X != F) F->err = X->err;
                    }
                    fin_mark(X, 1000 + j);
                }
                ready.clear();
            };
            for (int done = 0; done < nb; ++done) {
                int b = -1;
                for (;;) {
                    {
                        std::unique_lock<std::mutex> g(qm);
                        qcv.wait_for(g, std::chrono::microseconds(200), [&] { return !q.empty() || lanes_over; });
                        if (!q.empty()) {
                            b = q.front();
                            q.pop_front();
                            break;
                        }
                        if (lanes_over) break;
                    }
                    if (!ready.empty() && over()) flush();
                }
                if (b < 0) return;   // a lane failed: the remaining blocks never come
                if (fst != MIDAS_OK) continue;
                // wait for block b's eigen-solve, launching the ready columns once the lanes end
                bool bad = false;
                for (;;) {
                    const cudaError_t r = cudaEventQuery(ev_eig[b]);
                    if (r == cudaSuccess) break;
                    if (r != cudaErrorNotReady) { bad = true; break; }
                    if (!ready.empty() && over()) flush();
                    std::this_thread::sleep_for(std::chrono::microseconds(100));
                }
                if (bad) {
                    fst = F->err.set(MIDAS_ERR_CUDA, "cbf eigen-solve: stream failed");
                    continue;
                }
                fidx[b] = nfin++ % NF;
                midas_gpu_ctx *X = c->aux[fidx[b]];
                fst = finish_block(X, b, hW + (size_t)m * b);
                if (fst != MIDAS_OK && X != F) F->err = X->err;
                fin_mark(X, b);
                ready.push_back(b);
                if (over()) flush();
            }
            flush();
        });
        int st = cbf_generate(c, nb, S, &on_done, &lanes_idle);
        if (e_lanes) cudaEventRecord(e_lanes, c->stream);
        {
            std::lock_guard<std::mutex> g(qm);
            lanes_over = true;
        }
        qcv.notify_one();
        fin.join();
        for (int a = 0; a < NF; ++a) {
            cudaEvent_t ef;
            cudaEventCreateWithFlags(&ef, cudaEventDisableTiming);
            cudaEventRecord(ef, c->aux[a]->stream);
            cudaStreamWaitEvent(c->stream, ef, 0);
            cudaEventDestroy(ef);
        }
        for (int a = NF; a < na; ++a) cudaStreamSynchronize(c->aux[a]->stream);
        if (!fin_ev.empty()) {
            for (int a = 0; a < NF; ++a) cudaStreamSynchronize(c->aux[a]->stream);
            fprintf(stderr, "[midas] cbf finisher (C:block / T:block @ ms):");
            for (auto &fe : fin_ev) {
                float t = 0;
                cudaEventElapsedTime(&t, e0, fe.second);
                fprintf(stderr, " %c%d@%.0f", fe.first >= 1000 ? 'T' : 'C', fe.first % 1000, t);
                cudaEventDestroy(fe.second);
            }
            fprintf(stderr, "\n");
        }
        for (int b = 0; b < nb; ++b) {
            cudaEventDestroy(ev_gram[b]);
            cudaEventDestroy(ev_eig[b]);
        }
        cudaFreeHost(hW);
        for (int a = 0; a < na; ++a) c->launches += c->aux[a]->launches - a0[a];
        MIDAS_TRY(st);
        if (fst != MIDAS_OK) return c->err.set(fst, F->err.msg);
        for (int a = 0; a < na; ++a) {
            const int fs = check_flag(c->aux[a], a >= NF ? "cbf eigen-solve" : "cbf reduced assembly");
            if (fs != MIDAS_OK) return c->err.set(fs, c->aux[a]->err.msg);
        }
        for (int b = 0; b < nb; ++b) ir_max = std::max(ir_max, srefine[b]);
        cudaEventRecord(e1, c->stream);
    } else {
        // ---- 1. CBF generation: blocks run concurrently on the lanes ----------------
        MIDAS_TRY(cbf_generate(c, nb, S));
        if (e_lanes) cudaEventRecord(e_lanes, c->stream);
        for (int b = 0; b < nb; ++b) ir_max = std::max(ir_max, srefine[b]);
        // eigen-decomposition of every block's Gram matrix in one launch (one CTA per block)
        MIDAS_TRY(heev_dev(c, nb, m, Gall, m, (long long)mm, Hall, Vall, (long long)mm, Wall));
        std::vector<double> hWall((size_t)m * nb);
        MIDAS_CUDA(c, cudaMemcpyAsync(hWall.data(), Wall, sizeof(double) * m * nb, cudaMemcpyDeviceToHost, c->stream));
        MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
        MIDAS_TRY(check_flag(c, "cbf eigen-solve"));
        for (int b = 0; b < nb; ++b) MIDAS_TRY(finish_block(c, b, hWall.data() + (size_t)m * b));
        cudaEventRecord(e1, c->stream);
        // ---- 2. reduced matrix Zc = C^T Z C ----------------------------------------
        if (use_aca) {
            long long uo = 0, vo = 0;
            for (int i = 0; i < nb; ++i)
                for (int j = 0; j < nb; ++j) {
                    if (i == j) continue;
                    AcaPair &p = pairs[pidx(i, j)];
                    p.r0 = bo[i]; p.ni = bo[i + 1] - bo[i]; p.c0 = bo[j]; p.nj = bo[j + 1] - bo[j];
                    p.uoff = uo; p.voff = vo;
                    uo += 3LL * p.ni * aca_itmax;
                    vo += 3LL * p.nj * aca_itmax;
                }
            const size_t need = sizeof(double2) * (size_t)(uo + vo + (size_t)aca_itmax * m) +
                                sizeof(AcaPair) * npairs + sizeof(int) * npairs + 5 * 256;
            void *pa;
            MIDAS_TRY(ensure(c, S_ACA, need, &pa));
            Buf ba{c, 0, (char *)pa};
            Uaca = ba.take<double2>(uo);
            Vaca = ba.take<double2>(vo);
            Waca = ba.take<double2>((size_t)aca_itmax * m);
            AcaPair *d_pairs = ba.take<AcaPair>(npairs);
            int *d_rank = ba.take<int>(npairs);
            MIDAS_CUDA(c, cudaMemcpyAsync(d_pairs, pairs.data(), sizeof(AcaPair) * npairs, cudaMemcpyHostToDevice,
                                          c->stream));
            MIDAS_TRY(aca_batch(c, npairs, d_pairs, eps_aca, aca_itmax, Uaca, Vaca, d_rank));
            MIDAS_CUDA(c, cudaMemcpyAsync(rank.data(), d_rank, sizeof(int) * npairs, cudaMemcpyDeviceToHost, c->stream));
            MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
            for (int p = 0; p < npairs; ++p) n_far += std::min(rank[p], aca_itmax) < aca_itmax;
            if (c->opts.verbose >= 1) fprintf(stderr, "[midas] aca: %d of %d pairs low-rank\n", n_far, npairs);
        }
        for (int j = 0; j < nb; ++j) MIDAS_TRY(assemble_column(c, j));
    }
    std::vector<int> koff(nb + 1, 0);
    for (int b = 0; b < nb; ++b) koff[b + 1] = koff[b] + Kb[b];
    const int Kt = koff[nb];
    {
        std::vector<int> colmap(Kt);
        for (int b = 0; b < nb; ++b)
            for (int k = 0; k < Kb[b]; ++k) colmap[koff[b] + k] = b * m + k;
        MIDAS_CUDA(c, cudaMemcpyAsync(d_colmap, colmap.data(), sizeof(int) * Kt, cudaMemcpyHostToDevice, c->stream));
    }
    // Zc rows of block i = C_i^T T_i, FP32-grade split products.  With the lattice-table
    // fill (the FFT reduced residual below then corrects alpha) on fp16 pieces, each
    // operand scaled by a power of two from its largest entry; otherwise on TF32 pieces,
    // whose exponent range keeps the small entries of T (far pairs, ACA terms) at full
    // relative precision (fp16 pieces moved C_abs of the ACA trimer by 1.5e-6).
    for (int i = 0; i < nb; ++i) {
        const int ni = bo[i + 1] - bo[i];
        const double2 *Ci = Call + coff[i];
        const float2 *Ti = (const float2 *)(T + (size_t)3 * bo[i] * ldT);
        if (h16 && fft_correction)
            MIDAS_TRY(zgemm_x3h<double2, float2>(c, Kb[i], ncolp, 3 * ni, Ci, 3 * ni, 1, Ti, ncolp, 1,
                                                 Zcf + (size_t)koff[i] * ldT, ldT, MIDAS_KC_GEMM_PROD, 4));
        else
            MIDAS_TRY(zgemm_x3<double2, float2>(c, Kb[i], ncolp, 3 * ni, Ci, 3 * ni, 1, 0, Ti, ncolp, 1,
                                                Zcf + (size_t)koff[i] * ldT, ldT, 1.f, 0.f));
    }
    cudaEventRecord(e2, c->stream);
    // ---- 3. Vc, reduced solve, E -----------------------------------------------
    const int npd = pad64(Kt), nr = 2 * ntr;
    void *p64, *p32, *pb, *px, *pe;
    MIDAS_TRY(ensure(c, S_Z64, sizeof(double2) * (size_t)npd * npd, &p64));
    MIDAS_TRY(ensure(c, S_Z32, sizeof(float2) * (size_t)npd * npd, &p32));
    MIDAS_TRY(ensure(c, S_RHS64, sizeof(double2) * (size_t)npd * nr, &pb));
    MIDAS_TRY(ensure(c, S_X64, sizeof(double2) * (size_t)npd * nr, &px));
    MIDAS_TRY(ensure(c, S_EINC, sizeof(double2) * (size_t)3 * n * nr, &pe));
    {
        long long tot = (long long)npd * npd;
        ++c->launches;
        k_zc_to_sys<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(Kt, Zcf, ldT, d_colmap, (double2 *)p64,
                                                                          (float2 *)p32, npd);
    }
    double2 *Vc = (double2 *)pb, *Einc = (double2 *)pe;
    MIDAS_CUDA(c, cudaMemsetAsync(Vc, 0, sizeof(double2) * (size_t)npd * nr, c->stream));
    // the incident fields on every cell (column-major 3n x nr)
    MIDAS_TRY(launch_incident4<double2>(c, n, d_all, ntr, d_th, d_ph, Einc, 1, (size_t)3 * n));
    // reduced right-hand sides and residuals: rows koff_b of V = C_b^T F_b for every block,
    // one batched launch (F column-major 3n x nr)
    auto project = [&](const double2 *Fv, double2 *V) -> int {
        std::vector<ZdfJob> jobs;
        for (int b = 0; b < nb; ++b) {
            const int nbc = bo[b + 1] - bo[b];
            ZdfJob J{};
            J.M = Kb[b]; J.N = nr; J.K = 3 * nbc;
            J.A = Call + coff[b]; J.ars = 3 * nbc; J.acs = 1;
            J.B = Fv + 3 * (size_t)bo[b]; J.brs = 1; J.bcs = 3LL * n;
            J.C = V + koff[b]; J.crs = 1; J.ccs = npd;
            jobs.push_back(J);
        }
        return zgemm_df_batched(c, jobs);
    };
    MIDAS_TRY(project(Einc, Vc));
    midas_gpu_info sinfo;
    memset(&sinfo, 0, sizeof(sinfo));
    DenseLU rlu;
    MIDAS_TRY(mixed_solve(c, npd, (float2 *)p32, (double2 *)p64, Vc, (double2 *)px, nr, &sinfo, &rlu));
    // E = C alpha per block
    double2 *Eout = E_user;
    void *peo = nullptr;
    bool host_out = !is_device_ptr(E_user);
    if (host_out) {
        MIDAS_TRY(ensure(c, S_OUT0, sizeof(double2) * (size_t)3 * n * nr, &peo));
        Eout = (double2 *)peo;
    }
    auto reconstruct = [&]() -> int {
        std::vector<ZdfJob> jobs;
        for (int b = 0; b < nb; ++b) {
            const int nbc = bo[b + 1] - bo[b];
            ZdfJob J{};
            J.M = 3 * nbc; J.N = nr; J.K = Kb[b];
            J.A = Call + coff[b]; J.ars = 1; J.acs = 3 * nbc;
            J.B = (const double2 *)px + koff[b]; J.brs = 1; J.bcs = npd;
            J.C = Eout + 3 * (size_t)bo[b]; J.crs = 1; J.ccs = 3LL * n;
            jobs.push_back(J);
        }
        return zgemm_df_batched(c, jobs);
    };
    MIDAS_TRY(reconstruct());
    // One correction against the FP64 reduced residual.  The reduced matrix above
    // is FP32-grade (split-TF32 tensor products summed in FP32), which moves alpha
    // by ~1e-6 on a 27-block scene.  For lattice cells the exact reduced residual
    //   rho_b = C_b^T (Einc - Z E)_b,  E = C alpha,
    // costs one FFT product with the complex(4) dyads of Green_s_tr_partial (their
    // products with f_kapChe and E in FP64); alpha += Zc^-1 rho with the TF32
    // factors then leaves ~1e-3.5 of the error.  With ACA the reduced matrix is
    // itself an approximation of these blocks, so no correction is made.
    if (fft_correction) {
        const size_t nf = (size_t)3 * n * nr;
        void *pf;
        MIDAS_TRY(ensure(c, S_CREF, sizeof(double2) * nf + sizeof(float2) * (size_t)npd * nr + 1024, &pf));
        double2 *Rf = (double2 *)pf;
        float2 *d32 = (float2 *)(((uintptr_t)(Rf + nf) + 255) & ~(uintptr_t)255);
        MIDAS_TRY(lattice_matvec(c, nr, Eout, 3LL * n, Einc, 3LL * n, Rf, 3LL * n, S_LFFT, true));
        double2 *rho = Vc;   // Vc is no longer needed: the reduced residual takes its place
        MIDAS_CUDA(c, cudaMemsetAsync(rho, 0, sizeof(double2) * (size_t)npd * nr, c->stream));
        MIDAS_TRY(project(Rf, rho));
        const long long tot = (long long)npd * nr;
        ++c->launches;
        k_c64_to_c32<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(tot, rho, d32);
        MIDAS_TRY(lu_solve(c, rlu, d32, nr));
        ++c->launches;
        k_add_c32<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(tot, d32, (double2 *)px);
        MIDAS_CUDA(c, cudaGetLastError());
        MIDAS_TRY(reconstruct());
    }
    cudaEventRecord(e3, c->stream);
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    MIDAS_TRY(check_flag(c, "cbfm"));
    if (host_out) MIDAS_CUDA(c, cudaMemcpy(E_user, Eout, sizeof(double2) * (size_t)3 * n * nr, cudaMemcpyDeviceToHost));
    if (K_user) MIDAS_CUDA(c, cudaMemcpy(K_user, Kb.data(), sizeof(int) * nb, cudaMemcpyDefault));
    float t01, t12, t23;
    cudaEventElapsedTime(&t01, e0, e1);
    cudaEventElapsedTime(&t12, e1, e2);
    cudaEventElapsedTime(&t23, e2, e3);
    if (e_lanes) {
        float tl = 0;
        cudaEventElapsedTime(&tl, e0, e_lanes);
        fprintf(stderr, "[midas] cbfm step (%s): lanes end %.1f, CBFs end %.1f, assembly end %.1f, solve end %.1f ms\n",
                streamed ? "streamed" : "in sequence", tl, t01, t01 + t12, t01 + t12 + t23);
        cudaEventDestroy(e_lanes);
    }
    cudaEventDestroy(e0); cudaEventDestroy(e1); cudaEventDestroy(e2); cudaEventDestroy(e3);
    if (info) {
        info->status = MIDAS_OK;
        info->k_total = Kt;
        info->n_far_aca = n_far;
        info->ir_iters = sinfo.ir_iters;
        info->backward_error = sinfo.backward_error;
        info->anorm = sinfo.anorm;
        // streamed, the CBF generation phase also holds the eigen-solves and T = Z C, and
        // the assembly phase only the products C_i^T T_i
        info->t_fill_ms = t12;    // reduced-matrix assembly (fills + GEMMs)
        info->t_factor_ms = t01;  // CBF generation (block fills, LUs, refinement, SVDs)
        info->t_solve_ms = t23;   // Vc, reduced solve, E
        info->t_total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tw0).count();
    }
    (void)ir_max;
    return MIDAS_OK;
}


}  // namespace midas
