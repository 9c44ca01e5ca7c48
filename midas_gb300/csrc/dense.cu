// dense.cu -- dense complex solves for the MIDAS hot path (sm_103a).
//
// Replaces PZGESV / PZLANGE / PZGECON (src/Compute_EFields_MoM.f90:153-198,
// src/Compute_EFields_CBFME.f90:895-943) and the dense gesvx of the CBF block
// solves (src/Compute_EFields_CBFME.f90:402-407).
//
// Mixed precision: a right-looking blocked LU *without pivoting* in complex64
// whose panel solves and trailing updates are tensor-core GEMMs (gemm_tf32 with
// the real embedding), followed by iterative refinement with an FP64 residual
// b - Z x (Z kept in FP64).  The VIE matrices I - G diag(kappa chi) are
// diagonally dominant in practice (pivot growth ~1); a pivot below
// 1e-30 ||Z|| raises MIDAS_ERR_SINGULAR, and refinement that does not reach the
// tolerance returns MIDAS_ERR_NOT_CONVERGED -- no silent fallback.
//
// Data layout in HBM: the factor matrix is row-major complex64 (row i of Z is
// contiguous), so the L21 panel is a K-major TMA operand in place; the inverses
// of the nb x nb diagonal blocks (unit-lower L^-1, upper U^-1) are kept for the
// blocked triangular solves.
#include <cusolverDn.h>
#include <cmath>

#include "common.cuh"
#include "kernels.cuh"

namespace midas {

// ---------------------------------------------------------------------------
// diagonal block: unblocked LU of A11 (nb x nb, row-major, lda) in shared
// memory, then L11^-1 and U11^-1 by substitution.  One CTA, 512 threads.
// Writes L\U back to A11, Linv/Uinv to their slots, and the expanded U11^-1
// (the Bt operand of L21 = A21 U11^-1) to UinvExp (2nb x 2nb floats).
// ---------------------------------------------------------------------------
template <int NB>
__global__ void __launch_bounds__(512) k_diag_lu(float2 *A11, long long lda, float2 *Linv, float2 *Uinv,
                                                  float *UinvExp, float tiny, int *flag)
{
    extern __shared__ float2 sm[];
    float2 *a = sm;                 // NB x NB
    float2 *li = sm + NB * NB;      // NB x NB
    float2 *ui = li + NB * NB;      // NB x NB
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int i = tid; i < NB * NB; i += nt) a[i] = A11[(long long)(i / NB) * lda + (i % NB)];
    __syncthreads();
    // right-looking elimination without pivoting
    for (int j = 0; j < NB; ++j) {
        float2 piv = a[j * NB + j];
        float pm = piv.x * piv.x + piv.y * piv.y;
        if (tid == 0 && !(pm > tiny * tiny)) atomicOr(flag, DEV_ZERO_PIVOT);
        float2 ip = make_float2(piv.x / pm, -piv.y / pm);
        for (int i = j + 1 + tid; i < NB; i += nt) {
            float2 v = a[i * NB + j];
            a[i * NB + j] = make_float2(v.x * ip.x - v.y * ip.y, v.x * ip.y + v.y * ip.x);
        }
        __syncthreads();
        int m = NB - j - 1;
        for (int t = tid; t < m * m; t += nt) {
            int i = j + 1 + t / m, cc = j + 1 + t % m;
            float2 l = a[i * NB + j], u = a[j * NB + cc], d = a[i * NB + cc];
            a[i * NB + cc] = make_float2(d.x - (l.x * u.x - l.y * u.y), d.y - (l.x * u.y + l.y * u.x));
        }
        __syncthreads();
    }
    // L^-1 (unit lower): row i of X: X[i][c] = -sum_{m=c}^{i-1} L[i][m] X[m][c], X[c][c] = 1
    for (int t = tid; t < NB * NB; t += nt) li[t] = make_float2((t / NB == t % NB) ? 1.f : 0.f, 0.f);
    __syncthreads();
    for (int i = 1; i < NB; ++i) {
        for (int cc = tid; cc < i; cc += nt) {
            float2 s = make_float2(0.f, 0.f);
            for (int m = cc; m < i; ++m) {
                float2 l = a[i * NB + m], x = li[m * NB + cc];
                s.x += l.x * x.x - l.y * x.y;
                s.y += l.x * x.y + l.y * x.x;
            }
            li[i * NB + cc] = make_float2(-s.x, -s.y);
        }
        __syncthreads();
    }
    // U^-1 (upper): row i from the bottom: X[i][c] = (delta_ic - sum_{m=i+1}^{c} U[i][m] X[m][c]) / U[i][i]
    for (int t = tid; t < NB * NB; t += nt) ui[t] = make_float2(0.f, 0.f);
    __syncthreads();
    for (int i = NB - 1; i >= 0; --i) {
        float2 d = a[i * NB + i];
        float dm = d.x * d.x + d.y * d.y;
        float2 id = make_float2(d.x / dm, -d.y / dm);
        for (int cc = i + tid; cc < NB; cc += nt) {
            float2 s = make_float2(cc == i ? 1.f : 0.f, 0.f);
            for (int m = i + 1; m <= cc; ++m) {
                float2 u = a[i * NB + m], x = ui[m * NB + cc];
                s.x -= u.x * x.x - u.y * x.y;
                s.y -= u.x * x.y + u.y * x.x;
            }
            ui[i * NB + cc] = make_float2(s.x * id.x - s.y * id.y, s.x * id.y + s.y * id.x);
        }
        __syncthreads();
    }
    for (int i = tid; i < NB * NB; i += nt) {
        A11[(long long)(i / NB) * lda + (i % NB)] = a[i];
        Linv[i] = li[i];
        Uinv[i] = ui[i];
    }
    // expanded U^-1 as the Bt operand (rows = output columns j, along p):
    // Bt[2j][2p] = Ur(p,j), Bt[2j][2p+1] = -Ui(p,j), Bt[2j+1][2p] = Ui, Bt[2j+1][2p+1] = Ur
    for (int t = tid; t < NB * NB; t += nt) {
        int p = t / NB, j = t % NB;
        float2 u = ui[p * NB + j];
        float *r0 = UinvExp + (long long)(2 * j) * (2 * NB) + 2 * p;
        float *r1 = r0 + 2 * NB;
        r0[0] = u.x; r0[1] = -u.y;
        r1[0] = u.y; r1[1] = u.x;
    }
}

constexpr int LU_NB = 64;

int lu_factor_nopiv(midas_gpu_ctx *c, DenseLU &lu)
{
    const int n = lu.n, nb = LU_NB;
    lu.nb = nb;
    lu.nblk = (n + nb - 1) / nb;
    if (n % nb != 0) return c->err.set(MIDAS_ERR_ARG, "lu_factor_nopiv: n must be a multiple of 64 (pad)");
    void *p;
    MIDAS_TRY(ensure(c, S_LINV, sizeof(float2) * (size_t)lu.nblk * nb * nb * 2, &p));
    lu.Linv = (float2 *)p;
    lu.Uinv = lu.Linv + (size_t)lu.nblk * nb * nb;
    MIDAS_TRY(ensure(c, S_BEXP, sizeof(float) * (size_t)(2 * nb) * (2 * nb), &p));
    float *uexp = (float *)p;
    MIDAS_TRY(ensure(c, S_BEXP2, sizeof(float) * (size_t)2 * n * 2 * nb, &p));
    float *bexp = (float *)p;
    const size_t smem = sizeof(float2) * 3 * nb * nb;
    static bool attr = false;
    if (!attr) {
        MIDAS_CUDA(c, cudaFuncSetAttribute(k_diag_lu<LU_NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr = true;
    }
    const long long lda = lu.lda;
    float *Af = (float *)lu.A;
    for (int k = 0; k < lu.nblk; ++k) {
        const int j0 = k * nb, rem = n - j0 - nb;
        float2 *A11 = lu.A + (long long)j0 * lda + j0;
        ++c->launches;
        int kp = kp_begin(c);
        k_diag_lu<LU_NB><<<1, 512, smem, c->stream>>>(A11, lda, lu.Linv + (size_t)k * nb * nb,
                                                      lu.Uinv + (size_t)k * nb * nb, uexp, 1e-30f, c->d_flag);
        kp_end(c, kp, MIDAS_KC_DIAG_LU, 8.0 * nb * nb * nb, 8.0 * nb * nb * 4);
        MIDAS_CUDA(c, cudaGetLastError());
        if (rem == 0) break;
        // L21 = A21 U11^-1 (in place: each output row tile reads only its own rows)
        {
            GemmArgs g{rem, 2 * nb, 2 * nb, Af + 2 * ((long long)(j0 + nb) * lda + j0), 2 * lda, uexp, 2 * nb,
                       Af + 2 * ((long long)(j0 + nb) * lda + j0), 2 * lda, 1.f, 0.f};
            MIDAS_TRY(gemm_tf32(c, g));
        }
        // U12 = L11^-1 A12 : Bt = expand(A12) (copy), then write U12 in place
        MIDAS_TRY(expand_b(c, nb, rem, lu.A + (long long)j0 * lda + j0 + nb, lda, 1, bexp, 2 * nb));
        {
            GemmArgs g{nb, 2 * rem, 2 * nb, (const float *)(lu.Linv + (size_t)k * nb * nb), 2 * nb, bexp, 2 * nb,
                       Af + 2 * ((long long)j0 * lda + j0 + nb), 2 * lda, 1.f, 0.f};
            MIDAS_TRY(gemm_tf32(c, g));
        }
        // A22 -= L21 U12
        MIDAS_TRY(expand_b(c, nb, rem, lu.A + (long long)j0 * lda + j0 + nb, lda, 1, bexp, 2 * nb));
        {
            GemmArgs g{rem, 2 * rem, 2 * nb, Af + 2 * ((long long)(j0 + nb) * lda + j0), 2 * lda, bexp, 2 * nb,
                       Af + 2 * ((long long)(j0 + nb) * lda + j0 + nb), 2 * lda, -1.f, 1.f};
            MIDAS_TRY(gemm_tf32(c, g));
        }
    }
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// blocked triangular solves on X (n x nrhs column-major complex64, ld = n)
// ---------------------------------------------------------------------------
// X[rows r0..r0+nb) = Minv (nb x nb row-major) * X[rows]  (nb <= 64, one CTA per rhs)
__global__ void k_apply_inv(const float2 *Minv, int nb, float2 *X, long long ldx, int r0)
{
    __shared__ float2 t[64];
    float2 *x = X + (long long)blockIdx.x * ldx + r0;
    int i = threadIdx.x;
    if (i < nb) t[i] = x[i];
    __syncthreads();
    if (i < nb) {
        float2 s = make_float2(0.f, 0.f);
        for (int m = 0; m < nb; ++m) {
            float2 a = Minv[i * nb + m], v = t[m];
            s.x += a.x * v.x - a.y * v.y;
            s.y += a.x * v.y + a.y * v.x;
        }
        x[i] = s;
    }
}

// X[rows ra..ra+na) -= A[rows ra.., cols cb..cb+nb) * X[rows cb..cb+nb)  (warp per row)
__global__ void k_gemv_update(const float2 *A, long long lda, int ra, int na, int cb, int nb, float2 *X,
                              long long ldx, int nrhs)
{
    int w = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x % 32;
    if (w >= na) return;
    const float2 *row = A + (long long)(ra + w) * lda + cb;
    for (int r = 0; r < nrhs; ++r) {
        const float2 *xv = X + (long long)r * ldx + cb;
        float sx = 0.f, sy = 0.f;
        for (int m = lane; m < nb; m += 32) {
            float2 a = row[m], v = xv[m];
            sx += a.x * v.x - a.y * v.y;
            sy += a.x * v.y + a.y * v.x;
        }
        for (int o = 16; o > 0; o >>= 1) {
            sx += __shfl_down_sync(0xffffffffu, sx, o);
            sy += __shfl_down_sync(0xffffffffu, sy, o);
        }
        if (lane == 0) {
            float2 *d = X + (long long)r * ldx + ra + w;
            d->x -= sx;
            d->y -= sy;
        }
    }
}

int lu_solve(midas_gpu_ctx *c, const DenseLU &lu, float2 *R, int nrhs)
{
    const int n = lu.n, nb = lu.nb;
    // forward: L y = b  (right-looking: solve block k, then update the rows below)
    for (int k = 0; k < lu.nblk; ++k) {
        int r0 = k * nb;
        ++c->launches;
        int kp = kp_begin(c);
        k_apply_inv<<<nrhs, 64, 0, c->stream>>>(lu.Linv + (size_t)k * nb * nb, nb, R, n, r0);
        kp_end(c, kp, MIDAS_KC_TRSV, 8.0 * nb * nb * nrhs, 8.0 * nb * nb + 16.0 * nb * nrhs);
        int na = n - r0 - nb;
        if (na > 0) {
            ++c->launches;
            kp = kp_begin(c);
            k_gemv_update<<<(na * 32 + 255) / 256, 256, 0, c->stream>>>(lu.A, lu.lda, r0 + nb, na, r0, nb, R, n,
                                                                          nrhs);
            kp_end(c, kp, MIDAS_KC_TRSV, 8.0 * na * nb * nrhs, 8.0 * na * nb + 16.0 * na * nrhs + 8.0 * nb * nrhs);
        }
    }
    // backward: U x = y
    for (int k = lu.nblk - 1; k >= 0; --k) {
        int r0 = k * nb;
        ++c->launches;
        int kp = kp_begin(c);
        k_apply_inv<<<nrhs, 64, 0, c->stream>>>(lu.Uinv + (size_t)k * nb * nb, nb, R, n, r0);
        kp_end(c, kp, MIDAS_KC_TRSV, 8.0 * nb * nb * nrhs, 8.0 * nb * nb + 16.0 * nb * nrhs);
        if (r0 > 0) {
            ++c->launches;
            kp = kp_begin(c);
            k_gemv_update<<<(r0 * 32 + 255) / 256, 256, 0, c->stream>>>(lu.A, lu.lda, 0, r0, r0, nb, R, n, nrhs);
            kp_end(c, kp, MIDAS_KC_TRSV, 8.0 * r0 * nb * nrhs, 8.0 * r0 * nb + 16.0 * r0 * nrhs + 8.0 * nb * nrhs);
        }
    }
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// FP64 residual r = b - Z x (Z row-major FP64, warp per row), per-column
// inf-norms of r and x reduced with atomicMax on the bit pattern (>= 0 doubles).
// ---------------------------------------------------------------------------
__global__ void k_residual64(const double2 *Z, long long ldz, int n, const double2 *b, const double2 *x, int nrhs,
                             double2 *r, float2 *r32, unsigned long long *rmax)
{
    int w = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x % 32;
    if (w >= n) return;
    const double2 *row = Z + (long long)w * ldz;
    for (int k = 0; k < nrhs; ++k) {
        const double2 *xv = x + (long long)k * n;
        double sx = 0, sy = 0;
        for (int m = lane; m < n; m += 32) {
            double2 a = row[m], v = xv[m];
            sx += a.x * v.x - a.y * v.y;
            sy += a.x * v.y + a.y * v.x;
        }
        for (int o = 16; o > 0; o >>= 1) {
            sx += __shfl_down_sync(0xffffffffu, sx, o);
            sy += __shfl_down_sync(0xffffffffu, sy, o);
        }
        if (lane == 0) {
            double2 bb = b[(long long)k * n + w];
            double2 rr = make_double2(bb.x - sx, bb.y - sy);
            r[(long long)k * n + w] = rr;
            r32[(long long)k * n + w] = make_float2((float)rr.x, (float)rr.y);
            double a = fmax(fabs(rr.x), fabs(rr.y));
            atomicMax(rmax + k, __double_as_longlong(a));
        }
    }
}

__global__ void k_colmax(const double2 *v, int n, int nrhs, unsigned long long *out)
{
    int k = blockIdx.y;
    double m = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double2 a = v[(long long)k * n + i];
        m = fmax(m, fmax(fabs(a.x), fabs(a.y)));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out + k, __double_as_longlong(m));
}

__global__ void k_add_corr(double2 *x, const float2 *d, long long n)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) { x[i].x += d[i].x; x[i].y += d[i].y; }
}

__global__ void k_rowsum_abs(const double2 *Z, long long ldz, int n, unsigned long long *out)
{
    int w = (blockIdx.x * blockDim.x + threadIdx.x) / 32, lane = threadIdx.x % 32;
    if (w >= n) return;
    double s = 0;
    for (int m = lane; m < n; m += 32) { double2 a = Z[(long long)w * ldz + m]; s += hypot(a.x, a.y); }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) atomicMax(out, __double_as_longlong(s));
}

int inf_norm_rows(midas_gpu_ctx *c, const double2 *Z, long long ldz, int n, double *out)
{
    void *p;
    MIDAS_TRY(ensure(c, S_RED, 64, &p));
    MIDAS_CUDA(c, cudaMemsetAsync(p, 0, 8, c->stream));
    ++c->launches;
    k_rowsum_abs<<<(n * 32 + 255) / 256, 256, 0, c->stream>>>(Z, ldz, n, (unsigned long long *)p);
    MIDAS_CUDA(c, cudaGetLastError());
    unsigned long long h;
    MIDAS_CUDA(c, cudaMemcpyAsync(&h, p, 8, cudaMemcpyDeviceToHost, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    memcpy(out, &h, 8);
    return MIDAS_OK;
}

int ir_solve(midas_gpu_ctx *c, const DenseLU &lu, const double2 *Z64, long long ldz, const double2 *b, double2 *x,
             int nrhs, midas_gpu_info *info)
{
    const int n = lu.n;
    const size_t nn = (size_t)n * nrhs;
    void *p;
    MIDAS_TRY(ensure(c, S_R64, sizeof(double2) * nn, &p));
    double2 *r = (double2 *)p;
    MIDAS_TRY(ensure(c, S_T32B, sizeof(float2) * nn, &p));
    float2 *r32 = (float2 *)p;
    MIDAS_TRY(ensure(c, S_RED, sizeof(unsigned long long) * 3 * nrhs + 64, &p));
    unsigned long long *red = (unsigned long long *)p;
    double znorm;
    MIDAS_TRY(inf_norm_rows(c, Z64, ldz, n, &znorm));
    std::vector<unsigned long long> h(3 * nrhs);
    MIDAS_TRY(ensure(c, S_RED, sizeof(unsigned long long) * 3 * nrhs + 64, &p));
    red = (unsigned long long *)p;
    // bnorm
    MIDAS_CUDA(c, cudaMemsetAsync(red, 0, sizeof(unsigned long long) * 3 * nrhs, c->stream));
    ++c->launches;
    k_colmax<<<dim3(64, nrhs), 256, 0, c->stream>>>(b, n, nrhs, red + 2 * nrhs);
    // x = 0, r = b
    MIDAS_CUDA(c, cudaMemsetAsync(x, 0, sizeof(double2) * nn, c->stream));
    MIDAS_TRY(ensure(c, S_T32, sizeof(float2) * nn, &p));
    float2 *d32 = (float2 *)p;
    // initial residual is b itself
    MIDAS_CUDA(c, cudaMemcpyAsync(r, b, sizeof(double2) * nn, cudaMemcpyDeviceToDevice, c->stream));
    int it = 0;
    double berr = 1e300;
    const double tol = c->opts.ir_tol > 0 ? c->opts.ir_tol : 1e-13;
    const int itmax = c->opts.ir_max_iter > 0 ? c->opts.ir_max_iter : 30;
    // r32 = b (rounded) for the first correction
    {
        MIDAS_CUDA(c, cudaMemsetAsync(red, 0, sizeof(unsigned long long) * 2 * nrhs, c->stream));
        ++c->launches;
        k_residual64<<<(n * 32 + 255) / 256, 256, 0, c->stream>>>(Z64, ldz, n, b, x, nrhs, r, r32, red);
    }
    for (it = 0; it < itmax; ++it) {
        MIDAS_CUDA(c, cudaMemcpyAsync(d32, r32, sizeof(float2) * nn, cudaMemcpyDeviceToDevice, c->stream));
        MIDAS_TRY(lu_solve(c, lu, d32, nrhs));
        ++c->launches;
        k_add_corr<<<(unsigned)((nn + 255) / 256), 256, 0, c->stream>>>(x, d32, (long long)nn);
        MIDAS_CUDA(c, cudaMemsetAsync(red, 0, sizeof(unsigned long long) * 2 * nrhs, c->stream));
        ++c->launches;
        int kp = kp_begin(c);
        k_residual64<<<(n * 32 + 255) / 256, 256, 0, c->stream>>>(Z64, ldz, n, b, x, nrhs, r, r32, red);
        kp_end(c, kp, MIDAS_KC_RESID, 8.0 * n * n * nrhs, 16.0 * n * n + 40.0 * n * nrhs);
        ++c->launches;
        k_colmax<<<dim3(64, nrhs), 256, 0, c->stream>>>(x, n, nrhs, red + nrhs);
        MIDAS_CUDA(c, cudaGetLastError());
        MIDAS_CUDA(c, cudaMemcpyAsync(h.data(), red, sizeof(unsigned long long) * 3 * nrhs, cudaMemcpyDeviceToHost,
                                      c->stream));
        MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
        MIDAS_TRY(check_flag(c, "ir_solve"));
        berr = 0;
        for (int k = 0; k < nrhs; ++k) {
            double rn, xn, bn;
            memcpy(&rn, &h[k], 8);
            memcpy(&xn, &h[nrhs + k], 8);
            memcpy(&bn, &h[2 * nrhs + k], 8);
            double den = znorm * xn + bn;
            berr = fmax(berr, den > 0 ? rn / den : rn);
        }
        if (!(berr == berr)) return c->err.set(MIDAS_ERR_NOT_CONVERGED, "ir_solve: NaN residual");
        if (berr <= tol) { ++it; break; }
    }
    if (info) {
        info->ir_iters = it;
        info->backward_error = berr;
        info->anorm = znorm;
    }
    if (berr > tol) {
        char m[160];
        snprintf(m, sizeof m, "iterative refinement stalled at backward error %.3e after %d steps", berr, it);
        return c->err.set(MIDAS_ERR_NOT_CONVERGED, m);
    }
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// plain FP64 baseline: cuSOLVER zgetrf/zgetrs with partial pivoting (the
// "plain FP64 GPU MoM" of the throughput comparison).  Column-major A, B.
// ---------------------------------------------------------------------------
int zgesv_fp64(midas_gpu_ctx *c, int n, int nrhs, double2 *A, double2 *B, midas_gpu_info *info)
{
    if (!c->cusolver) {
        cusolverDnHandle_t h;
        if (cusolverDnCreate(&h) != CUSOLVER_STATUS_SUCCESS) return c->err.set(MIDAS_ERR_CUDA, "cusolverDnCreate");
        c->cusolver = h;
    }
    cusolverDnHandle_t h = (cusolverDnHandle_t)c->cusolver;
    cusolverDnSetStream(h, c->stream);
    int lwork = 0;
    if (cusolverDnZgetrf_bufferSize(h, n, n, (cuDoubleComplex *)A, n, &lwork) != CUSOLVER_STATUS_SUCCESS)
        return c->err.set(MIDAS_ERR_CUDA, "cusolverDnZgetrf_bufferSize");
    void *p;
    MIDAS_TRY(ensure(c, S_T32, sizeof(cuDoubleComplex) * (size_t)lwork + sizeof(int) * ((size_t)n + 2), &p));
    cuDoubleComplex *work = (cuDoubleComplex *)p;
    int *ipiv = (int *)(work + lwork);
    int *dinfo = ipiv + n;
    if (cusolverDnZgetrf(h, n, n, (cuDoubleComplex *)A, n, work, ipiv, dinfo) != CUSOLVER_STATUS_SUCCESS)
        return c->err.set(MIDAS_ERR_CUDA, "cusolverDnZgetrf");
    if (cusolverDnZgetrs(h, CUBLAS_OP_N, n, nrhs, (cuDoubleComplex *)A, n, ipiv, (cuDoubleComplex *)B, n, dinfo) !=
        CUSOLVER_STATUS_SUCCESS)
        return c->err.set(MIDAS_ERR_CUDA, "cusolverDnZgetrs");
    int hinfo = 0;
    MIDAS_CUDA(c, cudaMemcpyAsync(&hinfo, dinfo, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (hinfo > 0) return c->err.set(MIDAS_ERR_SINGULAR, "SINGULAR MATRIX (zgetrf info > 0)");
    if (info) { info->ir_iters = 0; info->backward_error = 0; }
    return MIDAS_OK;
}



// Mixed solve of a system whose FP64 row-major matrix Z64 and complex64 copy Z32
// (np x np, padded) are already in the pool slots; b/x are np x nrhs (ld np).
int mixed_solve(midas_gpu_ctx *c, int np, float2 *Z32, const double2 *Z64, const double2 *b, double2 *x,
                              int nrhs, midas_gpu_info *info)
{
    DenseLU lu;
    lu.n = np;
    lu.A = Z32;
    lu.lda = np;
    Timer tf(c->stream);
    MIDAS_TRY(lu_factor_nopiv(c, lu));
    MIDAS_TRY(check_flag(c, "lu_factor"));
    float tfac = tf.stop();
    Timer ts(c->stream);
    int st = ir_solve(c, lu, Z64, np, b, x, nrhs, info);
    float tsol = ts.stop();
    if (info) { info->t_factor_ms = tfac; info->t_solve_ms = tsol; }
    return st;
}


void destroy_cusolver(void *h) { cusolverDnDestroy((cusolverDnHandle_t)h); }

}  // namespace midas
