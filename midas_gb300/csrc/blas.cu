// blas.cu -- complex building blocks of the CBFM pipeline (sm_103a).
//
//  * zgemm_x3 : FP32-grade complex GEMM on the tensor cores.  Each operand is
//    split as v = hi + lo with hi = tf32(v) (round to nearest) and the product
//    formed as hi*hi + hi*lo + lo*hi by tripling K (A3 = [A_hi | A_hi | A_lo],
//    B3 = [B_hi ; B_lo ; B_hi]) in one tcgen05 GEMM.  Used where the reference
//    computes in FP64 on FP32 data (the ZGEMMs of the reduced matrix,
//    src/Compute_EFields_CBFME.f90:666-669,791-794).
//  * zgemm64  : strided FP64 complex GEMM on CUDA cores for the small products
//    (Gram matrices, CBF scaling, Vc = C^T Einc, E = C alpha).
//  * residual_df32 : r = B - Z X with Z single precision (exact), X given as a
//    double-float pair; products are exact (FMA two-product) and sums use
//    compensated double-float accumulation, giving an FP64-grade residual
//    without the GB300's slow FP64 pipe.
//  * heev_jacobi : Hermitian eigen-decomposition (parallel cyclic Jacobi, FP64)
//    of the CBF Gram matrices; one CTA per matrix.
#include <cmath>

#include "common.cuh"
#include "kernels.cuh"

namespace midas {

__device__ __forceinline__ float tf32_rna(float x)
{
    uint32_t u;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(x));
    return __uint_as_float(u);
}

template <typename T>
__device__ __forceinline__ double2 ld2(const T *p, long long i);
template <>
__device__ __forceinline__ double2 ld2<float2>(const float2 *p, long long i)
{
    float2 v = p[i];
    return make_double2(v.x, v.y);
}
template <>
__device__ __forceinline__ double2 ld2<double2>(const double2 *p, long long i)
{
    return p[i];
}

__device__ __forceinline__ void split2(double v, float &hi, float &lo)
{
    hi = tf32_rna((float)v);
    lo = tf32_rna((float)(v - (double)hi));
}

// A3[i][.] for element (i, k) = src[i*rs + k*cs] (optionally conjugated)
template <typename T>
__global__ void k_split_a(int M, int K, const T *src, long long rs, long long cs, int conj, float *A3, long long lda3)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    int i = blockIdx.y;
    if (k >= K || i >= M) return;
    double2 v = ld2<T>(src, (long long)i * rs + (long long)k * cs);
    if (conj) v.y = -v.y;
    float hr, lr, hi_, li;
    split2(v.x, hr, lr);
    split2(v.y, hi_, li);
    float *row = A3 + (long long)i * lda3;
    row[2 * k] = hr; row[2 * k + 1] = hi_;
    row[2 * K + 2 * k] = hr; row[2 * K + 2 * k + 1] = hi_;
    row[4 * K + 2 * k] = lr; row[4 * K + 2 * k + 1] = li;
}

// B3t rows 2j, 2j+1 for element (k, j) = src[k*rs + j*cs]
template <typename T>
__global__ void k_split_expand_b(int K, int N, const T *src, long long rs, long long cs, float *B3, long long ldb3)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    int j = blockIdx.y;
    if (k >= K || j >= N) return;
    double2 v = ld2<T>(src, (long long)k * rs + (long long)j * cs);
    float hr, lr, hi_, li;
    split2(v.x, hr, lr);
    split2(v.y, hi_, li);
    float *r0 = B3 + (long long)(2 * j) * ldb3, *r1 = r0 + ldb3;
    // segment 0: hi, segment 1: lo, segment 2: hi
    r0[2 * k] = hr; r0[2 * k + 1] = -hi_; r1[2 * k] = hi_; r1[2 * k + 1] = hr;
    r0[2 * K + 2 * k] = lr; r0[2 * K + 2 * k + 1] = -li; r1[2 * K + 2 * k] = li; r1[2 * K + 2 * k + 1] = lr;
    r0[4 * K + 2 * k] = hr; r0[4 * K + 2 * k + 1] = -hi_; r1[4 * K + 2 * k] = hi_; r1[4 * K + 2 * k + 1] = hr;
}

template <typename TA, typename TB>
int zgemm_x3(midas_gpu_ctx *c, int M, int N, int K, const TA *A, long long ars, long long acs, int conjA,
             const TB *B, long long brs, long long bcs, float *D, long long ldd, float alpha, float beta)
{
    if (M <= 0 || N <= 0 || K <= 0) return MIDAS_OK;
    long long K6 = (6LL * K + 3) / 4 * 4;   // row stride multiple of 4 floats (16 B)
    void *pa, *pb;
    MIDAS_TRY(ensure(c, S_CBF8, sizeof(float) * (size_t)M * K6, &pa));
    MIDAS_TRY(ensure(c, S_CBF9, sizeof(float) * (size_t)2 * N * K6, &pb));
    float *A3 = (float *)pa, *B3 = (float *)pb;
    if (K6 != 6LL * K) {   // keep the padding columns zero
        MIDAS_CUDA(c, cudaMemsetAsync(A3, 0, sizeof(float) * (size_t)M * K6, c->stream));
        MIDAS_CUDA(c, cudaMemsetAsync(B3, 0, sizeof(float) * (size_t)2 * N * K6, c->stream));
    }
    ++c->launches;
    k_split_a<TA><<<dim3((K + 127) / 128, M), 128, 0, c->stream>>>(M, K, A, ars, acs, conjA, A3, K6);
    ++c->launches;
    k_split_expand_b<TB><<<dim3((K + 127) / 128, N), 128, 0, c->stream>>>(K, N, B, brs, bcs, B3, K6);
    MIDAS_CUDA(c, cudaGetLastError());
    GemmArgs g{M, 2 * N, (int)K6, A3, K6, B3, K6, D, ldd, alpha, beta};
    return gemm_tf32(c, g);
}
template int zgemm_x3<float2, double2>(midas_gpu_ctx *, int, int, int, const float2 *, long long, long long, int,
                                       const double2 *, long long, long long, float *, long long, float, float);
template int zgemm_x3<double2, float2>(midas_gpu_ctx *, int, int, int, const double2 *, long long, long long, int,
                                       const float2 *, long long, long long, float *, long long, float, float);
template int zgemm_x3<double2, double2>(midas_gpu_ctx *, int, int, int, const double2 *, long long, long long, int,
                                        const double2 *, long long, long long, float *, long long, float, float);
template int zgemm_x3<float2, float2>(midas_gpu_ctx *, int, int, int, const float2 *, long long, long long, int,
                                      const float2 *, long long, long long, float *, long long, float, float);

// ---------------------------------------------------------------------------
// FP64 complex GEMM, strided: C(i,j) = alpha * sum_k opA(i,k) B(k,j) + beta * C(i,j)
// 16 x 16 tiles, K in chunks of 16.
// ---------------------------------------------------------------------------
__global__ void k_zgemm64(int M, int N, int K, const double2 *A, long long ars, long long acs, int conjA,
                          const double2 *B, long long brs, long long bcs, double2 *C, long long crs, long long ccs,
                          double2 alpha, double2 beta)
{
    __shared__ double2 As[16][17], Bs[16][17];
    int tx = threadIdx.x, ty = threadIdx.y;
    int i = blockIdx.y * 16 + ty, j = blockIdx.x * 16 + tx;
    double2 acc = make_double2(0, 0);
    for (int k0 = 0; k0 < K; k0 += 16) {
        int ka = k0 + tx, kb = k0 + ty;
        double2 a = make_double2(0, 0), b = make_double2(0, 0);
        if (i < M && ka < K) { a = A[(long long)i * ars + (long long)ka * acs]; if (conjA) a.y = -a.y; }
        if (kb < K && j < N) b = B[(long long)kb * brs + (long long)j * bcs];
        As[ty][tx] = a;
        Bs[ty][tx] = b;
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            double2 x = As[ty][kk], y = Bs[kk][tx];
            acc.x += x.x * y.x - x.y * y.y;
            acc.y += x.x * y.y + x.y * y.x;
        }
        __syncthreads();
    }
    if (i < M && j < N) {
        double2 *o = C + (long long)i * crs + (long long)j * ccs;
        double2 r = make_double2(alpha.x * acc.x - alpha.y * acc.y, alpha.x * acc.y + alpha.y * acc.x);
        if (beta.x != 0 || beta.y != 0) {
            double2 p = *o;
            r.x += beta.x * p.x - beta.y * p.y;
            r.y += beta.x * p.y + beta.y * p.x;
        }
        *o = r;
    }
}

int zgemm64(midas_gpu_ctx *c, int M, int N, int K, const double2 *A, long long ars, long long acs, int conjA,
            const double2 *B, long long brs, long long bcs, double2 *C, long long crs, long long ccs, double2 alpha,
            double2 beta)
{
    if (M <= 0 || N <= 0) return MIDAS_OK;
    dim3 blk(16, 16), grd((N + 15) / 16, (M + 15) / 16);
    ++c->launches;
    k_zgemm64<<<grd, blk, 0, c->stream>>>(M, N, K, A, ars, acs, conjA, B, brs, bcs, C, crs, ccs, alpha, beta);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// double-float residual: r = B - Z X,  Z (n x n row-major fp32, ldz), X = Xh + Xl
// (fp32 pairs, column-major ld = n), B fp32 column-major (ld n).  r is FP64.
// Tile: 32 rows x 32 rhs per CTA (256 threads, 4 outputs each).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

struct DF {
    float hi, lo;
};
__device__ __forceinline__ void df_add_prod(DF &acc, float a, float b)
{
    float p = a * b;
    float pe = fmaf(a, b, -p);   // exact product = p + pe
    float s, e;
    two_sum(acc.hi, p, s, e);
    acc.hi = s;
    acc.lo += e + pe;
}

__global__ void __launch_bounds__(256) k_residual_df32(int n, int nrhs, const float2 *Z, long long ldz,
                                                        const float2 *Xh, const float2 *Xl, const float2 *B,
                                                        double2 *R)
{
    __shared__ float2 Zs[32][33];
    __shared__ float2 Xhs[32][33], Xls[32][33];
    int tid = threadIdx.x;
    int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
    int lr = tid / 8;          // row within tile (0..31)
    int lc = (tid % 8) * 4;    // 4 rhs columns per thread
    DF accr[4], acci[4];
    float cr[4] = {0, 0, 0, 0}, ci[4] = {0, 0, 0, 0};   // lo-part products (plain fp32)
    for (int q = 0; q < 4; ++q) { accr[q] = {0.f, 0.f}; acci[q] = {0.f, 0.f}; }
    for (int k0 = 0; k0 < n; k0 += 32) {
        for (int t = tid; t < 32 * 32; t += 256) {
            int a = t / 32, b = t % 32;
            int row = r0 + a, k = k0 + b;
            Zs[a][b] = (row < n && k < n) ? Z[(long long)row * ldz + k] : make_float2(0.f, 0.f);
            int kk = k0 + a, col = c0 + b;
            bool ok = kk < n && col < nrhs;
            Xhs[a][b] = ok ? Xh[(long long)col * n + kk] : make_float2(0.f, 0.f);
            Xls[a][b] = ok ? Xl[(long long)col * n + kk] : make_float2(0.f, 0.f);
        }
        __syncthreads();
        for (int k = 0; k < 32; ++k) {
            float2 z = Zs[lr][k];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float2 xh = Xhs[k][lc + q], xl = Xls[k][lc + q];
                // real: z.x*xh.x - z.y*xh.y ; imag: z.x*xh.y + z.y*xh.x (exact products)
                df_add_prod(accr[q], z.x, xh.x);
                df_add_prod(accr[q], -z.y, xh.y);
                df_add_prod(acci[q], z.x, xh.y);
                df_add_prod(acci[q], z.y, xh.x);
                cr[q] += z.x * xl.x - z.y * xl.y;
                ci[q] += z.x * xl.y + z.y * xl.x;
            }
        }
        __syncthreads();
    }
    int row = r0 + lr;
    if (row >= n) return;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        int col = c0 + lc + q;
        if (col >= nrhs) continue;
        double zr = (double)accr[q].hi + (double)accr[q].lo + (double)cr[q];
        double zi = (double)acci[q].hi + (double)acci[q].lo + (double)ci[q];
        float2 b = B[(long long)col * n + row];
        R[(long long)col * n + row] = make_double2((double)b.x - zr, (double)b.y - zi);
    }
}

int residual_df32(midas_gpu_ctx *c, int n, int nrhs, const float2 *Z, long long ldz, const float2 *Xh,
                  const float2 *Xl, const float2 *B, double2 *R)
{
    dim3 grd((nrhs + 31) / 32, (n + 31) / 32);
    ++c->launches;
    k_residual_df32<<<grd, 256, 0, c->stream>>>(n, nrhs, Z, ldz, Xh, Xl, B, R);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// Hermitian Jacobi eigen-solver (FP64), one CTA per matrix.
// A: batch of m x m Hermitian matrices (row-major, leading dim lda, stride sa);
// on exit W (descending eigenvalues) and V (row-major m x m, columns = vectors).
// Parallel ordering: round-robin tournament, m/2 disjoint pairs per round.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) k_heev_jacobi(int m, double2 *A, long long lda, long long sa, double2 *V,
                                                      long long sv, double *W, int sweeps, double tol)
{
    extern __shared__ double sh[];
    int mm = m + (m & 1);    // even player count (a dummy when m is odd)
    int *perm = (int *)sh;   // mm ints
    double *cs = (double *)(perm + mm + (mm & 1));   // per pair: c, s*cos(phi), s*sin(phi)
    double *red = cs + 3 * (mm / 2);
    double2 *a = A + blockIdx.x * sa;
    double2 *v = V + blockIdx.x * sv;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int t = tid; t < m * m; t += nt) v[(t / m) * m + t % m] = make_double2((t / m == t % m) ? 1.0 : 0.0, 0.0);
    for (int t = tid; t < mm; t += nt) perm[t] = t;
    __syncthreads();
    for (int sw = 0; sw < sweeps; ++sw) {
        // off-diagonal norm vs diagonal norm
        double off = 0, dia = 0;
        for (int t = tid; t < m * m; t += nt) {
            int i = t / m, j = t % m;
            double2 x = a[(long long)i * lda + j];
            double q = x.x * x.x + x.y * x.y;
            if (i == j) dia += q; else off += q;
        }
        for (int o = 16; o > 0; o >>= 1) {
            off += __shfl_down_sync(0xffffffffu, off, o);
            dia += __shfl_down_sync(0xffffffffu, dia, o);
        }
        if ((tid & 31) == 0) { red[2 * (tid >> 5)] = off; red[2 * (tid >> 5) + 1] = dia; }
        __syncthreads();
        if (tid == 0) {
            double so = 0, sd = 0;
            for (int w = 0; w < nt / 32; ++w) { so += red[2 * w]; sd += red[2 * w + 1]; }
            red[0] = so; red[1] = sd;
        }
        __syncthreads();
        bool done = red[0] <= tol * tol * red[1];
        __syncthreads();
        if (done) break;
        for (int round = 0; round < mm - 1; ++round) {
            // pair t: (perm[t], perm[mm-1-t])
            for (int t = tid; t < mm / 2; t += nt) {
                int p = perm[t], q = perm[mm - 1 - t];
                if (p > q) { int tmp = p; p = q; q = tmp; }
                double c = 1, sr = 0, si = 0;
                if (q < m) {
                    double app = a[(long long)p * lda + p].x, aqq = a[(long long)q * lda + q].x;
                    double2 apq = a[(long long)p * lda + q];
                    double g = hypot(apq.x, apq.y);
                    if (g > 1e-300) {
                        // zero a_pq: tan(2 th) = 2|a_pq| / (a_qq - a_pp)
                        double th = 0.5 * atan2(2.0 * g, aqq - app);
                        double cth = cos(th), sth = sin(th);
                        c = cth;
                        sr = sth * apq.x / g;
                        si = sth * apq.y / g;
                    }
                }
                cs[3 * t] = c; cs[3 * t + 1] = sr; cs[3 * t + 2] = si;
            }
            __syncthreads();
            // rotation J on columns (p, q): J_pp = c, J_qq = c, J_pq = s e^{i phi}... applied as
            // A <- J^H A J, V <- V J with  col_p' = c col_p - conj(s) col_q,  col_q' = s col_p + c col_q
            // rows: row_p' = c row_p - s row_q, row_q' = conj(s) row_p + c row_q
            int npair = mm / 2;
            for (int t = tid; t < npair * m; t += nt) {   // rows
                int pr = t / m, k = t % m;
                int p = perm[pr], q = perm[mm - 1 - pr];
                if (p > q) { int tmp = p; p = q; q = tmp; }
                if (q >= m) continue;
                double c = cs[3 * pr], sr = cs[3 * pr + 1], si = cs[3 * pr + 2];
                double2 x = a[(long long)p * lda + k], y = a[(long long)q * lda + k];
                // row_p' = c x - s y ; row_q' = conj(s) x + c y     (s = sr + i si)
                a[(long long)p * lda + k] = make_double2(c * x.x - (sr * y.x - si * y.y), c * x.y - (sr * y.y + si * y.x));
                a[(long long)q * lda + k] = make_double2(sr * x.x + si * x.y + c * y.x, sr * x.y - si * x.x + c * y.y);
            }
            __syncthreads();
            for (int t = tid; t < npair * m; t += nt) {   // columns of A and V
                int pr = t / m, k = t % m;
                int p = perm[pr], q = perm[mm - 1 - pr];
                if (p > q) { int tmp = p; p = q; q = tmp; }
                if (q >= m) continue;
                double c = cs[3 * pr], sr = cs[3 * pr + 1], si = cs[3 * pr + 2];
                // col_p' = c x - conj(s) y ; col_q' = s x + c y
                double2 x = a[(long long)k * lda + p], y = a[(long long)k * lda + q];
                a[(long long)k * lda + p] = make_double2(c * x.x - (sr * y.x + si * y.y), c * x.y - (sr * y.y - si * y.x));
                a[(long long)k * lda + q] = make_double2(sr * x.x - si * x.y + c * y.x, sr * x.y + si * x.x + c * y.y);
                x = v[(long long)k * m + p];
                y = v[(long long)k * m + q];
                v[(long long)k * m + p] = make_double2(c * x.x - (sr * y.x + si * y.y), c * x.y - (sr * y.y - si * y.x));
                v[(long long)k * m + q] = make_double2(sr * x.x - si * x.y + c * y.x, sr * x.y + si * x.x + c * y.y);
            }
            __syncthreads();
            // rotate the tournament (player 0 fixed)
            if (tid == 0) {
                int last = perm[mm - 1];
                for (int t = mm - 1; t > 1; --t) perm[t] = perm[t - 1];
                perm[1] = last;
            }
            __syncthreads();
        }
    }
    // eigenvalues: diagonal, sorted descending together with the vectors (selection sort on indices)
    double *wv = W + blockIdx.x * m;
    for (int t = tid; t < m; t += nt) wv[t] = a[(long long)t * lda + t].x;
    __syncthreads();
    if (tid == 0) {
        for (int i = 0; i < m; ++i) perm[i] = i;
        for (int i = 0; i < m; ++i) {
            int b = i;
            for (int j = i + 1; j < m; ++j)
                if (wv[perm[j]] > wv[perm[b]]) b = j;
            int tmp = perm[i]; perm[i] = perm[b]; perm[b] = tmp;
        }
    }
    __syncthreads();
    // permute: write sorted eigenvalues into red scratch then back; vectors into A (as scratch)
    for (int t = tid; t < m * m; t += nt) {
        int k = t / m, j = t % m;
        a[(long long)k * lda + j] = v[(long long)k * m + perm[j]];
    }
    __syncthreads();
    for (int t = tid; t < m * m; t += nt) {
        int k = t / m, j = t % m;
        v[(long long)k * m + j] = a[(long long)k * lda + j];
    }
    double *tmpw = red;   // red has room for >= 2*32 doubles; use W directly with a second pass
    __syncthreads();
    if (tid == 0) {
        // in-place permutation of wv via V's first row is not available; use a simple O(m^2) rewrite
        for (int i = 0; i < m; ++i) tmpw[0] = 0;
    }
    __syncthreads();
    // sorted eigenvalues: read diag of the (unchanged) eigenvalue array through perm
    // (store into A's diagonal first to avoid aliasing)
    for (int t = tid; t < m; t += nt) a[(long long)t * lda + t].x = wv[perm[t]];
    __syncthreads();
    for (int t = tid; t < m; t += nt) wv[t] = a[(long long)t * lda + t].x;
}

int heev_jacobi(midas_gpu_ctx *c, int batch, int m, double2 *A, long long lda, long long sa, double2 *V,
                long long sv, double *W)
{
    int mm = m + (m & 1);
    size_t sm = sizeof(int) * (mm + 2) + sizeof(double) * (3 * (mm / 2) + 64) + 64;
    static int attr_set = 0;
    if (sm > 48 * 1024 && !attr_set) {
        MIDAS_CUDA(c, cudaFuncSetAttribute(k_heev_jacobi, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        attr_set = 1;
    }
    ++c->launches;
    k_heev_jacobi<<<batch, 1024, sm, c->stream>>>(m, A, lda, sa, V, sv, W, 30, 1e-15);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

}  // namespace midas
