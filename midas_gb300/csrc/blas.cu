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
//  * heev_dev : Hermitian eigen-decomposition (Householder tridiagonalisation +
//    implicit QL, FP64) of the CBF Gram matrices; one CTA per matrix.
#include <cuda_fp16.h>
#include <cmath>

#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace midas {


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
    if (k >= K) return;
    for (int i = blockIdx.y; i < M; i += gridDim.y) {   // rows beyond the 65535 grid limit loop
        double2 v = ld2<T>(src, (long long)i * rs + (long long)k * cs);
        if (conj) v.y = -v.y;
        float hr, lr, hi_, li;
        split2(v.x, hr, lr);
        split2(v.y, hi_, li);
        float *row = A3 + (long long)i * lda3;
        row[2 * k] = hr; row[2 * k + 1] = hi_;
        row[2 * K + 2 * k] = hr; row[2 * K + 2 * k + 1] = hi_;
        row[4 * K + 2 * k] = lr; row[4 * K + 2 * k + 1] = li;
        if (k == K - 1)   // the padding columns of the row
            for (long long p = 6LL * K; p < lda3; ++p) row[p] = 0.f;
    }
}

// B3t rows 2j, 2j+1 for element (k, j) = src[k*rs + j*cs]
template <typename T>
__global__ void k_split_expand_b(int K, int N, const T *src, long long rs, long long cs, float *B3, long long ldb3)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    for (int j = blockIdx.y; j < N; j += gridDim.y) {
        double2 v = ld2<T>(src, (long long)k * rs + (long long)j * cs);
        float hr, lr, hi_, li;
        split2(v.x, hr, lr);
        split2(v.y, hi_, li);
        float *r0 = B3 + (long long)(2 * j) * ldb3, *r1 = r0 + ldb3;
        // segment 0: hi, segment 1: lo, segment 2: hi
        r0[2 * k] = hr; r0[2 * k + 1] = -hi_; r1[2 * k] = hi_; r1[2 * k + 1] = hr;
        r0[2 * K + 2 * k] = lr; r0[2 * K + 2 * k + 1] = -li; r1[2 * K + 2 * k] = li; r1[2 * K + 2 * k + 1] = lr;
        r0[4 * K + 2 * k] = hr; r0[4 * K + 2 * k + 1] = -hi_; r1[4 * K + 2 * k] = hi_; r1[4 * K + 2 * k + 1] = hr;
        if (k == K - 1)
            for (long long p = 6LL * K; p < ldb3; ++p) { r0[p] = 0.f; r1[p] = 0.f; }
    }
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
    ++c->launches;
    int kp = kp_begin(c);
    k_split_a<TA><<<dim3((K + 127) / 128, std::min(M, 65535)), 128, 0, c->stream>>>(M, K, A, ars, acs, conjA, A3, K6);
    kp_end(c, kp, MIDAS_KC_SPLIT, 0.0, (double)M * K * sizeof(TA) + 4.0 * M * K6);
    ++c->launches;
    kp = kp_begin(c);
    k_split_expand_b<TB><<<dim3((K + 127) / 128, std::min(N, 65535)), 128, 0, c->stream>>>(K, N, B, brs, bcs, B3,
                                                                                            K6);
    kp_end(c, kp, MIDAS_KC_SPLIT, 0.0, (double)N * K * sizeof(TB) + 8.0 * N * K6);
    MIDAS_CUDA(c, cudaGetLastError());
    GemmArgs g{M, 2 * N, (int)K6, A3, K6, B3, K6, D, ldd, alpha, beta, 0, MIDAS_KC_GEMM_PROD};
    return gemm_tf32(c, g, true);
}
// the same product with A already split (hi | hi | lo rows of K6 floats, e.g.
// written by launch_block_fill4_a3)
template <typename TB>
int zgemm_x3_a3(midas_gpu_ctx *c, int M, int N, int K, const float *A3, long long K6, const TB *B, long long brs,
                long long bcs, float *D, long long ldd, float alpha, float beta, int kclass)
{
    if (M <= 0 || N <= 0 || K <= 0) return MIDAS_OK;
    if (K6 != (6LL * K + 3) / 4 * 4) return c->err.set(MIDAS_ERR_ARG, "zgemm_x3_a3: bad A3 stride");
    void *pb;
    MIDAS_TRY(ensure(c, S_CBF9, sizeof(float) * (size_t)2 * N * K6, &pb));
    float *B3 = (float *)pb;
    ++c->launches;
    int kp = kp_begin(c);
    k_split_expand_b<TB><<<dim3((K + 127) / 128, std::min(N, 65535)), 128, 0, c->stream>>>(K, N, B, brs, bcs, B3,
                                                                                            K6);
    kp_end(c, kp, MIDAS_KC_SPLIT, 0.0, (double)N * K * sizeof(TB) + 8.0 * N * K6);
    MIDAS_CUDA(c, cudaGetLastError());
    GemmArgs g{M, 2 * N, (int)K6, A3, K6, B3, K6, D, ldd, alpha, beta, 0, kclass};
    return gemm_tf32(c, g, true);
}
template int zgemm_x3_a3<double2>(midas_gpu_ctx *, int, int, int, const float *, long long, const double2 *,
                                  long long, long long, float *, long long, float, float, int);
template int zgemm_x3_a3<float2>(midas_gpu_ctx *, int, int, int, const float *, long long, const float2 *,
                                 long long, long long, float *, long long, float, float, int);

// ---------------------------------------------------------------------------
// The same split product on fp16 operands (kind::f16: the 11-bit significands of
// TF32 at half the bytes and twice the MMA rate).  FP16 has a narrow exponent
// range, so each operand is scaled by a power of two that puts its largest
// entry in [2^12, 2^13): the hi pieces of entries down to 2^-24 of the maximum
// stay normal, and what falls out of range is below 2^-37 of the maximum.  The
// GEMM multiplies by 1 / (sA sB), read from device memory.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_cabsmax(int M, int K, const T *src, long long rs, long long cs, unsigned *out)
{
    float m = 0.f;
    for (int i = blockIdx.x; i < M; i += gridDim.x)
        for (int k = threadIdx.x; k < K; k += blockDim.x) {
            const double2 v = ld2<T>(src, (long long)i * rs + (long long)k * cs);
            m = fmaxf(m, (float)fmax(fabs(v.x), fabs(v.y)));
        }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(out, __float_as_uint(m));
}

// s = 2^(12 - ceil(log2 max)) (1 for an all-zero operand); which = 0: A, 1: B and alpha = 1 / (sA sB)
__global__ void k_h16_scale(const unsigned *amax, float *sc, int which)
{
    const float m = __uint_as_float(*amax);
    int e = 0;
    if (m > 0.f) e = 12 - (int)ceilf(log2f(m));
    e = max(-120, min(120, e));
    sc[which] = ldexpf(1.f, e);
    if (which == 1) sc[2] = 1.f / (sc[0] * sc[1]);
}

__device__ __forceinline__ void split_h16(double v, float s, __half &hi, __half &lo)
{
    const double x = v * (double)s;
    hi = __float2half_rn((float)x);
    lo = __float2half_rn((float)(x - (double)__half2float(hi)));
}
// the same for an FP32 value, in FP32 (x - hi is exact: hi holds x's leading bits)
__device__ __forceinline__ void split_h16(float v, float s, __half &hi, __half &lo)
{
    const float x = v * s;
    hi = __float2half_rn(x);
    lo = __float2half_rn(x - __half2float(hi));
}
template <typename T> struct SplitIn;
template <> struct SplitIn<float2> {
    using V = float2;
    static __device__ __forceinline__ float2 ld(const float2 *p, long long i) { return p[i]; }
};
template <> struct SplitIn<double2> {
    using V = double2;
    static __device__ __forceinline__ double2 ld(const double2 *p, long long i) { return p[i]; }
};

// Rows 2j, 2j+1 of B3 for element (k, j) = (hr + lr) + i (hi + li): the real 2 x 2 form
// [re -im; im re] of each piece, pieces [hi | lo | hi] of pw halves; the thread of the
// last k zeroes the pieces' tails.
__device__ __forceinline__ void h16_b3_store(__half *r0, long long ldb3, int k, int K, long long pw, __half hr,
                                             __half hi_, __half lr, __half li)
{
    __half *r1 = r0 + ldb3;
    const __half nhi = __hneg(hi_), nli = __hneg(li);
    r0[2 * k] = hr; r0[2 * k + 1] = nhi; r1[2 * k] = hi_; r1[2 * k + 1] = hr;
    r0[pw + 2 * k] = lr; r0[pw + 2 * k + 1] = nli; r1[pw + 2 * k] = li; r1[pw + 2 * k + 1] = lr;
    r0[2 * pw + 2 * k] = hr; r0[2 * pw + 2 * k + 1] = nhi; r1[2 * pw + 2 * k] = hi_; r1[2 * pw + 2 * k + 1] = hr;
    if (k == K - 1)
        for (long long p = 2LL * K; p < pw; ++p)
            for (int q = 0; q < 3; ++q) { r0[q * pw + p] = __float2half(0.f); r1[q * pw + p] = __float2half(0.f); }
}

// A in the two-piece layout: row i = [hi | lo], each piece 2 h16_piece(K) halves
// (the thread of the last column zeroes the pieces' tails)
template <typename T>
__global__ void k_split_a_h16(int M, int K, const T *src, long long rs, long long cs, const float *sc, __half *A2,
                              long long lda2)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const float s = sc[0];
    const long long pw = 2 * h16_piece(K);   // halves per piece
    for (int i = blockIdx.y; i < M; i += gridDim.y) {
        const auto v = SplitIn<T>::ld(src, (long long)i * rs + (long long)k * cs);
        __half hr, lr, hi_, li;
        split_h16(v.x, s, hr, lr);
        split_h16(v.y, s, hi_, li);
        __half *row = A2 + (long long)i * lda2;
        row[2 * k] = hr; row[2 * k + 1] = hi_;
        row[pw + 2 * k] = lr; row[pw + 2 * k + 1] = li;
        if (k == K - 1)
            for (long long p = 2LL * K; p < pw; ++p) { row[p] = __float2half(0.f); row[pw + p] = __float2half(0.f); }
    }
}

template <typename T>
__global__ void k_split_expand_b_h16(int K, int N, const T *src, long long rs, long long cs, const float *sc,
                                     __half *B3, long long ldb3)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const float s = sc[1];
    const long long pw = 2 * h16_piece(K);   // halves per piece: [hi | lo | hi]
    for (int j = blockIdx.y; j < N; j += gridDim.y) {
        const auto v = SplitIn<T>::ld(src, (long long)k * rs + (long long)j * cs);
        __half hr, lr, hi_, li;
        split_h16(v.x, s, hr, lr);
        split_h16(v.y, s, hi_, li);
        h16_b3_store(B3 + (long long)(2 * j) * ldb3, ldb3, k, K, pw, hr, hi_, lr, li);
    }
}

// The same split and expansion of a row-major B (element (k, j) at src[k rs + j]),
// through a 32 x 32 tile in shared memory so that the reads (along j) and the writes
// (along k) both coalesce.  Block (j tile, k tile), 256 threads.
template <typename T>
__global__ void __launch_bounds__(256) k_split_expand_b_h16_t(int K, int N, const T *src, long long rs,
                                                              const float *sc, __half *B3, long long ldb3)
{
    using V = typename SplitIn<T>::V;
    __shared__ V tile[32][33];   // [k][j]
    const int j0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
    const int tx = threadIdx.x % 32, ty = threadIdx.x / 32;
    for (int r = ty; r < 32; r += 8) {
        const int k = k0 + r, j = j0 + tx;
        V v;
        v.x = 0; v.y = 0;
        if (k < K && j < N) v = SplitIn<T>::ld(src, (long long)k * rs + j);
        tile[r][tx] = v;
    }
    __syncthreads();
    const float s = sc[1];
    for (int r = ty; r < 32; r += 8) {
        const int j = j0 + r, k = k0 + tx;
        if (j >= N || k >= K) continue;
        const V v = tile[tx][r];
        __half hr, lr, hi_, li;
        split_h16(v.x, s, hr, lr);
        split_h16(v.y, s, hi_, li);
        h16_b3_store(B3 + (long long)(2 * j) * ldb3, ldb3, k, K, 2 * h16_piece(K), hr, hi_, lr, li);
    }
}

// A3h (fp16 [hi | lo] rows of K6h = h16_arow(K) halves) of a row-major complex64 M x K
// matrix, with its scale in sc[0] (sc: 4 floats of device memory after the split)
int zsplit_a3_h16(midas_gpu_ctx *c, int M, int K, const float2 *A, long long lda, __half *A3, long long K6h,
                  float *sc)
{
    if (M <= 0 || K <= 0) return MIDAS_OK;
    if (K6h != h16_arow(K)) return c->err.set(MIDAS_ERR_ARG, "zsplit_a3_h16: bad A row stride");
    ++c->launches;
    int kp = kp_begin(c);
    MIDAS_CUDA(c, cudaMemsetAsync(sc + 3, 0, sizeof(unsigned), c->stream));
    k_cabsmax<float2><<<std::min(M, 4096), 256, 0, c->stream>>>(M, K, A, lda, 1, (unsigned *)(sc + 3));
    k_h16_scale<<<1, 1, 0, c->stream>>>((const unsigned *)(sc + 3), sc, 0);
    k_split_a_h16<float2><<<dim3((K + 127) / 128, std::min(M, 65535)), 128, 0, c->stream>>>(M, K, A, lda, 1, sc, A3,
                                                                                             K6h);
    kp_end(c, kp, MIDAS_KC_SPLIT, 0.0, 16.0 * M * K + 2.0 * M * K6h);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// D (M x 2N floats, row-major, ld ldd) = A B with A given as its fp16 split A3h
// (M rows of K6h = h16_arow(K) halves: the [hi | lo] pieces, scale sA in sc[0]) and B
// (K x N complex, element (k, j) at B[k brs + j bcs]): B is scaled (sc[1]) and split here
// into [hi | lo | hi] rows, the GEMM reads A's hi piece twice and multiplies by
// 1 / (sA sB) (sc[2]); sc[3] is scratch.
template <typename TB>
int zgemm_x3h_a3(midas_gpu_ctx *c, int M, int N, int K, const __half *A3h, long long K6h, float *sc, const TB *B,
                 long long brs, long long bcs, float *D, long long ldd, int kclass, int promote_kb)
{
    if (M <= 0 || N <= 0 || K <= 0) return MIDAS_OK;
    if (K6h != h16_arow(K)) return c->err.set(MIDAS_ERR_ARG, "zgemm_x3h_a3: bad A row stride");
    const long long KB = h16_brow(K);   // halves per B3 row, the GEMM's K
    void *pb;
    MIDAS_TRY(ensure(c, S_CBF9, sizeof(__half) * (size_t)2 * N * KB + 256, &pb));
    __half *B3 = (__half *)pb;
    ++c->launches;
    int kp = kp_begin(c);
    MIDAS_CUDA(c, cudaMemsetAsync(sc + 3, 0, sizeof(unsigned), c->stream));
    k_cabsmax<TB><<<std::min(K, 4096), 256, 0, c->stream>>>(K, N, B, brs, bcs, (unsigned *)(sc + 3));
    k_h16_scale<<<1, 1, 0, c->stream>>>((const unsigned *)(sc + 3), sc, 1);
    if (bcs == 1 && brs != 1)   // row-major B: the transposing split
        k_split_expand_b_h16_t<TB><<<dim3((N + 31) / 32, (K + 31) / 32), 256, 0, c->stream>>>(K, N, B, brs, sc, B3,
                                                                                             KB);
    else
        k_split_expand_b_h16<TB><<<dim3((K + 127) / 128, std::min(N, 65535)), 128, 0, c->stream>>>(K, N, B, brs, bcs,
                                                                                                   sc, B3, KB);
    kp_end(c, kp, MIDAS_KC_SPLIT, 0.0, (double)sizeof(TB) * K * N + 4.0 * N * KB);
    MIDAS_CUDA(c, cudaGetLastError());
    GemmArgs g{M, 2 * N, (int)KB, (const float *)A3h, K6h, (const float *)B3, KB, D, ldd, 1.f, 0.f, 0, kclass};
    g.h16 = 1;
    g.alpha_dev = sc + 2;
    g.promote_kb = promote_kb;
    g.a_piece = 2 * h16_piece(K);
    return gemm_tf32(c, g, true);
}
template int zgemm_x3h_a3<double2>(midas_gpu_ctx *, int, int, int, const __half *, long long, float *,
                                   const double2 *, long long, long long, float *, long long, int, int);

// D (M x 2N floats) = A B on fp16 split pieces, both operands split here: A (M x K
// complex, element (i, k) at A[i ars + k acs]) scaled by sc[0], B as in zgemm_x3h_a3
template <typename TA, typename TB>
int zgemm_x3h(midas_gpu_ctx *c, int M, int N, int K, const TA *A, long long ars, long long acs, const TB *B,
              long long brs, long long bcs, float *D, long long ldd, int kclass, int promote_kb)
{
    if (M <= 0 || N <= 0 || K <= 0) return MIDAS_OK;
    const long long K6h = h16_arow(K);
    void *pa;
    MIDAS_TRY(ensure(c, S_CBF8, sizeof(__half) * (size_t)M * K6h + 256, &pa));
    __half *A3h = (__half *)pa;
    float *sc = (float *)(A3h + (size_t)M * K6h);
    ++c->launches;
    int kp = kp_begin(c);
    MIDAS_CUDA(c, cudaMemsetAsync(sc + 3, 0, sizeof(unsigned), c->stream));
    k_cabsmax<TA><<<std::min(M, 4096), 256, 0, c->stream>>>(M, K, A, ars, acs, (unsigned *)(sc + 3));
    k_h16_scale<<<1, 1, 0, c->stream>>>((const unsigned *)(sc + 3), sc, 0);
    k_split_a_h16<TA><<<dim3((K + 127) / 128, std::min(M, 65535)), 128, 0, c->stream>>>(M, K, A, ars, acs, sc, A3h,
                                                                                         K6h);
    kp_end(c, kp, MIDAS_KC_SPLIT, 0.0, (double)sizeof(TA) * M * K + 2.0 * M * K6h);
    MIDAS_CUDA(c, cudaGetLastError());
    return zgemm_x3h_a3<TB>(c, M, N, K, A3h, K6h, sc, B, brs, bcs, D, ldd, kclass, promote_kb);
}
template int zgemm_x3h<double2, float2>(midas_gpu_ctx *, int, int, int, const double2 *, long long, long long,
                                        const float2 *, long long, long long, float *, long long, int, int);

// sc[0] = s (a power of two) for a split written by a kernel that knew its scale
__global__ void k_set_scale(float *sc, float s) { sc[0] = s; }
int set_h16_scale(midas_gpu_ctx *c, float *sc, float s)
{
    ++c->launches;
    k_set_scale<<<1, 1, 0, c->stream>>>(sc, s);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// R[j * n + i] -= P[i][2j] + i P[i][2j + 1]   (P row-major n x 2m, FP32; R column-major FP64)
__global__ void k_sub_rowmajor(int n, int m, const float *P, double2 *R)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)n * m) return;
    const int i = (int)(t % n), j = (int)(t / n);
    const float2 p = *(const float2 *)(P + (long long)i * 2 * m + 2 * j);
    double2 r = R[t];
    r.x -= (double)p.x;
    r.y -= (double)p.y;
    R[t] = r;
}

// R -= Z D with Z given by its fp16 split A3h (n x n, scale in sc[0]) and D row-major
// n x m complex64: the FP32-grade product (hi*hi + hi*lo + lo*hi, relative error
// ~2^-22) on the tensor cores.  P (n x 2m floats) is scratch.
int resid_update_x3(midas_gpu_ctx *c, int n, int m, const __half *A3h, long long K6h, float *sc, const float2 *D,
                    float *P, double2 *R)
{
    // four-block chunks: the refinement's double-float residual checks the updates
    MIDAS_TRY(zgemm_x3h_a3<float2>(c, n, m, n, A3h, K6h, sc, D, m, 1, P, 2LL * m, MIDAS_KC_RESID32, 4));
    ++c->launches;
    int kp = kp_begin(c);
    const long long tot = (long long)n * m;
    k_sub_rowmajor<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(n, m, P, R);
    kp_end(c, kp, MIDAS_KC_RESID32, 2.0 * tot, 40.0 * tot);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
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
    int kp = kp_begin(c);
    k_zgemm64<<<grd, blk, 0, c->stream>>>(M, N, K, A, ars, acs, conjA, B, brs, bcs, C, crs, ccs, alpha, beta);
    kp_end(c, kp, MIDAS_KC_ZGEMM64, 8.0 * M * N * K, 16.0 * ((double)M * K + (double)K * N + 2.0 * M * N));
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// C = A B, complex, FP64 in and out (strided: A(i,k) at A[i*ars + k*acs], B(k,j)
// at B[k*brs + j*bcs], C(i,j) at C[i*crs + j*ccs]), computed in double float on
// the FP32 pipe: operands split into hi = fl32(x), lo = fl32(x - hi) as they are
// staged, products exact (FMA TwoProduct + cross terms), sums compensated
// (TwoSum) -- ~2^-48 relative, on a pipe 64x faster than GB300's FP64.  For the
// CBF construction C_b = X V Sigma^-1, Vc = C^T Einc and E = C alpha.  64 x 64
// output tiles, 4 x 4 per thread; the K range is split S ways when the tiles are
// too few to fill the GPU, the S partial (hi, lo) pairs summed in FP64.
// ---------------------------------------------------------------------------
constexpr int ZD_TK = 16, ZD_SMAX = 32;

__device__ __forceinline__ float4 zd_split(double2 v)
{
    float4 r;
    r.x = (float)v.x;
    r.y = (float)v.y;
    r.z = (float)(v.x - (double)r.x);
    r.w = (float)(v.y - (double)r.y);
    return r;
}

// one 64 x 64 tile of C (or of split partial sp in P) over k in [sp kchunk, (sp+1) kchunk)
__device__ __forceinline__ void zgemm_df_tile(int M, int N, int K, const double2 *__restrict__ A, long long ars,
                                              long long acs, const double2 *__restrict__ B, long long brs,
                                              long long bcs, double2 *C, long long crs, long long ccs, int kchunk,
                                              float4 *P, int i0, int j0, int sp)
{
    __shared__ float4 As[ZD_TK][64], Bs[ZD_TK][64];
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    const int kb = sp * kchunk, ke = min(K, kb + kchunk);
    float rh[4][4], rl[4][4], ih[4][4], il[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) rh[a][b] = rl[a][b] = ih[a][b] = il[a][b] = 0.f;
    for (int k0 = kb; k0 < ke; k0 += ZD_TK) {
        for (int e = tid; e < ZD_TK * 64; e += 256) {
            const int kk = e / 64, c = e % 64, k = k0 + kk;
            const int i = i0 + c, j = j0 + c;
            As[kk][c] = (k < ke && i < M) ? zd_split(A[(long long)i * ars + (long long)k * acs])
                                          : make_float4(0.f, 0.f, 0.f, 0.f);
            Bs[kk][c] = (k < ke && j < N) ? zd_split(B[(long long)k * brs + (long long)j * bcs])
                                          : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        __syncthreads();
#pragma unroll 1
        for (int kk = 0; kk < ZD_TK; ++kk) {
            float4 a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) a[u] = As[kk][ty + 16 * u];
#pragma unroll
            for (int u = 0; u < 4; ++u) b[u] = Bs[kk][tx + 16 * u];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    // re += ar br - ai bi, im += ar bi + ai br (hi = .x/.y, lo = .z/.w)
                    df_fma(rh[u][v], rl[u][v], a[u].x, b[v].x, a[u].z, b[v].z);
                    df_fma(rh[u][v], rl[u][v], -a[u].y, b[v].y, -a[u].w, b[v].w);
                    df_fma(ih[u][v], il[u][v], a[u].x, b[v].y, a[u].z, b[v].w);
                    df_fma(ih[u][v], il[u][v], a[u].y, b[v].x, a[u].w, b[v].z);
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int i = i0 + ty + 16 * u, j = j0 + tx + 16 * v;
            if (i >= M || j >= N) continue;
            if (P)
                P[((long long)sp * M + i) * N + j] = make_float4(rh[u][v], ih[u][v], rl[u][v], il[u][v]);
            else
                C[(long long)i * crs + (long long)j * ccs] =
                    make_double2((double)rh[u][v] + (double)rl[u][v], (double)ih[u][v] + (double)il[u][v]);
        }
}

__global__ void __launch_bounds__(256) k_zgemm_df(int M, int N, int K, const double2 *__restrict__ A, long long ars,
                                                   long long acs, const double2 *__restrict__ B, long long brs,
                                                   long long bcs, double2 *C, long long crs, long long ccs,
                                                   int kchunk, float4 *P)
{
    zgemm_df_tile(M, N, K, A, ars, acs, B, brs, bcs, C, crs, ccs, kchunk, P, blockIdx.y * 64, blockIdx.x * 64,
                  blockIdx.z);
}

// many independent products in one launch: blockIdx.z = job * nsplit + split part
__global__ void __launch_bounds__(256) k_zgemm_df_batched(const ZdfJob *__restrict__ jobs, int nsplit, float4 *P)
{
    const ZdfJob J = jobs[blockIdx.z / nsplit];
    const int i0 = blockIdx.y * 64, j0 = blockIdx.x * 64;
    if (i0 >= J.M || j0 >= J.N) return;   // the whole CTA: the job is smaller than the grid
    zgemm_df_tile(J.M, J.N, J.K, J.A, J.ars, J.acs, J.B, J.brs, J.bcs, J.C, J.crs, J.ccs, J.kchunk,
                  nsplit > 1 ? P + J.poff : nullptr, i0, j0, blockIdx.z % nsplit);
}

__global__ void k_zgemm_df_batched_reduce(const ZdfJob *__restrict__ jobs, int njobs, long long tot, int nsplit,
                                          const float4 *P)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
         e += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = njobs - 1;   // the job holding output e: the last with eoff <= e
        while (lo < hi) {
            const int mid = (lo + hi + 1) / 2;
            if (jobs[mid].eoff <= e) lo = mid; else hi = mid - 1;
        }
        const ZdfJob &J = jobs[lo];
        const long long q = e - J.eoff, mn = (long long)J.M * J.N;
        double re = 0, im = 0;
        for (int sp = 0; sp < nsplit; ++sp) {
            const float4 p = P[J.poff + sp * mn + q];
            re += (double)p.x + (double)p.z;
            im += (double)p.y + (double)p.w;
        }
        const int i = (int)(q / J.N), j = (int)(q % J.N);
        J.C[(long long)i * J.crs + (long long)j * J.ccs] = make_double2(re, im);
    }
}

__global__ void k_zgemm_df_reduce(int M, int N, int nsplit, const float4 *P, double2 *C, long long crs, long long ccs)
{
    const long long tot = (long long)M * N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
         e += (long long)gridDim.x * blockDim.x) {
        double re = 0, im = 0;
        for (int s = 0; s < nsplit; ++s) {
            const float4 p = P[(long long)s * tot + e];
            re += (double)p.x + (double)p.z;
            im += (double)p.y + (double)p.w;
        }
        const int i = (int)(e / N), j = (int)(e % N);
        C[(long long)i * crs + (long long)j * ccs] = make_double2(re, im);
    }
}

int zgemm_df(midas_gpu_ctx *c, int M, int N, int K, const double2 *A, long long ars, long long acs,
             const double2 *B, long long brs, long long bcs, double2 *C, long long crs, long long ccs)
{
    if (M <= 0 || N <= 0) return MIDAS_OK;
    if (K <= 0) return c->err.set(MIDAS_ERR_ARG, "zgemm_df: K must be positive");
    const long long tiles = (long long)((M + 63) / 64) * ((N + 63) / 64);
    int nsplit = (int)std::min<long long>(ZD_SMAX, std::max<long long>(1, 300 / tiles));
    nsplit = std::max(1, std::min(nsplit, K / 64));
    const int kchunk = ((K + nsplit - 1) / nsplit + ZD_TK - 1) / ZD_TK * ZD_TK;
    float4 *P = nullptr;
    if (nsplit > 1) {
        void *p;
        MIDAS_TRY(ensure(c, S_ZDF, sizeof(float4) * (size_t)nsplit * M * N + 256, &p));
        P = (float4 *)p;
    }
    ++c->launches;
    int kp = kp_begin(c);
    k_zgemm_df<<<dim3((N + 63) / 64, (M + 63) / 64, nsplit), 256, 0, c->stream>>>(M, N, K, A, ars, acs, B, brs, bcs,
                                                                                  C, crs, ccs, kchunk, P);
    if (nsplit > 1) {
        ++c->launches;
        const long long tot = (long long)M * N;
        k_zgemm_df_reduce<<<(unsigned)std::min<long long>((tot + 255) / 256, 4096), 256, 0, c->stream>>>(
            M, N, nsplit, P, C, crs, ccs);
    }
    kp_end(c, kp, MIDAS_KC_ZGEMM64, 8.0 * M * (double)N * K, 16.0 * ((double)M * K + (double)K * N + (double)M * N));
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

int zgemm_df_batched(midas_gpu_ctx *c, std::vector<ZdfJob> &jobs)
{
    const int nj = (int)jobs.size();
    if (nj == 0) return MIDAS_OK;
    long long tiles = 0;
    int mt = 0, nt = 0, kmax = 0;
    for (const ZdfJob &J : jobs) {
        if (J.M <= 0 || J.N <= 0 || J.K <= 0) return c->err.set(MIDAS_ERR_ARG, "zgemm_df_batched: empty job");
        tiles += (long long)((J.M + 63) / 64) * ((J.N + 63) / 64);
        mt = std::max(mt, (J.M + 63) / 64);
        nt = std::max(nt, (J.N + 63) / 64);
        kmax = std::max(kmax, J.K);
    }
    // split K while the tiles of all jobs together fill less than ~4 CTAs per SM (a job
    // with a short K leaves its trailing parts empty: they add zeros)
    int nsplit = (int)std::min<long long>(ZD_SMAX, std::max<long long>(1, 600 / tiles));
    nsplit = std::max(1, std::min(nsplit, kmax / 64));
    if ((long long)nj * nsplit > 65535) return c->err.set(MIDAS_ERR_ARG, "zgemm_df_batched: too many jobs");
    long long poff = 0, eoff = 0;
    for (ZdfJob &J : jobs) {
        J.kchunk = ((J.K + nsplit - 1) / nsplit + ZD_TK - 1) / ZD_TK * ZD_TK;
        J.poff = poff;
        J.eoff = eoff;
        poff += (long long)nsplit * J.M * J.N;
        eoff += (long long)J.M * J.N;
    }
    const size_t jb = (sizeof(ZdfJob) * nj + 255) / 256 * 256;
    void *p;
    MIDAS_TRY(ensure(c, S_ZDF, jb + (nsplit > 1 ? sizeof(float4) * (size_t)poff : 0) + 256, &p));
    ZdfJob *d_jobs = (ZdfJob *)p;
    float4 *P = (float4 *)((char *)p + jb);
    MIDAS_CUDA(c, cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(ZdfJob) * nj, cudaMemcpyHostToDevice, c->stream));
    double flops = 0, bytes = 0;
    for (const ZdfJob &J : jobs) {
        flops += 8.0 * J.M * (double)J.N * J.K;
        bytes += 16.0 * ((double)J.M * J.K + (double)J.K * J.N + (double)J.M * J.N);
    }
    ++c->launches;
    int kp = kp_begin(c);
    k_zgemm_df_batched<<<dim3(nt, mt, nj * nsplit), 256, 0, c->stream>>>(d_jobs, nsplit, P);
    if (nsplit > 1) {
        ++c->launches;
        k_zgemm_df_batched_reduce<<<(unsigned)std::min<long long>((eoff + 255) / 256, 4096), 256, 0, c->stream>>>(
            d_jobs, nj, eoff, nsplit, P);
    }
    kp_end(c, kp, MIDAS_KC_ZGEMM64, flops, bytes);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// Gram matrix G = X^H X (m x m, row-major FP64) of a block's CBF solutions in
// double float on the FP32 pipe (the FP64 pipe of GB300 runs at 1/64 of it).
// X = Xh + Xl (the refinement's own hi/lo copies), element (k, j) at
// X[k * rs + j * cs], k < K.  64 x 64 output tiles on the upper tile triangle,
// K split S ways (the m <= ~200 Gram has only a handful of tiles); every CTA
// writes its partial (hi, lo) pairs, and k_gram_reduce sums them in FP64 and
// mirrors the upper triangle, so G is exactly Hermitian.  The products are exact
// (FMA TwoProduct + cross terms) and the sums compensated: ~2^-48 relative, far
// below the 1e-11 to which the refinement determines X.
// ---------------------------------------------------------------------------
constexpr int GR_TK = 8, GR_SMAX = 24;   // 2 stages x (A + B) x 8 x 64 float4 = 32 KB static shared memory

__device__ __forceinline__ void gr_cp8(void *dst, const void *src, bool ok)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(sa), "l"(src), "r"(ok ? 8 : 0));
}

__global__ void __launch_bounds__(256) k_gram_df(int m, int K, const float2 *Xh, const float2 *Xl, long long rs,
                                                  long long cs, int kchunk, float4 *P)
{
    __shared__ __align__(16) float4 As[2][GR_TK][64], Bs[2][GR_TK][64];
    // tile pair (I, J), I <= J, from blockIdx.x; split from blockIdx.y
    const int nt = (m + 63) / 64;
    int t = blockIdx.x, I = 0;
    while (t >= nt - I) { t -= nt - I; ++I; }
    const int J = I + t, i0 = 64 * I, j0 = 64 * J, sp = blockIdx.y;
    const int kb = sp * kchunk, ke = min(K, kb + kchunk);
    const int nkt = ke > kb ? (ke - kb + GR_TK - 1) / GR_TK : 0;
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    auto load = [&](int st, int k0) {
        for (int e = tid; e < GR_TK * 64; e += 256) {
            const int kk = e / 64, c = e % 64, k = k0 + kk;
            const int ia = i0 + c, jb = j0 + c;
            const bool oka = k < ke && ia < m, okb = k < ke && jb < m;
            const long long oa = oka ? (long long)k * rs + (long long)ia * cs : 0;
            const long long ob = okb ? (long long)k * rs + (long long)jb * cs : 0;
            gr_cp8(&As[st][kk][c].x, Xh + oa, oka);
            gr_cp8(&As[st][kk][c].z, Xl + oa, oka);
            gr_cp8(&Bs[st][kk][c].x, Xh + ob, okb);
            gr_cp8(&Bs[st][kk][c].z, Xl + ob, okb);
        }
        asm volatile("cp.async.commit_group;\n" ::);
    };
    float rh[4][4], rl[4][4], ih[4][4], il[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) rh[a][b] = rl[a][b] = ih[a][b] = il[a][b] = 0.f;
    if (nkt > 0) load(0, kb);
    for (int q = 0; q < nkt; ++q) {
        if (q + 1 < nkt) {
            load((q + 1) & 1, kb + (q + 1) * GR_TK);
            asm volatile("cp.async.wait_group 1;\n" ::);
        } else {
            asm volatile("cp.async.wait_group 0;\n" ::);
        }
        __syncthreads();
        const int st = q & 1;
#pragma unroll 1
        for (int kk = 0; kk < GR_TK; ++kk) {
            float4 a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) a[u] = As[st][kk][tx + 16 * u];
#pragma unroll
            for (int u = 0; u < 4; ++u) b[u] = Bs[st][kk][ty + 16 * u];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    // conj(a) b: re = ar br + ai bi, im = ar bi - ai br (hi = .x/.y, lo = .z/.w)
                    df_fma(rh[u][v], rl[u][v], a[u].x, b[v].x, a[u].z, b[v].z);
                    df_fma(rh[u][v], rl[u][v], a[u].y, b[v].y, a[u].w, b[v].w);
                    df_fma(ih[u][v], il[u][v], a[u].x, b[v].y, a[u].z, b[v].w);
                    df_fma(ih[u][v], il[u][v], -a[u].y, b[v].x, -a[u].w, b[v].z);
                }
        }
        __syncthreads();   // stage st is refilled by the next iteration's prefetch
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int i = i0 + tx + 16 * u, j = j0 + ty + 16 * v;
            if (i < m && j < m) P[((long long)sp * m + i) * m + j] = make_float4(rh[u][v], ih[u][v], rl[u][v], il[u][v]);
        }
}

__global__ void k_gram_reduce(int m, int nsplit, const float4 *P, double2 *G)
{
    const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m || j < i) return;
    double re = 0, im = 0;
    for (int s = 0; s < nsplit; ++s) {
        const float4 p = P[((long long)s * m + i) * m + j];
        re += (double)p.x + (double)p.z;
        im += (double)p.y + (double)p.w;
    }
    if (i == j) im = 0;   // conj(x) x is real; the exact products cancel to 0 already
    G[(long long)i * m + j] = make_double2(re, im);
    G[(long long)j * m + i] = make_double2(re, -im);
}

size_t gram_df_scratch_bytes(int m) { return sizeof(float4) * (size_t)GR_SMAX * m * m + 256; }

int gram_df(midas_gpu_ctx *c, int m, int K, const float2 *Xh, const float2 *Xl, long long rs, long long cs,
            double2 *G, float4 *P)
{
    if (m <= 0) return MIDAS_OK;
    const int nt = (m + 63) / 64, npair = nt * (nt + 1) / 2;
    const int nsplit = std::max(1, std::min(GR_SMAX, K / 512));
    const int kchunk = (K + nsplit - 1) / nsplit;
    ++c->launches;
    int kp = kp_begin(c);
    k_gram_df<<<dim3(npair, nsplit), 256, 0, c->stream>>>(m, K, Xh, Xl, rs, cs, kchunk, P);
    kp_end(c, kp, MIDAS_KC_ZGEMM64, 8.0 * m * (double)m * K, 16.0 * (double)m * K + 16.0 * m * m);
    ++c->launches;
    k_gram_reduce<<<dim3((m + 127) / 128, m), 128, 0, c->stream>>>(m, nsplit, P, G);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// double-float residual: r = B - Z X,  Z (n x n row-major fp32, ldz), X = Xh + Xl
// (fp32 pairs, column-major ld = n), B fp32 column-major (ld n).  r is FP64.
// Tile: 32 rows x 32 rhs per CTA (256 threads, 4 outputs each).
// ---------------------------------------------------------------------------
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
    float arh[4], arl[4], aih[4], ail[4];
    float cr[4] = {0, 0, 0, 0}, ci[4] = {0, 0, 0, 0};   // lo-part products (plain fp32)
    for (int q = 0; q < 4; ++q) arh[q] = arl[q] = aih[q] = ail[q] = 0.f;
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
                df_fma(arh[q], arl[q], z.x, xh.x);
                df_fma(arh[q], arl[q], -z.y, xh.y);
                df_fma(aih[q], ail[q], z.x, xh.y);
                df_fma(aih[q], ail[q], z.y, xh.x);
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
        double zr = (double)arh[q] + (double)arl[q] + (double)cr[q];
        double zi = (double)aih[q] + (double)ail[q] + (double)ci[q];
        float2 b = B[(long long)col * n + row];
        R[(long long)col * n + row] = make_double2((double)b.x - zr, (double)b.y - zi);
    }
}

int residual_df32(midas_gpu_ctx *c, int n, int nrhs, const float2 *Z, long long ldz, const float2 *Xh,
                  const float2 *Xl, const float2 *B, double2 *R)
{
    dim3 grd((nrhs + 31) / 32, (n + 31) / 32);
    ++c->launches;
    int kp = kp_begin(c);
    k_residual_df32<<<grd, 256, 0, c->stream>>>(n, nrhs, Z, ldz, Xh, Xl, B, R);
    kp_end(c, kp, MIDAS_KC_RESID, 8.0 * n * n * nrhs, 8.0 * n * n + 32.0 * n * nrhs);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// Hermitian eigen-decomposition (FP64) in three kernels:
//  * k_heev_tridiag, one CTA per matrix: Householder tridiagonalisation (the
//    zhetd2 recurrence: H = I - tau v v^H, x = tau A v, w = x - tau/2 (x^H v) v,
//    A <- A - v w^H - w v^H) and the implicit-shift QL sweeps on the real
//    tridiagonal; one thread generates the Givens rotations of each sweep and
//    logs them, eigenvalues sorted by decreasing value;
//  * k_heev_rot: Z = (the logged rotations applied in order to I), rows of Z
//    split over CTAs (each row takes every rotation; rows are independent);
//  * k_heev_back: V = H_0 .. H_{m-2} Z, columns split over CTAs, written in the
//    sorted order.
// The FP64 pipe of GB300 is the limit (60 % busy in the single-CTA form), so
// the two O(m^3) phases that parallelise go to many SMs.  Backward stable:
// absolute errors ~ eps ||A||, so the CBF threshold subspace is resolved to
// eps ||A|| / gap.  A (m x m row-major, lda) is destroyed; H (m x m) holds the
// reflectors (tau_k on its diagonal); V (row-major m x m) the eigenvectors.
// ---------------------------------------------------------------------------
__device__ double block_sum_d(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    return s;
}

__global__ void __launch_bounds__(256) k_heev_tridiag(int m, double2 *Ab, long long lda, long long sa, double2 *Hb,
                                                      long long sv, double *Wb, int *posb, double2 *logb,
                                                      long long logcap, long long *logn, int *flag)
{
    extern __shared__ double shm[];
    double *d = shm, *e = d + m, *red = e + m;   // red: 32 doubles
    double2 *tau = (double2 *)(red + 32), *v = tau + m, *x = v + m;
    __shared__ double2 s_tau, s_scale;
    __shared__ double s_beta;
    double2 *A = Ab + blockIdx.x * sa;
    double2 *H = Hb + blockIdx.x * sv;
    double *W = Wb + (long long)blockIdx.x * m;
    int *pos = posb + (long long)blockIdx.x * m;
    double2 *lg = logb + blockIdx.x * logcap;   // per sweep: (mm, nrot), then nrot (s, c)
    const int tid = threadIdx.x, nt = blockDim.x;
    // ---- tridiagonalisation --------------------------------------------------
    for (int k = 0; k < m - 1; ++k) {
        const int L = m - k - 1;   // trailing size
        double xn2 = 0;
        for (int r = k + 2 + tid; r < m; r += nt) {
            double2 a = A[(long long)r * lda + k];
            xn2 += a.x * a.x + a.y * a.y;
        }
        xn2 = block_sum_d(xn2, red);
        if (tid == 0) {
            double2 al = A[(long long)(k + 1) * lda + k];
            if (xn2 == 0 && al.y == 0) {
                s_tau = make_double2(0, 0);
                s_beta = al.x;
            } else {
                double beta = -copysign(sqrt(al.x * al.x + al.y * al.y + xn2), al.x);
                s_tau = make_double2((beta - al.x) / beta, -al.y / beta);
                double2 dnm = make_double2(al.x - beta, al.y);   // 1/(alpha - beta)
                double q = dnm.x * dnm.x + dnm.y * dnm.y;
                s_scale = make_double2(dnm.x / q, -dnm.y / q);
                s_beta = beta;
            }
        }
        __syncthreads();
        const double2 t = s_tau;
        for (int i = tid; i < L; i += nt) {
            double2 vi;
            if (i == 0) vi = make_double2(1, 0);
            else {
                double2 a = A[(long long)(k + 1 + i) * lda + k];
                vi = make_double2(a.x * s_scale.x - a.y * s_scale.y, a.x * s_scale.y + a.y * s_scale.x);
            }
            v[i] = vi;
            H[(long long)(k + 1 + i) * m + k] = vi;
        }
        if (tid == 0) { tau[k] = t; H[(long long)k * m + k] = t; }
        __syncthreads();
        if (t.x != 0 || t.y != 0) {
            // x = tau * A22 v, a warp per row (the lanes read the row coalesced)
            for (int i = tid / 32; i < L; i += nt / 32) {
                const double2 *row = A + (long long)(k + 1 + i) * lda + (k + 1);
                double sx = 0, sy = 0;
                for (int j = tid % 32; j < L; j += 32) {
                    double2 a = row[j], vj = v[j];
                    sx += a.x * vj.x - a.y * vj.y;
                    sy += a.x * vj.y + a.y * vj.x;
                }
                for (int o = 16; o > 0; o >>= 1) {
                    sx += __shfl_down_sync(0xffffffffu, sx, o);
                    sy += __shfl_down_sync(0xffffffffu, sy, o);
                }
                if (tid % 32 == 0) x[i] = make_double2(t.x * sx - t.y * sy, t.x * sy + t.y * sx);
            }
            __syncthreads();
            // dot = x^H v ; alpha = -1/2 tau dot ; w = x + alpha v  (w stored in x)
            double pr = 0, pi = 0;
            for (int i = tid; i < L; i += nt) {
                double2 a = x[i], b = v[i];
                pr += a.x * b.x + a.y * b.y;
                pi += a.x * b.y - a.y * b.x;
            }
            pr = block_sum_d(pr, red);
            pi = block_sum_d(pi, red);
            double2 al = make_double2(-0.5 * (t.x * pr - t.y * pi), -0.5 * (t.x * pi + t.y * pr));
            __syncthreads();
            for (int i = tid; i < L; i += nt) {
                double2 b = v[i];
                x[i] = make_double2(x[i].x + al.x * b.x - al.y * b.y, x[i].y + al.x * b.y + al.y * b.x);
            }
            __syncthreads();
            // A22 -= v w^H + w v^H (a warp per row, the lanes along it)
            for (int i = tid / 32; i < L; i += nt / 32) {
                const double2 vi = v[i], wi = x[i];
                double2 *row = A + (long long)(k + 1 + i) * lda + (k + 1);
                for (int j = tid % 32; j < L; j += 32) {
                    const double2 vj = v[j], wj = x[j];
                    double2 *a = row + j;
                    a->x -= (vi.x * wj.x + vi.y * wj.y) + (wi.x * vj.x + wi.y * vj.y);
                    a->y -= (vi.y * wj.x - vi.x * wj.y) + (wi.y * vj.x - wi.x * vj.y);
                }
            }
        }
        if (tid == 0) {
            e[k] = s_beta;
            d[k] = A[(long long)k * lda + k].x;
        }
        __syncthreads();
    }
    if (tid == 0) { d[m - 1] = A[(long long)(m - 1) * lda + (m - 1)].x; e[m - 1] = 0; }
    if (tid == 0) H[(long long)(m - 1) * m + (m - 1)] = make_double2(0, 0);   // no reflector k = m - 1
    __syncthreads();
    // ---- implicit QL on (d, e), warp 0 ------------------------------------------
    // deflation: |e| <= eps (|d_i| + |d_i+1|), or |e| <= eps ||T|| -- eigenvalues at the
    // roundoff level of a rank-deficient Gram matrix never pass the relative test alone.
    // The lanes test 32 off-diagonals at a time for the split point; lane 0 runs each
    // sweep (the rotation chain is serial) with the next rotation's d and e loaded ahead,
    // and logs the rotations straight to global memory.
    const double eps = 2.220446049250313e-16;
    if (tid < 32) {
        const int lane = tid;
        double tn = 0;
        for (int i = lane; i < m; i += 32) tn = fmax(tn, fabs(d[i]) + fabs(e[i]) + (i > 0 ? fabs(e[i - 1]) : 0.0));
        for (int o = 16; o > 0; o >>= 1) tn = fmax(tn, __shfl_xor_sync(0xffffffffu, tn, o));
        const double tnorm = tn;
        long long lp = 0;   // log length (the same in every lane)
        bool fail = false;
        for (int l = 0; l < m && !fail; ++l) {
            for (int iter = 0;; ++iter) {
                int mm = -1;   // first split point at or after l (m - 1 at the latest)
                for (int base = l; mm < 0; base += 32) {
                    const int q = base + lane;
                    bool split = true;
                    if (q < m - 1) {
                        const double eq = fabs(e[q]);
                        split = eq <= eps * (fabs(d[q]) + fabs(d[q + 1])) || eq <= eps * tnorm;
                    }
                    const unsigned bal = __ballot_sync(0xffffffffu, split);
                    if (bal) mm = base + __ffs(bal) - 1;
                }
                if (mm == l) break;
                if (iter >= 200 || lp + 1 + (mm - l) > logcap) {
                    // no convergence, or the rotation log is full (not expected: ~1.5 m^2 rotations)
                    if (lane == 0) atomicOr(flag, DEV_BAD_ARG);
                    fail = true;
                    break;
                }
                int cnt = 0;
                if (lane == 0) {
                    double2 *out = lg + lp + 1;   // per sweep: (mm, nrot), then nrot (s, c)
                    double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
                    const double r0 = sqrt(g * g + 1.0);
                    g = d[mm] - d[l] + e[l] / (g + copysign(r0, g));
                    double s = 1, c = 1, p = 0;
                    double ei = e[mm - 1], di = d[mm - 1], dh = d[mm];   // e[i], d[i], d[i+1] (not yet updated)
                    bool broke = false;
                    for (int i = mm - 1; i >= l; --i) {
                        const double en = i > l ? e[i - 1] : 0.0, dn = i > l ? d[i - 1] : 0.0;
                        const double f = s * ei, b = c * ei;
                        // r = sqrt(f^2 + g^2) and 1 / r: the FP32 reciprocal square root refined by
                        // two Newton-Raphson steps y <- y (3/2 - q y^2 / 2) in FP64 (error ~1 ulp),
                        // a shorter dependent chain than an FP64 square root and divide.  |g| is
                        // bounded by ~||T|| / eps after the deflation test, so q cannot overflow.
                        const double q2 = f * f + g * g;
                        if (q2 == 0.0) { e[i + 1] = 0.0; d[i + 1] = dh - p; broke = true; break; }
                        const float qf = (float)q2;
                        double ir = (qf > 1e-37f && qf < 1e37f) ? (double)rsqrtf(qf) : 1.0 / sqrt(q2);
                        const double hq = 0.5 * q2;
                        ir = ir * (1.5 - hq * ir * ir);
                        ir = ir * (1.5 - hq * ir * ir);
                        e[i + 1] = q2 * ir;
                        s = f * ir;
                        c = g * ir;
                        g = dh - p;
                        const double r = (di - g) * s + 2.0 * c * b;
                        p = s * r;
                        d[i + 1] = g + p;
                        g = c * r - b;
                        out[cnt++] = make_double2(s, c);
                        ei = en; dh = di; di = dn;
                    }
                    if (!broke) { d[l] -= p; e[l] = g; }
                    e[mm] = 0.0;
                    if (cnt > 0) lg[lp] = make_double2((double)mm, (double)cnt);
                }
                __syncwarp();
                cnt = __shfl_sync(0xffffffffu, cnt, 0);
                if (cnt > 0) lp += 1 + cnt;
            }
        }
        if (lane == 0) logn[blockIdx.x] = fail ? 0 : lp;
    }
    __syncthreads();
    // ---- sort (descending): each eigenvalue's rank, ties in index order ------------
    for (int i = tid; i < m; i += nt) {
        const double di = d[i];
        if (!(di == di)) atomicOr(flag, DEV_BAD_ARG);   // NaN
        int rank = 0;
        for (int j = 0; j < m; ++j) {
            const double dj = d[j];
            rank += (dj > di) || (dj == di && j < i);
        }
        W[rank] = di;
        pos[i] = rank;   // eigenvector i goes to column pos[i]
    }
}

// Z = R_N ... R_1 I for the logged rotations, rows of Z split over CTAs (thread
// per row).  Z is real, column-major (m x m per matrix in its own buffer), so
// the threads' accesses to one column coalesce.  Within a sweep, rotation q
// mixes z[i] and z[i+1] (i = mm-1-q) and its new z[i] is the next rotation's
// z[i+1]: it stays in a register.
__global__ void k_heev_rot(int m, double *Zb, const double2 *logb, long long logcap, const long long *logn)
{
    const int r = blockIdx.y * blockDim.x + threadIdx.x;
    if (r >= m) return;
    double *Z = Zb + (long long)blockIdx.x * m * m;
    const double2 *lg = logb + blockIdx.x * logcap;
    for (int col = 0; col < m; ++col) Z[(long long)col * m + r] = col == r ? 1.0 : 0.0;
    const long long n = logn[blockIdx.x];
    for (long long lp = 0; lp < n;) {
        const double2 h = lg[lp];
        const int mm = (int)h.x, nrot = (int)h.y;
        double f = Z[(long long)mm * m + r];
        for (int q = 0; q < nrot; ++q) {
            const int i = mm - 1 - q;
            const double2 sc = lg[lp + 1 + q];
            const double zi = Z[(long long)i * m + r];
            Z[(long long)(i + 1) * m + r] = sc.x * zi + sc.y * f;
            f = sc.y * zi - sc.x * f;
        }
        Z[(long long)(mm - nrot) * m + r] = f;
        lp += 1 + nrot;
    }
}

// V = H_0 H_1 ... H_{m-2} Z: a CTA takes CB columns of Z into shared memory
// (complex), applies the reflectors from k = m-2 down to 0 -- column j gets
// w = tau (v^H z_j), z_j -= v w, each column's sum split over P = 256 / CB
// threads and met by shuffles -- and writes the columns to their sorted places.
__global__ void __launch_bounds__(256) k_heev_back(int m, int cb, const double2 *Hb, const double *Zb, double2 *Vb,
                                                   long long sv, const int *posb)
{
    extern __shared__ double2 hb_sm[];
    double2 *Zs = hb_sm;                        // [m][cb]
    double2 *vk = hb_sm + (size_t)m * cb;       // [m] current reflector
    const double2 *H = Hb + blockIdx.x * sv;
    double2 *V = Vb + blockIdx.x * sv;
    const double *Z = Zb + (long long)blockIdx.x * m * m;   // column-major real, from k_heev_rot
    const int *pos = posb + (long long)blockIdx.x * m;
    const int j0 = blockIdx.y * cb, ncol = min(cb, m - j0);
    const int P = blockDim.x / cb, tid = threadIdx.x, jj = tid / P, part = tid % P;
    for (int q = tid; q < m * cb; q += blockDim.x) {
        const int jc = q / m, r = q % m;        // consecutive threads: consecutive rows of one column
        Zs[(size_t)r * cb + jc] = make_double2(jc < ncol ? Z[(long long)(j0 + jc) * m + r] : 0.0, 0.0);
    }
    __syncthreads();
    for (int k = m - 2; k >= 0; --k) {
        const double2 t = H[(long long)k * m + k];
        if (t.x == 0 && t.y == 0) continue;
        const int L = m - k - 1;
        for (int r = tid; r < L; r += blockDim.x) vk[r] = H[(long long)(k + 1 + r) * m + k];
        __syncthreads();
        double wr = 0, wi = 0;   // w_j = sum_r conj(v_r) Z[k+1+r][j]
        for (int r = part; r < L; r += P) {
            const double2 vr = vk[r], z = Zs[(size_t)(k + 1 + r) * cb + jj];
            wr += vr.x * z.x + vr.y * z.y;
            wi += vr.x * z.y - vr.y * z.x;
        }
        for (int o = P / 2; o > 0; o >>= 1) {
            wr += __shfl_xor_sync(0xffffffffu, wr, o);
            wi += __shfl_xor_sync(0xffffffffu, wi, o);
        }
        const double2 tw = make_double2(t.x * wr - t.y * wi, t.x * wi + t.y * wr);
        for (int r = part; r < L; r += P) {
            const double2 vr = vk[r];
            double2 *z = Zs + (size_t)(k + 1 + r) * cb + jj;
            z->x -= vr.x * tw.x - vr.y * tw.y;
            z->y -= vr.x * tw.y + vr.y * tw.x;
        }
        __syncthreads();   // vk is reloaded for the next reflector
    }
    for (int q = tid; q < m * cb; q += blockDim.x) {
        const int r = q / cb, jc = q % cb;
        if (jc < ncol) V[(long long)r * m + pos[j0 + jc]] = Zs[(size_t)r * cb + jc];
    }
}

int heev_dev(midas_gpu_ctx *c, int batch, int m, double2 *A, long long lda, long long sa, double2 *H, double2 *V,
             long long sv, double *W)
{
    if (m > 1024) return c->err.set(MIDAS_ERR_ARG, "heev: m > 1024");
    // scratch: rotation log (16 m^2 + m entries per matrix; QL takes ~1.5 m^2),
    // log lengths, sort positions, Z (m x m real per matrix)
    const long long logcap = 16LL * m * m + m;
    const size_t need = sizeof(double2) * (size_t)batch * logcap + sizeof(long long) * batch +
                        sizeof(int) * (size_t)batch * m + sizeof(double) * (size_t)batch * m * m + 4 * 256;
    void *p;
    MIDAS_TRY(ensure(c, S_HEEV, need, &p));
    size_t off = 0;
    auto take = [&](size_t bytes) {
        off = (off + 255) & ~(size_t)255;
        char *q = (char *)p + off;
        off += bytes;
        return q;
    };
    double2 *lg = (double2 *)take(sizeof(double2) * (size_t)batch * logcap);
    long long *logn = (long long *)take(sizeof(long long) * batch);
    int *pos = (int *)take(sizeof(int) * (size_t)batch * m);
    double *Z = (double *)take(sizeof(double) * (size_t)batch * m * m);
    size_t sm = sizeof(double) * (2 * (size_t)m + 32) + sizeof(double2) * 3 * (size_t)m;
    int cb = 32;   // columns per back-transformation CTA: Z columns [m][cb] + the reflector [m]
    while (cb > 8 && sizeof(double2) * (size_t)m * (cb + 1) > 200 * 1024) cb /= 2;
    const size_t smb = sizeof(double2) * (size_t)m * (cb + 1);
    MIDAS_CUDA(c, cudaFuncSetAttribute(k_heev_back, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smb));
    c->launches += 3;
    int kp = kp_begin(c);
    k_heev_tridiag<<<batch, 256, sm, c->stream>>>(m, A, lda, sa, H, sv, W, pos, lg, logcap, logn, c->d_flag);
    k_heev_rot<<<dim3(batch, (m + 31) / 32), 32, 0, c->stream>>>(m, Z, lg, logcap, logn);   // a warp per CTA: more SMs
    k_heev_back<<<dim3(batch, (m + cb - 1) / cb), 256, smb, c->stream>>>(m, cb, H, Z, V, sv, pos);
    kp_end(c, kp, MIDAS_KC_EIG, 0.0, 0.0);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

}  // namespace midas
