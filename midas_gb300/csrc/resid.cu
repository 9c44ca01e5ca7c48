// resid.cu -- refinement residuals of the dense mixed-precision solve (sm_103a).
//
// The dense solve (ir_solve) factors a complex64 copy of Z on the TF32 tensor
// cores and refines x against the FP64 matrix, the precision the reference's
// ScaLAPACK/LAPACK solve works in (src/Compute_EFields.f90:145-176,
// PZGESV/ZGESV).  GB300 issues FP64 at ~1/64 of its FP32 rate, so a refinement
// residual b - Z x over the FP64 matrix is FP64-pipe bound (8 n^2 nrhs flops,
// ~2.5 s for n = 60,000 and 64 right-hand sides).  Here the residuals run on
// the FP32 cores instead:
//
//  * z_split: Z64 is rewritten in place as double-float pairs, each complex
//    element (re, im) -> float4 (hi.re, hi.im, lo.re, lo.im) with
//    hi = fl32(z), lo = fl32(z - hi) (hi + lo = z to ~2^-48), in the same
//    16 bytes; the pass also returns ||Z||_inf (FP32 magnitudes; it only scales
//    the backward error).
//  * resid_dense<DF = true>: r = base - (Zh + Zl)(Xh + Xl) with every product
//    formed exactly (FMA TwoProduct + cross terms) and summed by TwoSum into a
//    (hi, lo) pair per output: an FP64-grade residual at ~48 FP32 operations
//    per complex multiply-add.
//  * resid_dense<DF = false>: r = base - Zh X in plain FP32 (4 FMA per complex
//    multiply-add), used where a relative error of ~1e-7 of the product is
//    enough: the first residual (x0 from the TF32 factors is ~1e-4 off) and the
//    updates r -= Z d once the corrections d are below 1e-5 of x.
//
// Both are register-tiled SIMT GEMMs: a CTA of 256 threads owns TM rows x TN
// right-hand sides (4 x 4 complex outputs per thread), stages Z (TM x TK) and
// X (TK x TN) tiles into shared memory with a 3-deep cp.async pipeline, and the
// K range is split S ways so that the grid covers the 152 SMs in several waves.
// Each split writes its partial sums; resid_reduce adds them in FP64, forms
// r = base - sum, the complex64 copy the next triangular solve reads and the
// per-column max |r|.
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace midas {

namespace {

constexpr int RD_THREADS = 256, RD_STAGES = 3, RD_SMAX = 8;

template <bool DF>
struct RdElem;
template <>
struct RdElem<true> {
    using T = float4;
};
template <>
struct RdElem<false> {
    using T = float2;
};

// TN right-hand sides per CTA (16 or 64); 4 x 4 outputs per thread.
template <int TN>
struct RdShape {
    static constexpr int TY = TN / 4, TX = RD_THREADS / TY, TM = 4 * TX, TK = 1024 / TM, ZLD = TM + 1;
};

__device__ __forceinline__ uint32_t rd_smem(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

template <int BYTES>
__device__ __forceinline__ void rd_cp_async(void *dst, const void *src)
{
    if constexpr (BYTES == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(rd_smem(dst)), "l"(src));
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(rd_smem(dst)), "l"(src));
}
__device__ __forceinline__ void rd_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void rd_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

template <bool DF, int TN>
constexpr size_t rd_smem_bytes()
{
    using S = RdShape<TN>;
    return sizeof(typename RdElem<DF>::T) * (size_t)RD_STAGES * S::TK * (S::ZLD + TN);
}

// Z: n x n double-float pairs (float4 per complex element, row-major, ldz);
// X: n x ldx operand rows (k-major, RHS fastest), zero beyond nrhs;
// P: S partial results, P[(s * ldx + j) * n + i].
// Requires n % 64 == 0 and kchunk % 64 == 0 (the host pads the system to 64).
template <bool DF, int TN>
__global__ void __launch_bounds__(RD_THREADS, 2)
    k_resid_dense(int n, const float4 *__restrict__ Z, long long ldz, const typename RdElem<DF>::T *__restrict__ X,
                  int ldx, int kchunk, typename RdElem<DF>::T *__restrict__ P)
{
    using S = RdShape<TN>;
    using V = typename RdElem<DF>::T;
    constexpr int TM = S::TM, TK = S::TK, TX = S::TX, TY = S::TY, ZLD = S::ZLD;
    extern __shared__ __align__(16) unsigned char rd_sm[];
    V *Zs = (V *)rd_sm;                              // [stage][TK][ZLD]
    V *Xs = Zs + (size_t)RD_STAGES * TK * ZLD;       // [stage][TK][TN]
    const int tid = threadIdx.x, tx = tid % TX, ty = tid / TX;
    const int r0 = blockIdx.x * TM, c0 = blockIdx.y * TN, sp = blockIdx.z;
    const int kb = sp * kchunk, ke = min(n, kb + kchunk);
    const int nkt = ke > kb ? (ke - kb) / TK : 0;

    auto load = [&](int st, int k0) {
        V *zs = Zs + (size_t)st * TK * ZLD;
#pragma unroll
        for (int q = 0; q < TM * TK / RD_THREADS; ++q) {
            const int e = tid + RD_THREADS * q, row = e / TK, kk = e % TK;
            const int gr = min(r0 + row, n - 1);   // rows past n (TM = 256 tiles) load a valid row, results dropped
            const float4 *src = Z + (long long)gr * ldz + k0 + kk;
            rd_cp_async<sizeof(V)>(zs + kk * ZLD + row, src);   // the hi pair is the first 8 bytes
        }
        V *xs = Xs + (size_t)st * TK * TN;
        for (int e = tid; e < TK * TN; e += RD_THREADS) {
            const int kk = e / TN, j = e % TN;
            rd_cp_async<sizeof(V)>(xs + e, X + (long long)(k0 + kk) * ldx + c0 + j);
        }
    };

    float ah[4][4], bh[4][4];
    // double-float: the low parts; FP32: this k-tile's sums, added to (ah, bh) once
    // per tile, so the rounding-error bound is ~(2 TK + K / TK) u instead of 2 K u
    float al[4][4], bl[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) ah[i][j] = bh[i][j] = al[i][j] = bl[i][j] = 0.f;

#pragma unroll
    for (int t = 0; t < RD_STAGES - 1; ++t) {
        if (t < nkt) load(t, kb + t * TK);
        rd_commit();
    }
    for (int t = 0; t < nkt; ++t) {
        rd_wait<RD_STAGES - 2>();
        __syncthreads();   // tile t landed for every thread; stage (t - 1) % STAGES is free again
        const int tn = t + RD_STAGES - 1;
        if (tn < nkt) load(tn % RD_STAGES, kb + tn * TK);
        rd_commit();
        const V *zs = Zs + (size_t)(t % RD_STAGES) * TK * ZLD;
        const V *xs = Xs + (size_t)(t % RD_STAGES) * TK * TN;
        if constexpr (!DF) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) al[i][j] = bl[i][j] = 0.f;
        }
        // the 4 x 4 micro-tile is unrolled; the k loop is not (fully unrolled, the
        // double-float body is ~12k instructions and the kernel stalls on
        // instruction fetch)
#pragma unroll(DF ? 1 : 4)
        for (int kk = 0; kk < TK; ++kk) {
            V z[4], x[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) z[i] = zs[kk * ZLD + tx + TX * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) x[j] = xs[kk * TN + ty + TY * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if constexpr (DF) {
                        // re += zr xr - zi xi ; im += zr xi + zi xr  (hi = .x/.y, lo = .z/.w)
                        df_fma(ah[i][j], al[i][j], z[i].x, x[j].x, z[i].z, x[j].z);
                        df_fma(ah[i][j], al[i][j], -z[i].y, x[j].y, -z[i].w, x[j].w);
                        df_fma(bh[i][j], bl[i][j], z[i].x, x[j].y, z[i].z, x[j].w);
                        df_fma(bh[i][j], bl[i][j], z[i].y, x[j].x, z[i].w, x[j].z);
                    } else {
                        al[i][j] = fmaf(z[i].x, x[j].x, fmaf(-z[i].y, x[j].y, al[i][j]));
                        bl[i][j] = fmaf(z[i].x, x[j].y, fmaf(z[i].y, x[j].x, bl[i][j]));
                    }
                }
        }
        if constexpr (!DF) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    ah[i][j] += al[i][j];
                    bh[i][j] += bl[i][j];
                }
        }
    }
    rd_wait<0>();
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const long long col = (long long)sp * ldx + c0 + ty + TY * j;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int row = r0 + tx + TX * i;
            if (row >= n) continue;
            V v;
            if constexpr (DF)
                v = make_float4(ah[i][j], bh[i][j], al[i][j], bl[i][j]);
            else
                v = make_float2(ah[i][j], bh[i][j]);
            P[col * n + row] = v;
        }
    }
}

// r = base - sum_s P_s (FP64), r32 = fl32(r), rmax[j] = max_i max(|Re r|, |Im r|).
// base may alias r (an update r -= Z d).
template <bool DF>
__global__ void k_resid_reduce(int n, int nrhs, int ldx, int nsplit, const typename RdElem<DF>::T *__restrict__ P,
                               const double2 *base, double2 *r, float2 *__restrict__ r32,
                               unsigned long long *__restrict__ rmax)
{
    const long long tot = (long long)n * nrhs;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
         e += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(e / n), i = (int)(e % n);
        double tr = 0, ti = 0;
        for (int s = 0; s < nsplit; ++s) {
            const auto p = P[((long long)s * ldx + j) * n + i];
            if constexpr (DF) {
                tr += (double)p.x + (double)p.z;
                ti += (double)p.y + (double)p.w;
            } else {
                tr += (double)p.x;
                ti += (double)p.y;
            }
        }
        const double2 b = base[e];
        const double2 rr = make_double2(b.x - tr, b.y - ti);
        r[e] = rr;
        r32[e] = make_float2((float)rr.x, (float)rr.y);
        double m = fmax(fabs(rr.x), fabs(rr.y));
        // n % 64 == 0: the 32 lanes of a warp share one column j
        for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31) == 0) atomicMax(rmax + j, (unsigned long long)__double_as_longlong(m));
    }
}

// X operand rows (k-major): double-float split of x (cm, ld n) or fl32 copy of d.
__global__ void k_xop_df(int n, int nrhs, int ldx, const double2 *__restrict__ x, float4 *__restrict__ X)
{
    const long long tot = (long long)n * ldx;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
         e += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(e / ldx), j = (int)(e % ldx);
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (j < nrhs) {
            const double2 a = x[(long long)j * n + k];
            v.x = (float)a.x;
            v.y = (float)a.y;
            v.z = (float)(a.x - (double)v.x);
            v.w = (float)(a.y - (double)v.y);
        }
        X[e] = v;
    }
}

__global__ void k_xop_f32(int n, int nrhs, int ldx, const float2 *__restrict__ d, float2 *__restrict__ X)
{
    const long long tot = (long long)n * ldx;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
         e += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(e / ldx), j = (int)(e % ldx);
        X[e] = j < nrhs ? d[(long long)j * n + k] : make_float2(0.f, 0.f);
    }
}

// In-place split of the FP64 matrix (row-major, ldz complex elements) into
// float4 double-float pairs; atomicMax of the row sums of |z| (FP32, >= 0, so
// the bit pattern orders like the value).
__global__ void __launch_bounds__(256) k_z_split(int n, long long ldz, double2 *Z, unsigned *znorm)
{
    __shared__ float red[8];
    for (int row = blockIdx.x; row < n; row += gridDim.x) {
        double2 *zr = Z + (long long)row * ldz;
        float s = 0.f;
        for (int m = threadIdx.x; m < n; m += blockDim.x) {
            const double2 a = zr[m];
            float4 v;
            v.x = (float)a.x;
            v.y = (float)a.y;
            v.z = (float)(a.x - (double)v.x);
            v.w = (float)(a.y - (double)v.y);
            reinterpret_cast<float4 *>(zr)[m] = v;
            s += hypotf(v.x, v.y);
        }
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            float t = 0.f;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
            atomicMax(znorm, __float_as_uint(t));
        }
        __syncthreads();
    }
}

int sm_count(midas_gpu_ctx *c) { return device_sms(c); }

int rd_ldx(int nrhs) { return nrhs <= 16 ? 16 : (nrhs + 63) / 64 * 64; }

int rd_splits(midas_gpu_ctx *c, int n, int nrhs)
{
    const int tn = nrhs <= 16 ? 16 : 64, tm = 4096 / tn;
    const long long tiles = (long long)((n + tm - 1) / tm) * (rd_ldx(nrhs) / tn);
    const long long want = 16LL * sm_count(c);   // ~8 waves at 2 CTAs per SM
    int s = (int)std::min<long long>(RD_SMAX, (want + tiles - 1) / tiles);
    return std::max(1, std::min(s, n / 256));
}

template <bool DF, int TN>
int launch_resid(midas_gpu_ctx *c, int n, int nrhs, const float4 *Z, long long ldz, const void *X, int ldx,
                 int nsplit, void *P)
{
    using S = RdShape<TN>;
    using V = typename RdElem<DF>::T;
    constexpr size_t smem = rd_smem_bytes<DF, TN>();
    static_assert(smem <= 110 * 1024, "two CTAs per SM");
    MIDAS_CUDA(c, cudaFuncSetAttribute(k_resid_dense<DF, TN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    const int kchunk = ((n + nsplit - 1) / nsplit + 63) / 64 * 64;
    dim3 grid((n + S::TM - 1) / S::TM, ldx / TN, nsplit);
    ++c->launches;
    k_resid_dense<DF, TN><<<grid, RD_THREADS, smem, c->stream>>>(n, Z, ldz, (const V *)X, ldx, kchunk, (V *)P);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

}  // namespace

double resid_update_error_factor(midas_gpu_ctx *c, int n, int nrhs)
{
    const int nsplit = rd_splits(c, n, nrhs);
    const int kchunk = ((n + nsplit - 1) / nsplit + 63) / 64 * 64;
    const int tk = nrhs <= 16 ? RdShape<16>::TK : RdShape<64>::TK;
    // FMA chains of 2 TK real products per tile (re: zr xr - zi xi), the FP32 sum of
    // the kchunk / TK tile sums, the dropped Zl d (u), the FP64 sum of the splits (< u)
    return (2 * tk + kchunk / tk + 2) * 0x1p-24;
}

size_t resid_scratch_bytes(int n, int nrhs)
{
    const size_t ldx = (size_t)rd_ldx(nrhs);
    const size_t smax = (size_t)std::max(1, std::min(RD_SMAX, n / 256));   // rd_splits never exceeds this
    return sizeof(float4) * ldx * n * (1 + smax) + 256;
}

int z_split_inplace(midas_gpu_ctx *c, double2 *Z64, long long ldz, int n, double *znorm)
{
    void *p;
    MIDAS_TRY(ensure(c, S_RED, 64, &p));
    unsigned *d = (unsigned *)p;
    MIDAS_CUDA(c, cudaMemsetAsync(d, 0, sizeof(unsigned), c->stream));
    ++c->launches;
    int kp = kp_begin(c);
    k_z_split<<<std::min(n, 8 * sm_count(c)), 256, 0, c->stream>>>(n, ldz, Z64, d);
    kp_end(c, kp, MIDAS_KC_OTHER, 0.0, 32.0 * n * (double)n);
    MIDAS_CUDA(c, cudaGetLastError());
    unsigned h = 0;
    MIDAS_CUDA(c, cudaMemcpyAsync(&h, d, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    float f;
    memcpy(&f, &h, 4);
    *znorm = f;
    return MIDAS_OK;
}

int resid_dense(midas_gpu_ctx *c, int n, int nrhs, const float4 *Zs, long long ldz, bool df, const double2 *x,
                const float2 *d, const double2 *base, double2 *r, float2 *r32, unsigned long long *rmax)
{
    if (n % 64 != 0 || nrhs <= 0) return c->err.set(MIDAS_ERR_ARG, "resid_dense: n must be a multiple of 64");
    const int ldx = rd_ldx(nrhs), nsplit = rd_splits(c, n, nrhs);
    void *p;
    MIDAS_TRY(ensure(c, S_RPART, resid_scratch_bytes(n, nrhs), &p));
    float4 *X = (float4 *)p;
    void *P = X + (size_t)ldx * n;
    const long long tot = (long long)n * ldx;
    const unsigned g = (unsigned)std::min<long long>((tot + 255) / 256, 8LL * sm_count(c));
    ++c->launches;
    if (df)
        k_xop_df<<<g, 256, 0, c->stream>>>(n, nrhs, ldx, x, X);
    else
        k_xop_f32<<<g, 256, 0, c->stream>>>(n, nrhs, ldx, d, (float2 *)X);
    MIDAS_CUDA(c, cudaGetLastError());
    int kp = kp_begin(c);
    const double fl = 8.0 * n * (double)n * nrhs, by = (df ? 16.0 : 8.0) * n * (double)n;
    if (nrhs <= 16)
        MIDAS_TRY(df ? launch_resid<true, 16>(c, n, nrhs, Zs, ldz, X, ldx, nsplit, P)
                     : launch_resid<false, 16>(c, n, nrhs, Zs, ldz, X, ldx, nsplit, P));
    else
        MIDAS_TRY(df ? launch_resid<true, 64>(c, n, nrhs, Zs, ldz, X, ldx, nsplit, P)
                     : launch_resid<false, 64>(c, n, nrhs, Zs, ldz, X, ldx, nsplit, P));
    kp_end(c, kp, MIDAS_KC_RESID, fl, by);
    const long long tr = (long long)n * nrhs;
    const unsigned gr = (unsigned)std::min<long long>((tr + 255) / 256, 8LL * sm_count(c));
    ++c->launches;
    if (df)
        k_resid_reduce<true><<<gr, 256, 0, c->stream>>>(n, nrhs, ldx, nsplit, (const float4 *)P, base, r, r32, rmax);
    else
        k_resid_reduce<false><<<gr, 256, 0, c->stream>>>(n, nrhs, ldx, nsplit, (const float2 *)P, base, r, r32,
                                                          rmax);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

}  // namespace midas
