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
//
// The trailing update (the dominant GEMM) reads FP16 copies of its L and U
// panels: every final L / U entry is stored rounded to TF32 (11-bit
// significand), which FP16 holds exactly once the panel is scaled by a power of
// two that puts its largest entry in [2^14, 2^15).  kind::f16 MMAs then form
// the same products as kind::tf32 at half the operand bytes and twice the rate;
// the epilogue multiplies by the inverse scales.  Entries more than 2^28 below
// the panel maximum fall into the FP16 subnormal range (absolute error below
// 2^-40 of the maximum, far under the TF32 rounding of the large entries).
#include <cuda_fp16.h>
#include <cusolverDn.h>
#include <cmath>

#include "common.cuh"
#include "kernels.cuh"

namespace midas {

// ---------------------------------------------------------------------------
// diagonal block: unblocked LU of A11 (nb x nb, row-major, lda) without pivoting,
// with L11^-1 built alongside (Gauss-Jordan on [A | I]) and U11^-1 by a backward
// Gauss-Jordan sweep.  One CTA of 512 threads; the block, L^-1 and U^-1 stay in
// registers (thread (tx, ty): column tx, rows ty + 8k), only the pivot row, the
// multiplier column and the reciprocal diagonal go through shared memory.
// Writes L\U back to A11, Linv/Uinv (rounded to TF32: GEMM operands), and the
// expanded U11^-1 (the Bt operand of L21 = A21 U11^-1) to UinvExp (2nb x 2nb floats).
// ---------------------------------------------------------------------------
template <int NB>
__global__ void __launch_bounds__(512) k_diag_lu(float2 *A11, long long lda, float2 *Linv, float2 *Uinv,
                                                  float *UinvExp, float tiny, int *flag)
{
    // register-resident: thread (tx, ty) holds column tx, rows ty + 8k (k < 8), of
    // the block (ra), of L^-1 (rx) and of U^-1 (ry); only the pivot row, the
    // multiplier column and the reciprocal diagonal go through shared memory.
    static_assert(NB == 64, "thread mapping assumes 64-wide blocks");
    constexpr int R = NB / 8;
    __shared__ float2 prow[2][NB], xrow[2][NB], lcol[NB], rdiag[NB];
    __shared__ float2 stage[NB][NB + 1];
    const int tid = threadIdx.x;
    if (blockDim.x != 8 * NB) {
        if (tid == 0) atomicOr(flag, DEV_BAD_ARG);
        return;
    }
    const int tx = tid % NB, ty = tid / NB;
    float2 ra[R], rx[R], ry[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int i = ty + 8 * k;
        ra[k] = A11[(long long)i * lda + tx];
        rx[k] = make_float2(i == tx ? 1.f : 0.f, 0.f);
        ry[k] = rx[k];
    }
    if (ty == 0) { prow[0][tx] = ra[0]; xrow[0][tx] = rx[0]; }
    __syncthreads();
    // ---- elimination with L^-1 by Gauss-Jordan on [A | I] ----------------------
    for (int j = 0; j < NB; ++j) {
        const int b = j & 1;
        const float2 piv = prow[b][j];
        const float pm = piv.x * piv.x + piv.y * piv.y;
        if (tid == 0 && !(pm > tiny * tiny)) atomicOr(flag, DEV_ZERO_PIVOT);
        if (tx == j) {   // multipliers of column j (kept as the L entries)
            const float rp = __frcp_rn(pm);
            const float2 ip = make_float2(piv.x * rp, -piv.y * rp);
#pragma unroll
            for (int k = 0; k < R; ++k) {
                const int i = ty + 8 * k;
                if (i > j) {
                    const float2 v = ra[k];
                    ra[k] = make_float2(v.x * ip.x - v.y * ip.y, v.x * ip.y + v.y * ip.x);
                    lcol[i] = ra[k];
                }
            }
        }
        __syncthreads();
        const float2 u = prow[b][tx], xv = xrow[b][tx];
#pragma unroll
        for (int k = 0; k < R; ++k) {
            const int i = ty + 8 * k;
            if (i > j) {
                const float2 l = lcol[i];
                if (tx > j) ra[k] = make_float2(ra[k].x - (l.x * u.x - l.y * u.y), ra[k].y - (l.x * u.y + l.y * u.x));
                else rx[k] = make_float2(rx[k].x - (l.x * xv.x - l.y * xv.y), rx[k].y - (l.x * xv.y + l.y * xv.x));
            }
        }
        if (j + 1 < NB && ty == (j + 1) % 8) {   // row j + 1 is final now: publish it
            const int ks = (j + 1) / 8;
            float2 sa = ra[0], sx = rx[0];   // select chains, not an indexed access: the arrays stay in registers
#pragma unroll
            for (int k = 1; k < R; ++k) {
                sa = ks == k ? ra[k] : sa;
                sx = ks == k ? rx[k] : sx;
            }
            prow[b ^ 1][tx] = sa;
            xrow[b ^ 1][tx] = sx;
        }
        __syncthreads();
    }
    // ---- U^-1 by backward Gauss-Jordan on [U | I] ------------------------------
#pragma unroll
    for (int k = 0; k < R; ++k)
        if (ty + 8 * k == tx) {
            const float2 d = ra[k];
            const float rp = __frcp_rn(d.x * d.x + d.y * d.y);
            rdiag[tx] = make_float2(d.x * rp, -d.y * rp);
        }
    __syncthreads();
    for (int j = NB - 1; j >= 0; --j) {
        const int b = j & 1;
        if (ty == j % 8) {   // row j of Y scaled by 1 / U[j][j]
            const float2 r = rdiag[j];
            const int ks = j / 8;
#pragma unroll
            for (int k = 0; k < R; ++k) {
                const float2 sc = make_float2(ry[k].x * r.x - ry[k].y * r.y, ry[k].x * r.y + ry[k].y * r.x);
                ry[k] = ks == k ? sc : ry[k];
            }
            float2 sy = ry[0];
#pragma unroll
            for (int k = 1; k < R; ++k) sy = ks == k ? ry[k] : sy;
            xrow[b][tx] = sy;
        }
        if (tx == j) {   // column j of U above the diagonal
#pragma unroll
            for (int k = 0; k < R; ++k)
                if (ty + 8 * k < j) lcol[ty + 8 * k] = ra[k];
        }
        __syncthreads();
        const float2 yv = xrow[b][tx];
#pragma unroll
        for (int k = 0; k < R; ++k) {
            const int i = ty + 8 * k;
            if (i < j) {
                const float2 uu = lcol[i];
                ry[k] = make_float2(ry[k].x - (uu.x * yv.x - uu.y * yv.y), ry[k].y - (uu.x * yv.y + uu.y * yv.x));
            }
        }
        __syncthreads();
    }
    // ---- write-back: L\U, the inverses rounded to TF32 (GEMM operands), and the
    // expanded U^-1 as the Bt operand of L21 = A21 U11^-1:
    // Bt[2j][2p] = Ur(p,j), Bt[2j][2p+1] = -Ui(p,j), Bt[2j+1][2p] = Ui, Bt[2j+1][2p+1] = Ur
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int i = ty + 8 * k;
        A11[(long long)i * lda + tx] = ra[k];
        Linv[i * NB + tx] = make_float2(tf32_rna(rx[k].x), tf32_rna(rx[k].y));
        const float2 uq = make_float2(tf32_rna(ry[k].x), tf32_rna(ry[k].y));
        Uinv[i * NB + tx] = uq;
        stage[i][tx] = uq;
    }
    __syncthreads();
    for (int t = tid; t < NB * NB; t += blockDim.x) {
        const int jo = t / NB, p = t % NB;   // consecutive threads: consecutive p, coalesced writes
        const float2 uq = stage[p][jo];
        float *r0 = UinvExp + (long long)(2 * jo) * (2 * NB) + 2 * p;
        float *r1 = r0 + 2 * NB;
        r0[0] = uq.x; r0[1] = -uq.y;
        r1[0] = uq.y; r1[1] = uq.x;
    }
}

// ---------------------------------------------------------------------------
// FP16 panels of the trailing update
// ---------------------------------------------------------------------------
// max over rows x cols complex entries of max(|re|, |im|), as FP32 bits (>= 0)
__global__ void k_panel_absmax(int rows0, int cols0, const float2 *A0, int rows1, int cols1, const float2 *A1,
                               long long lda, unsigned *out)
{
    const int which = blockIdx.y;
    const int rows = which ? rows1 : rows0, cols = which ? cols1 : cols0;
    const float2 *A = which ? A1 : A0;
    const long long tot = (long long)rows * cols;
    float m = 0.f;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
         e += (long long)gridDim.x * blockDim.x) {
        const float2 v = A[(e / cols) * lda + e % cols];
        m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(out + which, __float_as_uint(m));
}

// power of two taking the panel maximum into [2^14, 2^15)
__device__ __forceinline__ float h16_scale(unsigned bits)
{
    const float m = __uint_as_float(bits);
    if (!(m > 0.f) || m > 3.0e38f) return 1.f;
    int e;
    frexpf(m, &e);   // m = f 2^e, f in [0.5, 1)
    return ldexpf(1.f, 15 - e);
}

// L panel (rows x kc complex, row-major lda) -> A16 rows of 2 kc fp16 (re, im
// interleaved), scaled; alpha = -1 / (sL sU) for the update D -= L U.
__global__ void k_pack_a16(int rows, int kc, const float2 *A, long long lda, const unsigned *mx, __half2 *A16,
                           float *alpha)
{
    const float sl = h16_scale(mx[0]);
    if (blockIdx.x == 0 && threadIdx.x == 0) *alpha = -1.f / (sl * h16_scale(mx[1]));
    const long long tot = (long long)rows * kc;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
         e += (long long)gridDim.x * blockDim.x) {
        const float2 v = A[(e / kc) * lda + e % kc];
        A16[e] = __floats2half2_rn(v.x * sl, v.y * sl);
    }
}

// U panel (k x n complex, element (p, j) at B[p * ldb + j]) -> Bt16 (2n rows of
// 2k fp16): row 2j = (Br, -Bi), row 2j+1 = (Bi, Br) along p, scaled.  32 x 32
// tiles through shared memory: reads along j and writes along p both coalesce.
__global__ void k_expand_b16(int k, int n, const float2 *B, long long ldb, const unsigned *mx, __half2 *Bt,
                             long long ldt2)
{
    __shared__ float2 t[32][33];
    const float su = h16_scale(mx[1]);
    const int p0 = blockIdx.x * 32, tx = threadIdx.x, ty = threadIdx.y;
    for (int j0 = blockIdx.y * 32; j0 < n; j0 += gridDim.y * 32) {
#pragma unroll
        for (int q = 0; q < 32; q += 8) {
            const int p = p0 + ty + q, j = j0 + tx;
            t[ty + q][tx] = (p < k && j < n) ? B[(long long)p * ldb + j] : make_float2(0.f, 0.f);
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 32; q += 8) {
            const int j = j0 + ty + q, p = p0 + tx;
            if (j < n && p < k) {
                const float2 b = t[tx][ty + q];
                Bt[(long long)(2 * j) * ldt2 + p] = __floats2half2_rn(b.x * su, -b.y * su);
                Bt[(long long)(2 * j + 1) * ldt2 + p] = __floats2half2_rn(b.y * su, b.x * su);
            }
        }
        __syncthreads();
    }
}

size_t lu_h16_scratch_bytes(int n) { return sizeof(__half) * (size_t)3 * n * 2 * lu_panel_width(n) + 256; }

// ---------------------------------------------------------------------------
// Inverses of the LU_MB x LU_MB (256) diagonal blocks of L and U, for the
// triangular solves: one apply of a 256-row inverse replaces four applies of the
// 64-row inverses and the three small GEMMs between them.  Built per panel
// from the 64-block inverses D_i and the factor blocks inside the diagonal
// block, by block substitution in FP32 on the CUDA cores (the operands are the
// stored TF32-rounded factor entries):
//   L: X_jj = D_j,  X_ij = -D_i sum_{k=j}^{i-1} L_ik X_kj        (i > j)
//   U: X_jj = D_j,  X_ij = -D_i sum_{k=i+1}^{j} U_ik X_kj        (i < j)
// One CTA per (diagonal block, block column j, L or U); X is stored transposed
// (XT[c * LU_MB + r]) so that the apply reads it coalesced, zero outside the
// triangle.
// ---------------------------------------------------------------------------
constexpr int MI_LD = 65;   // padded row stride of the 64 x 64 shared tiles

// 64 x 64 block of a row-major complex matrix into a shared tile
__device__ __forceinline__ void mi_load(float2 *t, const float2 *g, long long ld)
{
    for (int e = threadIdx.x; e < 64 * 64; e += blockDim.x) t[(e / 64) * MI_LD + (e % 64)] = g[(long long)(e / 64) * ld + (e % 64)];
}

// acc (this thread's 4 x 4 outputs, rows ty + 16a, cols tx + 16b) += A B
__device__ __forceinline__ void mi_mma(const float2 *A, const float2 *B, float2 acc[4][4], int tx, int ty)
{
#pragma unroll 4
    for (int k = 0; k < 64; ++k) {
        float2 a[4], b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) a[u] = A[(ty + 16 * u) * MI_LD + k];
#pragma unroll
        for (int u = 0; u < 4; ++u) b[u] = B[k * MI_LD + tx + 16 * u];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                acc[u][v].x = fmaf(a[u].x, b[v].x, fmaf(-a[u].y, b[v].y, acc[u][v].x));
                acc[u][v].y = fmaf(a[u].x, b[v].y, fmaf(a[u].y, b[v].x, acc[u][v].y));
            }
    }
}

__global__ void __launch_bounds__(256) k_macro_inv(const float2 *A, long long lda, int n, int mac0,
                                                    const float2 *Linv, const float2 *Uinv, float2 *MLinvT,
                                                    float2 *MUinvT)
{
    extern __shared__ float2 mi_sm[];
    float2 *As = mi_sm, *Bs = mi_sm + 64 * MI_LD;
    const int mac = mac0 + blockIdx.x / 4, j = blockIdx.x % 4, upper = blockIdx.y;
    const int I0 = mac * LU_MB, mb = min(LU_MB, n - I0), nbk = mb / 64;
    if (j >= nbk) return;
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    const float2 *D = upper ? Uinv : Linv;   // 64-block inverses, row-major
    float2 *XT = (upper ? MUinvT : MLinvT) + (size_t)mac * LU_MB * LU_MB;
    const float2 *Ab = A + (long long)I0 * lda + I0;
    auto put = [&](int bi, const float2 acc[4][4], float sgn) {   // block (bi, j) of X from registers
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                const int r = 64 * bi + ty + 16 * u, cc = 64 * j + tx + 16 * v;
                XT[(size_t)cc * LU_MB + r] = make_float2(sgn * acc[u][v].x, sgn * acc[u][v].y);
            }
    };
    // zero blocks of column j outside the triangle, and the diagonal block D_j
    for (int bi = 0; bi < LU_MB / 64; ++bi) {
        const bool zero = bi >= nbk || (upper ? bi > j : bi < j);
        if (!zero && bi != j) continue;
        for (int e = tid; e < 64 * 64; e += blockDim.x) {
            const int cc = e / 64, rr = e % 64;   // consecutive threads write consecutive rows
            XT[(size_t)(64 * j + cc) * LU_MB + 64 * bi + rr] =
                zero ? make_float2(0.f, 0.f) : D[(size_t)(I0 / 64 + j) * 4096 + rr * 64 + cc];
        }
    }
    __syncthreads();
    const int step = upper ? -1 : 1;
    for (int i = j + step; upper ? i >= 0 : i < nbk; i += step) {
        float2 acc[4][4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] = make_float2(0.f, 0.f);
        // T = sum over k between i and j of F_ik X_kj (F = L below, U above the diagonal)
        const int k0 = upper ? i + 1 : j, k1 = upper ? j : i - 1;
        for (int k = k0; k <= k1; ++k) {
            mi_load(As, Ab + (long long)(64 * i) * lda + 64 * k, lda);
            for (int e = tid; e < 64 * 64; e += blockDim.x) {   // X_kj from XT (written above)
                const int cc = e / 64, rr = e % 64;
                Bs[rr * MI_LD + cc] = XT[(size_t)(64 * j + cc) * LU_MB + 64 * k + rr];
            }
            __syncthreads();
            mi_mma(As, Bs, acc, tx, ty);
            __syncthreads();
        }
        // X_ij = -D_i T
        mi_load(As, D + (size_t)(I0 / 64 + i) * 4096, 64);
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) Bs[(ty + 16 * u) * MI_LD + tx + 16 * v] = acc[u][v];
        __syncthreads();
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] = make_float2(0.f, 0.f);
        mi_mma(As, Bs, acc, tx, ty);
        put(i, acc, -1.f);
        __syncthreads();   // X_ij is read back by the next i; the tiles are reloaded
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
    MIDAS_TRY(ensure(c, S_LINV, lu_inv_bytes(n), &p));
    lu.nmac = (n + LU_MB - 1) / LU_MB;
    lu.Linv = (float2 *)p;
    lu.Uinv = lu.Linv + (size_t)lu.nblk * nb * nb;
    lu.MLinvT = lu.Uinv + (size_t)lu.nblk * nb * nb;
    lu.MUinvT = lu.MLinvT + (size_t)lu.nmac * LU_MB * LU_MB;
    MIDAS_TRY(ensure(c, S_BEXP, sizeof(float) * (size_t)(2 * nb) * (2 * nb), &p));
    float *uexp = (float *)p;
    const int nb2 = lu_panel_width(n);
    MIDAS_TRY(ensure(c, S_BEXP2, lu_bexp2_bytes(n), &p));
    float *bexp = (float *)p;
    // FP16 trailing-update panels (tcgen05 engine): A16 (n x 2 nb2), B16 (2n x 2 nb2), maxima, alpha
    const bool h16 = gemm_tc_engine();
    __half *a16 = nullptr, *b16 = nullptr;
    unsigned *hmax = nullptr;
    float *halpha = nullptr;
    if (h16) {
        MIDAS_TRY(ensure(c, S_H16, lu_h16_scratch_bytes(n), &p));
        a16 = (__half *)p;
        b16 = a16 + (size_t)n * 2 * nb2;
        hmax = (unsigned *)(b16 + (size_t)2 * n * 2 * nb2);
        halpha = (float *)(hmax + 2);
    }
    const size_t mi_smem = sizeof(float2) * 2 * 64 * MI_LD;
    static PerDeviceOnce once;
    MIDAS_CUDA(c, once.run(c->device, [mi_smem] {
        return cudaFuncSetAttribute(k_macro_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mi_smem);
    }));
    const long long lda = lu.lda;
    float *Af = (float *)lu.A;
    // the 256-row diagonal-block inverses only feed the later solves: off the
    // critical path on the side stream (joined when the factorisation returns;
    // on the main stream while per-kernel profiling is on)
    cudaStream_t mi_stream = c->stream;
    if (c->allow_side && !c->kprof.on) MIDAS_TRY(side_stream(c, &mi_stream));
    struct Join {
        midas_gpu_ctx *c;
        bool on;
        ~Join() {
            if (on) {
                cudaEventRecord(c->ev_join, c->side);
                cudaStreamWaitEvent(c->stream, c->ev_join, 0);
            }
        }
    } join{c, mi_stream != c->stream};
    // rnd = 1 for the GEMMs that produce final L or U entries: those are stored
    // rounded to TF32 (round to nearest), as every later use reads them in TF32
    auto gemm = [&](int M, int N, int K, const float *A, long long la, const float *B, long long lb, float *D,
                    long long ld, float alpha, float beta, int rnd, int kc = MIDAS_KC_GEMM_PANEL) {
        GemmArgs g{M, N, K, A, la, B, lb, D, ld, alpha, beta, rnd, kc};
        return gemm_tf32(c, g);
    };
    // Two levels: panels of nb2 columns are factored with LU_NB-wide steps that
    // update only the panel; the rows of U to the right of the panel follow by a
    // blocked forward substitution, and the trailing matrix takes one update with
    // K = nb2 -- 1/4 to 1/16 of the trailing-matrix traffic of LU_NB-wide updates.
    for (int J0 = 0; J0 < n; J0 += nb2) {
        const int J1 = std::min(n, J0 + nb2);
        for (int j0 = J0; j0 < J1; j0 += nb) {
            const int k = j0 / nb, rem = n - j0 - nb, wp = J1 - j0 - nb;
            float2 *A11 = lu.A + (long long)j0 * lda + j0;
            ++c->launches;
            int kp = kp_begin(c);
            k_diag_lu<LU_NB><<<1, 512, 0, c->stream>>>(A11, lda, lu.Linv + (size_t)k * nb * nb,
                                                          lu.Uinv + (size_t)k * nb * nb, uexp, 1e-30f, c->d_flag);
            kp_end(c, kp, MIDAS_KC_DIAG_LU, 8.0 * nb * nb * nb, 8.0 * nb * nb * 4);
            MIDAS_CUDA(c, cudaGetLastError());
            if (rem == 0) break;
            // L21 = A21 U11^-1 (in place: each output row tile reads only its own rows)
            MIDAS_TRY(gemm(rem, 2 * nb, 2 * nb, Af + 2 * ((long long)(j0 + nb) * lda + j0), 2 * lda, uexp, 2 * nb,
                           Af + 2 * ((long long)(j0 + nb) * lda + j0), 2 * lda, 1.f, 0.f, 1));
            if (wp == 0) continue;
            // panel columns right of the step: U12 = L11^-1 A12, then A22(panel) -= L21 U12
            MIDAS_TRY(expand_b(c, nb, wp, lu.A + (long long)j0 * lda + j0 + nb, lda, 1, bexp, 2 * nb));
            MIDAS_TRY(gemm(nb, 2 * wp, 2 * nb, (const float *)(lu.Linv + (size_t)k * nb * nb), 2 * nb, bexp, 2 * nb,
                           Af + 2 * ((long long)j0 * lda + j0 + nb), 2 * lda, 1.f, 0.f, 1));
            MIDAS_TRY(expand_b(c, nb, wp, lu.A + (long long)j0 * lda + j0 + nb, lda, 1, bexp, 2 * nb));
            MIDAS_TRY(gemm(rem, 2 * wp, 2 * nb, Af + 2 * ((long long)(j0 + nb) * lda + j0), 2 * lda, bexp, 2 * nb,
                           Af + 2 * ((long long)(j0 + nb) * lda + j0 + nb), 2 * lda, -1.f, 1.f, 0));
        }
        {   // inverses of the solve's 256-row diagonal blocks inside this panel (final now;
            // nothing later in the factorisation writes the panel's diagonal region)
            const int m0 = J0 / LU_MB, m1 = (J1 + LU_MB - 1) / LU_MB;
            if (join.on) {
                MIDAS_CUDA(c, cudaEventRecord(c->ev_fork, c->stream));
                MIDAS_CUDA(c, cudaStreamWaitEvent(mi_stream, c->ev_fork, 0));
            }
            ++c->launches;
            int kp = join.on ? -1 : kp_begin(c);
            k_macro_inv<<<dim3(4 * (m1 - m0), 2), 256, mi_smem, mi_stream>>>(lu.A, lda, n, m0, lu.Linv, lu.Uinv,
                                                                            lu.MLinvT, lu.MUinvT);
            kp_end(c, kp, MIDAS_KC_DIAG_LU, 8.0 * 64 * 64 * 64 * 16 * (m1 - m0), 0.0);
            MIDAS_CUDA(c, cudaGetLastError());
        }
        const int rt = n - J1;
        if (rt == 0) break;
        // U(J0:J1, J1:n) = L(J0:J1, J0:J1)^-1 A(J0:J1, J1:n), LU_NB rows at a time
        for (int j0 = J0; j0 < J1; j0 += nb) {
            const int k = j0 / nb, below = J1 - j0 - nb;
            MIDAS_TRY(expand_b(c, nb, rt, lu.A + (long long)j0 * lda + J1, lda, 1, bexp, 2 * nb));
            MIDAS_TRY(gemm(nb, 2 * rt, 2 * nb, (const float *)(lu.Linv + (size_t)k * nb * nb), 2 * nb, bexp, 2 * nb,
                           Af + 2 * ((long long)j0 * lda + J1), 2 * lda, 1.f, 0.f, 1));
            if (below == 0) continue;
            MIDAS_TRY(expand_b(c, nb, rt, lu.A + (long long)j0 * lda + J1, lda, 1, bexp, 2 * nb));
            MIDAS_TRY(gemm(below, 2 * rt, 2 * nb, Af + 2 * ((long long)(j0 + nb) * lda + j0), 2 * lda, bexp, 2 * nb,
                           Af + 2 * ((long long)(j0 + nb) * lda + J1), 2 * lda, -1.f, 1.f, 0));
        }
        // trailing matrix: A(J1:n, J1:n) -= L(J1:n, J0:J1) U(J0:J1, J1:n), K = J1 - J0
        const int kw = J1 - J0;
        if (h16) {
            const float2 *Lp = lu.A + (long long)J1 * lda + J0, *Up = lu.A + (long long)J0 * lda + J1;
            MIDAS_CUDA(c, cudaMemsetAsync(hmax, 0, 2 * sizeof(unsigned), c->stream));
            const long long big = (long long)rt * kw;
            const unsigned gx = (unsigned)std::min<long long>((big + 255) / 256, 4LL * 152);
            c->launches += 3;
            k_panel_absmax<<<dim3(gx, 2), 256, 0, c->stream>>>(rt, kw, Lp, kw, rt, Up, lda, hmax);
            k_pack_a16<<<gx, 256, 0, c->stream>>>(rt, kw, Lp, lda, hmax, (__half2 *)a16, halpha);
            k_expand_b16<<<dim3((kw + 31) / 32, (unsigned)std::min(65535, (rt + 31) / 32)), dim3(32, 8), 0,
                           c->stream>>>(kw, rt, Up, lda, hmax, (__half2 *)b16, kw);
            MIDAS_CUDA(c, cudaGetLastError());
            GemmArgs g{rt, 2 * rt, 2 * kw, (const float *)a16, 2 * kw, (const float *)b16, 2 * kw,
                       Af + 2 * ((long long)J1 * lda + J1), 2 * lda, -1.f, 1.f, 0, MIDAS_KC_GEMM_TC};
            g.h16 = 1;
            g.alpha_dev = halpha;
            MIDAS_TRY(gemm_tf32(c, g));
            continue;
        }
        MIDAS_TRY(expand_b(c, kw, rt, lu.A + (long long)J0 * lda + J1, lda, 1, bexp, 2 * kw));
        MIDAS_TRY(gemm(rt, 2 * rt, 2 * kw, Af + 2 * ((long long)J1 * lda + J0), 2 * lda, bexp, 2 * kw,
                       Af + 2 * ((long long)J1 * lda + J1), 2 * lda, -1.f, 1.f, 0, MIDAS_KC_GEMM_TC));
    }
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// blocked triangular solves on the tensor cores.  The right-hand sides are
// solved in row-major form Rt (n x nrhs), so every update is one tcgen05 GEMM
// whose A operand is the L or U panel read in place (row-major, no copy):
//   Rt[rows below] -= L[rows below, block] * Y[block]      (forward)
//   Rt[rows above] -= U[rows above, block] * X[block]      (backward)
// Two levels: inside a super-block of SOLVE_SB rows the 256-row diagonal
// blocks are applied one after the other (their inverses come from the
// factorisation) and update only the rows of the super-block; one GEMM with
// K = SOLVE_SB then updates every row outside it.  The right-hand-side
// traffic per super-block is then O(n nrhs) instead of O(n nrhs) per 64 rows.
// ---------------------------------------------------------------------------
constexpr int SOLVE_SB = 512;
static_assert(SOLVE_SB % LU_MB == 0, "super-blocks hold whole diagonal blocks");

size_t lu_solve_scratch_bytes(int n, int nrhs)
{
    return sizeof(float2) * (size_t)n * nrhs + sizeof(float) * 4 * (size_t)nrhs * SOLVE_SB + 512;
}

// column-major R (n x nrhs, ld n) -> row-major Rt (n x nrhs), 32 x 32 tiles
__global__ void k_cm_to_rm(const float2 *R, int n, int nrhs, float2 *Rt)
{
    __shared__ float2 tile[32][33];
    const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32, tx = threadIdx.x;
    for (int k = threadIdx.y; k < 32; k += blockDim.y)
        if (r0 + tx < n && c0 + k < nrhs) tile[k][tx] = R[(long long)(c0 + k) * n + r0 + tx];
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y)
        if (r0 + k < n && c0 + tx < nrhs) Rt[(long long)(r0 + k) * nrhs + c0 + tx] = tile[tx][k];
}

// row-major Rt -> column-major R
__global__ void k_rm_to_cm(const float2 *Rt, int n, int nrhs, float2 *R)
{
    __shared__ float2 tile[32][33];
    const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32, tx = threadIdx.x;
    for (int k = threadIdx.y; k < 32; k += blockDim.y)
        if (r0 + k < n && c0 + tx < nrhs) tile[k][tx] = Rt[(long long)(r0 + k) * nrhs + c0 + tx];
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y)
        if (r0 + tx < n && c0 + k < nrhs) R[(long long)(c0 + k) * n + r0 + tx] = tile[tx][k];
}

// Y = X * Rt[r0 .. r0+mb) for a 256-row diagonal-block inverse X (transposed,
// XT[c * LU_MB + r]; block lower triangular for L, upper for U), in place, 4
// right-hand sides per CTA.  Each row's columns are split over AM_CS threads
// (thread (s, r) takes columns s, s + AM_CS, ...; a warp is 32 rows of one s,
// so the reads of XT coalesce), which keeps the chain of L2 loads per thread
// short; the partial sums meet in shared memory.  The expanded copy of Y for the
// next GEMM's B operand goes to Bt: rows 2j, 2j+1 hold (Yr, -Yi) and (Yi, Yr),
// rounded to TF32, interleaved along the mb rows from column col0.
constexpr int AM_RC = 4, AM_CS = 4;
__global__ void __launch_bounds__(LU_MB * AM_CS) k_apply_minv(const float2 *XT, int mb, int upper, float2 *Rt,
                                                              int nrhs, int r0, float *Bt, long long ldb, int col0)
{
    __shared__ float2 t[LU_MB][AM_RC];
    __shared__ float2 part[AM_CS - 1][LU_MB][AM_RC];
    const int c0 = blockIdx.x * AM_RC, r = threadIdx.x % LU_MB, sp = threadIdx.x / LU_MB;
    for (int q = threadIdx.x; q < mb * AM_RC; q += blockDim.x) {
        const int rr = q / AM_RC, j = q % AM_RC;
        t[rr][j] = c0 + j < nrhs ? Rt[(long long)(r0 + rr) * nrhs + c0 + j] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 acc[AM_RC];
#pragma unroll
    for (int j = 0; j < AM_RC; ++j) acc[j] = make_float2(0.f, 0.f);
    if (r < mb) {
        // the nonzero 64-column blocks of row r (warp-uniform bounds)
        const int cb = upper ? (r / 64) * 64 : 0, ce = upper ? mb : (r / 64 + 1) * 64;
#pragma unroll 8
        for (int cc = cb + sp; cc < ce; cc += AM_CS) {
            const float2 x = XT[(size_t)cc * LU_MB + r];
#pragma unroll
            for (int j = 0; j < AM_RC; ++j) {
                const float2 v = t[cc][j];
                acc[j].x = fmaf(x.x, v.x, fmaf(-x.y, v.y, acc[j].x));
                acc[j].y = fmaf(x.x, v.y, fmaf(x.y, v.x, acc[j].y));
            }
        }
    }
    if (sp > 0) {
#pragma unroll
        for (int j = 0; j < AM_RC; ++j) part[sp - 1][r][j] = acc[j];
    }
    __syncthreads();
    if (sp > 0 || r >= mb) return;
#pragma unroll
    for (int s2 = 0; s2 < AM_CS - 1; ++s2)
#pragma unroll
        for (int j = 0; j < AM_RC; ++j) {
            acc[j].x += part[s2][r][j].x;
            acc[j].y += part[s2][r][j].y;
        }
#pragma unroll
    for (int j = 0; j < AM_RC; ++j) {
        const int col = c0 + j;
        if (col >= nrhs) break;
        Rt[(long long)(r0 + r) * nrhs + col] = acc[j];
        float *b0 = Bt + (long long)(2 * col) * ldb + col0 + 2 * r, *b1 = b0 + ldb;
        const float yr = tf32_rna(acc[j].x), yi = tf32_rna(acc[j].y);   // GEMM operand: unbiased TF32
        b0[0] = yr; b0[1] = -yi;
        b1[0] = yi; b1[1] = yr;
    }
}

static int apply_minv(midas_gpu_ctx *c, const float2 *XT, int mb, int upper, float2 *Rt, int nrhs, int r0, float *Bt,
                      long long ldb, int col0)
{
    ++c->launches;
    int kp = kp_begin(c);
    k_apply_minv<<<(nrhs + AM_RC - 1) / AM_RC, LU_MB * AM_CS, 0, c->stream>>>(XT, mb, upper, Rt, nrhs, r0, Bt, ldb,
                                                                                col0);
    kp_end(c, kp, MIDAS_KC_TRSV, 4.0 * mb * mb * nrhs, 8.0 * mb * mb / 2 * ((nrhs + AM_RC - 1) / AM_RC) +
                                                         32.0 * mb * nrhs);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

int lu_solve(midas_gpu_ctx *c, const DenseLU &lu, float2 *R, int nrhs)
{
    const int n = lu.n, nb = lu.nb;
    if (nb != 64) return c->err.set(MIDAS_ERR_ARG, "lu_solve: block size must be 64");
    void *p;
    MIDAS_TRY(ensure(c, S_SOLVE, lu_solve_scratch_bytes(n, nrhs), &p));
    float2 *Rt = (float2 *)p;
    float *Bt = (float *)((char *)p + (((sizeof(float2) * (size_t)n * nrhs) + 255) & ~(size_t)255));
    float *Rtf = (float *)Rt;
    const float *Af = (const float *)lu.A;
    const long long lda = lu.lda;
    dim3 tb(32, 8), tg((n + 31) / 32, (nrhs + 31) / 32);
    ++c->launches;
    k_cm_to_rm<<<tg, tb, 0, c->stream>>>(R, n, nrhs, Rt);
    MIDAS_CUDA(c, cudaGetLastError());
    const int nsb = (n + SOLVE_SB - 1) / SOLVE_SB;
    // forward: L Y = B
    for (int S = 0; S < nsb; ++S) {
        const int K0 = S * SOLVE_SB, K1 = std::min(n, K0 + SOLVE_SB), ldb = 2 * (K1 - K0);
        for (int r0 = K0; r0 < K1; r0 += LU_MB) {
            const int mb = std::min(LU_MB, K1 - r0);
            MIDAS_TRY(apply_minv(c, lu.MLinvT + (size_t)(r0 / LU_MB) * LU_MB * LU_MB, mb, 0, Rt, nrhs, r0, Bt, ldb,
                                 2 * (r0 - K0)));
            const int rows = K1 - (r0 + mb);
            if (rows > 0) {
                GemmArgs g{rows, 2 * nrhs, 2 * mb, Af + 2 * ((r0 + mb) * lda + r0), 2 * lda, Bt + 2 * (r0 - K0), ldb,
                           Rtf + 2LL * (r0 + mb) * nrhs, 2LL * nrhs, -1.f, 1.f, 0, MIDAS_KC_GEMM_SOLVE};
                MIDAS_TRY(gemm_tf32(c, g));
            }
        }
        if (K1 < n) {
            GemmArgs g{n - K1, 2 * nrhs, ldb, Af + 2 * (K1 * lda + K0), 2 * lda, Bt, ldb, Rtf + 2LL * K1 * nrhs,
                       2LL * nrhs, -1.f, 1.f, 0, MIDAS_KC_GEMM_SOLVE};
            MIDAS_TRY(gemm_tf32(c, g));
        }
    }
    // backward: U X = Y
    for (int S = nsb - 1; S >= 0; --S) {
        const int K0 = S * SOLVE_SB, K1 = std::min(n, K0 + SOLVE_SB), ldb = 2 * (K1 - K0);
        for (int r0 = (K1 - 1) / LU_MB * LU_MB; r0 >= K0; r0 -= LU_MB) {
            const int mb = std::min(LU_MB, K1 - r0);
            MIDAS_TRY(apply_minv(c, lu.MUinvT + (size_t)(r0 / LU_MB) * LU_MB * LU_MB, mb, 1, Rt, nrhs, r0, Bt, ldb,
                                 2 * (r0 - K0)));
            const int rows = r0 - K0;
            if (rows > 0) {
                GemmArgs g{rows, 2 * nrhs, 2 * mb, Af + 2 * (K0 * lda + r0), 2 * lda, Bt + 2 * (r0 - K0), ldb,
                           Rtf + 2LL * K0 * nrhs, 2LL * nrhs, -1.f, 1.f, 0, MIDAS_KC_GEMM_SOLVE};
                MIDAS_TRY(gemm_tf32(c, g));
            }
        }
        if (K0 > 0) {
            GemmArgs g{K0, 2 * nrhs, ldb, Af + 2 * K0, 2 * lda, Bt, ldb, Rtf, 2LL * nrhs, -1.f, 1.f, 0,
                       MIDAS_KC_GEMM_SOLVE};
            MIDAS_TRY(gemm_tf32(c, g));
        }
    }
    ++c->launches;
    k_rm_to_cm<<<tg, tb, 0, c->stream>>>(Rt, n, nrhs, R);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// FP64 residual r = b - Z x (Z row-major FP64, warp per row), per-column
// inf-norms of r and x reduced with atomicMax on the bit pattern (>= 0 doubles).
// ---------------------------------------------------------------------------
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

// x += d; dmax[j] = max over column j (ld n, n % 32 == 0) of max(|Re d|, |Im d|)
__global__ void k_add_corr(double2 *x, const float2 *d, long long nn, int n, unsigned long long *dmax)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double m = 0;
    if (i < nn) {
        const float2 v = d[i];
        x[i].x += v.x;
        x[i].y += v.y;
        m = fmax(fabs((double)v.x), fabs((double)v.y));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && i < nn) atomicMax(dmax + i / n, (unsigned long long)__double_as_longlong(m));
}

__global__ void k_to32(const double2 *v, long long n, float2 *out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = make_float2((float)v[i].x, (float)v[i].y);
}

// Refinement (the FP64 answer of the reference's ZGESV/PZGESV solve,
// src/Compute_EFields.f90:145-176, from TF32 factors).  x0 = LU^-1 b is ~1e-4
// off, and each step gains ~3 decimal digits.  Residuals on the FP32 cores:
//   step 0   r = b - Zh x0 in FP32: x0 is only ~1e-4 accurate, the ~1e-7
//            error of the product does not limit the next correction;
//   then     r = b - Z x in double-float (FP64 grade), or the update
//            r -= Zh d in FP32 (d the correction just added to x).
// An update moves r away from the true residual b - Z x by at most
// g |Z|_inf |d|_inf (g = resid_update_error_factor: the FP32 partial sums of
// the product).  That drift bound D is carried (reset by a double-float
// residual, set to g after the FP32 step 0), an update is taken only while
// D + g |d| / |x| stays within tol / 4, and convergence is accepted when
// berr + D <= tol -- so the backward error of b - Z x in FP64 grade is within
// the tolerance, whichever residual ended the iteration.
int ir_solve(midas_gpu_ctx *c, const DenseLU &lu, double2 *Z64, long long ldz, const double2 *b, double2 *x,
             int nrhs, midas_gpu_info *info)
{
    const int n = lu.n;
    const size_t nn = (size_t)n * nrhs;
    double znorm;
    MIDAS_TRY(z_split_inplace(c, Z64, ldz, n, &znorm));
    const float4 *Zs = (const float4 *)Z64;
    void *p;
    MIDAS_TRY(ensure(c, S_R64, sizeof(double2) * nn, &p));
    double2 *r = (double2 *)p;
    MIDAS_TRY(ensure(c, S_T32B, sizeof(float2) * nn, &p));
    float2 *r32 = (float2 *)p;
    MIDAS_TRY(ensure(c, S_T32, sizeof(float2) * nn, &p));
    float2 *d32 = (float2 *)p;
    MIDAS_TRY(ensure(c, S_RED, sizeof(unsigned long long) * 4 * nrhs + 64, &p));
    // red: [0, nrhs) max|r|, [nrhs, 2 nrhs) max|x|, [2 nrhs, 3 nrhs) max|b|, [3 nrhs, 4 nrhs) max|d|
    unsigned long long *red = (unsigned long long *)p;
    std::vector<unsigned long long> h(4 * nrhs);
    auto colmax = [&](int k, int slot) {
        double v;
        memcpy(&v, &h[(size_t)slot * nrhs + k], 8);
        return v;
    };
    MIDAS_CUDA(c, cudaMemsetAsync(red, 0, sizeof(unsigned long long) * 4 * nrhs, c->stream));
    ++c->launches;
    k_colmax<<<dim3(64, nrhs), 256, 0, c->stream>>>(b, n, nrhs, red + 2 * nrhs);
    MIDAS_CUDA(c, cudaMemsetAsync(x, 0, sizeof(double2) * nn, c->stream));
    ++c->launches;
    k_to32<<<(unsigned)std::min<size_t>((nn + 255) / 256, 65535), 256, 0, c->stream>>>(b, (long long)nn, r32);
    MIDAS_CUDA(c, cudaGetLastError());
    const double tol = c->opts.ir_tol > 0 ? c->opts.ir_tol : 1e-13;
    const int itmax = c->opts.ir_max_iter > 0 ? c->opts.ir_max_iter : 30;
    const double g = resid_update_error_factor(c, n, nrhs);
    double berr = 1e300, drift = 1e300;
    int it;
    bool done = false;
    for (it = 0; it < itmax && !done; ++it) {
        MIDAS_CUDA(c, cudaMemcpyAsync(d32, r32, sizeof(float2) * nn, cudaMemcpyDeviceToDevice, c->stream));
        MIDAS_TRY(lu_solve(c, lu, d32, nrhs));
        MIDAS_CUDA(c, cudaMemsetAsync(red, 0, sizeof(unsigned long long) * 2 * nrhs, c->stream));
        MIDAS_CUDA(c, cudaMemsetAsync(red + 3 * nrhs, 0, sizeof(unsigned long long) * nrhs, c->stream));
        ++c->launches;
        k_add_corr<<<(unsigned)((nn + 255) / 256), 256, 0, c->stream>>>(x, d32, (long long)nn, n, red + 3 * nrhs);
        ++c->launches;
        k_colmax<<<dim3(64, nrhs), 256, 0, c->stream>>>(x, n, nrhs, red + nrhs);
        MIDAS_CUDA(c, cudaGetLastError());
        // |d| / |x| of this correction decides between an update and a double-float residual
        double dn = 0;
        if (it > 0) {
            MIDAS_CUDA(c, cudaMemcpyAsync(h.data(), red, sizeof(unsigned long long) * 4 * nrhs,
                                          cudaMemcpyDeviceToHost, c->stream));
            MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
            for (int k = 0; k < nrhs; ++k) {
                const double xn = colmax(k, 1), dk = colmax(k, 3);
                dn = std::max(dn, xn > 0 ? dk / xn : (dk > 0 ? 1e300 : 0.0));
            }
        }
        const int mode = it == 0 ? 0 : (drift + g * dn <= 0.25 * tol ? 1 : 2);   // 0 fp32, 1 update, 2 double-float
        if (mode == 0)   // x = d exactly
            MIDAS_TRY(resid_dense(c, n, nrhs, Zs, ldz, false, nullptr, d32, b, r, r32, red));
        else if (mode == 1)
            MIDAS_TRY(resid_dense(c, n, nrhs, Zs, ldz, false, nullptr, d32, r, r, r32, red));
        else
            MIDAS_TRY(resid_dense(c, n, nrhs, Zs, ldz, true, x, nullptr, b, r, r32, red));
        drift = mode == 0 ? g : mode == 1 ? drift + g * dn : 0.0;
        MIDAS_CUDA(c, cudaMemcpyAsync(h.data(), red, sizeof(unsigned long long) * 4 * nrhs, cudaMemcpyDeviceToHost,
                                      c->stream));
        MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
        MIDAS_TRY(check_flag(c, "ir_solve"));
        berr = 0;
        for (int k = 0; k < nrhs; ++k) {
            const double den = znorm * colmax(k, 1) + colmax(k, 2);
            const double rn = colmax(k, 0);
            berr = fmax(berr, den > 0 ? rn / den : rn);
        }
        if (!(berr == berr)) return c->err.set(MIDAS_ERR_NOT_CONVERGED, "ir_solve: NaN residual");
        if (c->opts.verbose)
            fprintf(stderr, "[midas] ir step %d (%s residual): backward error %.3e, drift bound %.1e\n", it,
                    mode == 0 ? "fp32" : mode == 1 ? "fp32 update" : "double-float", berr, drift);
        done = berr + drift <= tol;
    }
    if (info) {
        info->ir_iters = it;
        info->backward_error = berr + drift;
        info->anorm = znorm;
    }
    if (!done) {
        char m[160];
        snprintf(m, sizeof m, "iterative refinement stalled at backward error %.3e after %d steps", berr + drift, it);
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
int mixed_solve(midas_gpu_ctx *c, int np, float2 *Z32, double2 *Z64, const double2 *b, double2 *x,
                              int nrhs, midas_gpu_info *info, DenseLU *lu_out)
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
    if (lu_out) *lu_out = lu;
    return st;
}


// ||Z||_inf of the complex64 matrix (row sums of |z| in FP32, as k_z_split forms
// them from the FP64 matrix), before the factorisation overwrites it
__global__ void __launch_bounds__(256) k_row_abs_max(int n, long long ldz, const float2 *Z, unsigned *znorm)
{
    __shared__ float red[8];
    for (int row = blockIdx.x; row < n; row += gridDim.x) {
        const float2 *zr = Z + (long long)row * ldz;
        float s = 0.f;
        for (int m = threadIdx.x; m < n; m += blockDim.x) s += hypotf(zr[m].x, zr[m].y);
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

// Refinement whose every residual b - Z x is the FP64 FFT lattice operator
// (fft.cu): no FP64 matrix, no double-float pass, no drift bookkeeping -- each
// residual is FP64-grade.  x0 = LU^-1 b from the TF32 factors, then x += LU^-1 r
// until the normwise backward error is <= ir_tol.  b, x column-major (ld n, the
// padded size); rows >= 3 ncell are the identity padding (b = 0 there, so x and
// r stay 0).
static int ir_solve_lattice(midas_gpu_ctx *c, const DenseLU &lu, double znorm, const double2 *b, double2 *x,
                            int nrhs, midas_gpu_info *info)
{
    const int n = lu.n;
    const size_t nn = (size_t)n * nrhs;
    void *p;
    MIDAS_TRY(ensure(c, S_R64, sizeof(double2) * nn, &p));
    double2 *r = (double2 *)p;
    MIDAS_TRY(ensure(c, S_T32, sizeof(float2) * nn, &p));
    float2 *d32 = (float2 *)p;
    MIDAS_TRY(ensure(c, S_RED, sizeof(unsigned long long) * 4 * nrhs + 64, &p));
    unsigned long long *red = (unsigned long long *)p;   // max|r|, max|x|, max|b|, max|d| per column
    std::vector<unsigned long long> h(4 * nrhs);
    auto colmax = [&](int k, int slot) {
        double v;
        memcpy(&v, &h[(size_t)slot * nrhs + k], 8);
        return v;
    };
    MIDAS_CUDA(c, cudaMemsetAsync(red, 0, sizeof(unsigned long long) * 4 * nrhs, c->stream));
    ++c->launches;
    k_colmax<<<dim3(64, nrhs), 256, 0, c->stream>>>(b, n, nrhs, red + 2 * nrhs);
    MIDAS_CUDA(c, cudaMemsetAsync(x, 0, sizeof(double2) * nn, c->stream));
    MIDAS_CUDA(c, cudaMemcpyAsync(r, b, sizeof(double2) * nn, cudaMemcpyDeviceToDevice, c->stream));
    const double tol = c->opts.ir_tol > 0 ? c->opts.ir_tol : 1e-13;
    const int itmax = c->opts.ir_max_iter > 0 ? c->opts.ir_max_iter : 30;
    double berr = 1e300;
    int it;
    bool done = false;
    for (it = 0; it < itmax && !done; ++it) {
        ++c->launches;
        k_to32<<<(unsigned)std::min<size_t>((nn + 255) / 256, 65535), 256, 0, c->stream>>>(r, (long long)nn, d32);
        MIDAS_TRY(lu_solve(c, lu, d32, nrhs));
        MIDAS_CUDA(c, cudaMemsetAsync(red, 0, sizeof(unsigned long long) * 2 * nrhs, c->stream));
        ++c->launches;
        k_add_corr<<<(unsigned)((nn + 255) / 256), 256, 0, c->stream>>>(x, d32, (long long)nn, n, red + 3 * nrhs);
        ++c->launches;
        k_colmax<<<dim3(64, nrhs), 256, 0, c->stream>>>(x, n, nrhs, red + nrhs);
        MIDAS_CUDA(c, cudaGetLastError());
        MIDAS_TRY(lattice_matvec(c, nrhs, x, n, b, n, r, n, S_LFFT));   // r = b - Z x
        ++c->launches;
        k_colmax<<<dim3(64, nrhs), 256, 0, c->stream>>>(r, n, nrhs, red);
        MIDAS_CUDA(c, cudaMemcpyAsync(h.data(), red, sizeof(unsigned long long) * 4 * nrhs, cudaMemcpyDeviceToHost,
                                      c->stream));
        MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
        MIDAS_TRY(check_flag(c, "ir_solve_lattice"));
        berr = 0;
        for (int k = 0; k < nrhs; ++k) {
            const double den = znorm * colmax(k, 1) + colmax(k, 2);
            const double rn = colmax(k, 0);
            berr = fmax(berr, den > 0 ? rn / den : rn);
        }
        if (!(berr == berr)) return c->err.set(MIDAS_ERR_NOT_CONVERGED, "ir_solve_lattice: NaN residual");
        if (c->opts.verbose)
            fprintf(stderr, "[midas] ir step %d (FFT lattice residual): backward error %.3e\n", it, berr);
        done = berr <= tol;
    }
    if (info) {
        info->ir_iters = it;
        info->backward_error = berr;
        info->anorm = znorm;
    }
    if (!done) {
        char m[160];
        snprintf(m, sizeof m, "iterative refinement stalled at backward error %.3e after %d steps", berr, it);
        return c->err.set(MIDAS_ERR_NOT_CONVERGED, m);
    }
    return MIDAS_OK;
}

// Mixed solve of the MoM system of lattice cells: Z32 (row-major np x np, padded
// with an identity) factorised in place, residuals from the FFT operator.
int mixed_solve_lattice(midas_gpu_ctx *c, int np, float2 *Z32, const double2 *b, double2 *x, int nrhs,
                        midas_gpu_info *info)
{
    void *p;
    MIDAS_TRY(ensure(c, S_RED2, 64, &p));
    unsigned *dnorm = (unsigned *)p;
    MIDAS_CUDA(c, cudaMemsetAsync(dnorm, 0, sizeof(unsigned), c->stream));
    ++c->launches;
    k_row_abs_max<<<std::min(np, 4 * device_sms(c)), 256, 0, c->stream>>>(np, np, Z32, dnorm);
    unsigned hn = 0;
    MIDAS_CUDA(c, cudaMemcpyAsync(&hn, dnorm, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    MIDAS_TRY(lattice_fft_prepare(c));
    DenseLU lu;
    lu.n = np;
    lu.A = Z32;
    lu.lda = np;
    Timer tf(c->stream);
    MIDAS_TRY(lu_factor_nopiv(c, lu));
    MIDAS_TRY(check_flag(c, "lu_factor"));
    float tfac = tf.stop();
    float znf;
    memcpy(&znf, &hn, 4);
    Timer ts(c->stream);
    int st = ir_solve_lattice(c, lu, (double)znf, b, x, nrhs, info);
    float tsol = ts.stop();
    if (info) { info->t_factor_ms = tfac; info->t_solve_ms = tsol; }
    return st;
}

void destroy_cusolver(void *h) { cusolverDnDestroy((cusolverDnHandle_t)h); }

}  // namespace midas
