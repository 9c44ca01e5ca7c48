// gemm.cu -- FP32-in / FP32-accumulate GEMM for the MIDAS dense solves (sm_103a).
//
//   D[M x N] = alpha * A[M x K] * Bt[N x K]^T + beta * D        (row-major, K contiguous)
//
// Complex matrices use the real embedding: an interleaved complex row of length
// k is a real row of length 2k; the complex right operand is expanded by
// expand_b() into Bt rows (Br, -Bi) / (Bi, Br), so one real GEMM computes the
// complex product with 8mnk flops (the 4M count) and no separate planes.
//
// Engine "tcgen05": TMA (cp.async.bulk.tensor, 128B swizzle) feeds a 4-stage
// shared-memory ring; one elected thread issues tcgen05.mma.kind::tf32 with the
// 128 x BN accumulator in tensor memory; four epilogue warps drain TMEM with
// tcgen05.ld and apply alpha/beta.  Every mbarrier wait is bounded: on expiry
// the kernel raises DEV_TIMEOUT in the context flag and unwinds (TMEM freed).
// A register-tiled CUDA-core kernel (k_gemm_simt) is the device-side check of the
// tensor path in gemm_selftest; no product of the library runs on it.
#include <cuda.h>
#include <cuda_fp16.h>
#include <atomic>
#include <cstdlib>
#include <cstring>

#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace midas {

// ---------------------------------------------------------------------------
// SIMT engine: 64 x 64 tile, 256 threads, 4 x 4 outputs per thread.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_gemm_simt(GemmArgs g)
{
    __shared__ float As[16][64 + 4];
    __shared__ float Bs[16][64 + 4];
    int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < g.K; k0 += 16) {
        for (int i = threadIdx.x; i < 64 * 16; i += 256) {
            int r = i / 16, kk = i % 16;
            int gm = m0 + r, gn = n0 + r, gk = k0 + kk;
            As[kk][r] = (gm < g.M && gk < g.K) ? g.A[(long long)gm * g.lda + gk] : 0.f;
            Bs[kk][r] = (gn < g.N && gk < g.K) ? g.Bt[(long long)gn * g.ldb + gk] : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) { a[i] = As[kk][ty * 4 + i]; b[i] = Bs[kk][tx * 4 + i]; }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int gm = m0 + ty * 4 + i, gn = n0 + tx * 4 + j;
            if (gm < g.M && gn < g.N) {
                float *d = g.D + (long long)gm * g.ldd + gn;
                *d = g.alpha * acc[i][j] + (g.beta != 0.f ? g.beta * *d : 0.f);
            }
        }
}

// ---------------------------------------------------------------------------
// tcgen05 engine
// ---------------------------------------------------------------------------
constexpr int TC_BM = 128;
constexpr int TC_BN = 128;
constexpr int TC_BK = 32;          // 32 fp32 = 128 B = one 128B-swizzle row
constexpr int TC_THREADS = 192;    // warp0 TMA, warp1 MMA/TMEM, warps2-5 epilogue
constexpr int TC_A_BYTES = TC_BM * TC_BK * 4;
constexpr int TC_B_BYTES = TC_BN * TC_BK * 4;
constexpr int TC_STAGE_BYTES = TC_A_BYTES + TC_B_BYTES;
// 4 stages for long K; 2 stages (and two CTAs per SM, so one CTA's epilogue
// overlaps the other's loads) for the K <= 256 updates of the LU and the solves
__host__ __device__ constexpr int tc_smem(int stages) { return stages * TC_STAGE_BYTES + 1024 /*align*/ + 256; }
constexpr int TC_EPI_PITCH = 36;   // floats per staged row (32 + 4: conflict-free float4 access)
constexpr uint32_t TC_SPIN_LIMIT = 1u << 26;   // bounded waits (~seconds with backoff)

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ bool mbar_try(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait: returns false (and raises the abort flag) when `limit` polls expire
__device__ __forceinline__ bool mbar_wait_n(uint64_t *bar, uint32_t parity, volatile int *abort_flag, int *gflag,
                                            uint32_t limit)
{
    for (uint32_t i = 0; i < limit; ++i) {
        if (mbar_try(bar, parity)) return true;
        if (*abort_flag) return false;
        if (i > 64) __nanosleep(64);
    }
    *abort_flag = 1;
    atomicOr(gflag, DEV_TIMEOUT);
    return false;
}

__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag, int *gflag)
{
    return mbar_wait_n(bar, parity, abort_flag, gflag, TC_SPIN_LIMIT);
}

__device__ __forceinline__ void mbar_arrive_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::
            "r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

// shared-memory matrix descriptor: K-major, 128B swizzle, 8-row atoms 1024 B apart
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)(16 >> 4) << 16;          // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;        // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1 << 46;                  // descriptor version (tcgen05)
    d |= (uint64_t)2 << 61;                  // SWIZZLE_128B
    return d;
}

// instruction descriptor: kind::tf32, D f32, A/B tf32, K-major both, M x N
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N)
{
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate)
{
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// kind::f16 with A/B fp16 (type 0), D f32: the same 11-bit operand significands
// as TF32, half the bytes, twice the rate
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N)
{
    return (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate)
{
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float v[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// PROMOTE = true: the K loop is cut into chunks of TC_PROMOTE_KB k-blocks; each
// chunk is accumulated by the tensor core into one of two TMEM buffers (2 x BN
// columns) and the epilogue warps add it into IEEE FP32 register accumulators
// while the MMA fills the other buffer.  The tensor core's own accumulation
// (coarser than an FMA chain) then only spans 64 products, which brings long-K
// products with cancellation (the CBF reduced matrix) to FP32-FMA accuracy.
// With H16 the operands are fp16 (the same 11-bit significands as TF32, half the
// bytes, twice the MMA rate): a k-block is 64 elements, and the caller sets the chunk
// (promote_kb k-blocks): two (128 products) where the product is final, four where an
// FP64-grade correction follows (the CBF residual updates under refinement, the
// reduced matrix before its FFT residual correction), which measured 16 % faster (the
// drain of two-block chunks holds up the MMA); alpha may be read from device memory
// (the inverse of the operands' power-of-two scales).
constexpr int TC_PROMOTE_KB = 2;
constexpr int TC_H16_STAGES = 6;


template <bool PROMOTE, int TC_STAGES, bool H16 = false>
__global__ void __launch_bounds__(TC_THREADS, TC_STAGES == 2 ? 2 : 1)
    k_gemm_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M, int N, int K,
              float *D, long long ldd, float alpha, float beta, int rnd, int *gflag, const float *alpha_dev = nullptr,
              int promote_kb = TC_PROMOTE_KB, int a_piece = 0)
{
    constexpr int BKE = H16 ? 2 * TC_BK : TC_BK;   // elements per k-block (128 bytes of a row)
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = (uint64_t *)(smem + TC_STAGES * TC_STAGE_BYTES);
    uint64_t *empty = full + TC_STAGES;
    uint64_t *accf = empty + TC_STAGES;     // [2]: chunk accumulated (tcgen05.commit)
    uint64_t *acce = accf + 2;              // [2]: chunk drained (128 epilogue arrivals)
    volatile uint32_t *tmem_slot = (volatile uint32_t *)(acce + 2);
    volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
    constexpr uint32_t NCOL = PROMOTE ? 2 * TC_BN : TC_BN;

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int m0 = blockIdx.y * TC_BM, n0 = blockIdx.x * TC_BN;
    const int nk = (K + BKE - 1) / BKE;
    const int KC = PROMOTE ? promote_kb : (nk > 0 ? nk : 1);
    const int nchunk = (nk + KC - 1) / KC;

    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        mbar_init(&accf[0], 1); mbar_init(&accf[1], 1);
        mbar_init(&acce[0], 128); mbar_init(&acce[1], 128);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmA) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmB) : "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32((const void *)tmem_slot)),
                     "r"(NCOL));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            for (int kb = 0; kb < nk; ++kb) {
                int s = kb % TC_STAGES;
                if (!mbar_wait(&empty[s], ((kb / TC_STAGES) + 1) & 1, abort_flag, gflag)) break;
                uint8_t *sa = smem + s * TC_STAGE_BYTES;
                uint8_t *sb = sa + TC_A_BYTES;
                mbar_arrive_tx(&full[s], TC_STAGE_BYTES);
                // two-piece A ([hi | lo], a_piece elements each): k >= a_piece reads A at k - a_piece,
                // so the hi piece serves the first two thirds of K (a_piece is a multiple of BKE)
                const int ka = kb * BKE;
                tma_load_2d(sa, &tmA, &full[s], (a_piece && ka >= a_piece) ? ka - a_piece : ka, m0);
                tma_load_2d(sb, &tmB, &full[s], ka, n0);
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = H16 ? idesc_f16(TC_BM, TC_BN) : idesc_tf32(TC_BM, TC_BN);
            bool ok = true;
            for (int ch = 0; ch < nchunk && ok; ++ch) {
                const int buf = PROMOTE ? (ch & 1) : 0;
                if (PROMOTE && ch >= 2)
                    if (!mbar_wait(&acce[buf], ((ch >> 1) - 1) & 1, abort_flag, gflag)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t dst = tmem + (uint32_t)(buf * TC_BN);
                const int kb1 = min(nk, (ch + 1) * KC);
                for (int kb = ch * KC; kb < kb1; ++kb) {
                    int s = kb % TC_STAGES;
                    if (!mbar_wait(&full[s], (kb / TC_STAGES) & 1, abort_flag, gflag)) { ok = false; break; }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    uint32_t sa = smem_u32(smem + s * TC_STAGE_BYTES);
                    uint32_t sb = sa + TC_A_BYTES;
#pragma unroll
                    for (int k4 = 0; k4 < TC_BK / 8; ++k4) {   // 32 bytes of K per MMA: 8 tf32 or 16 fp16
                        uint64_t ad = smem_desc_sw128(sa + k4 * 32);
                        uint64_t bd = smem_desc_sw128(sb + k4 * 32);
                        if constexpr (H16)
                            mma_f16(dst, ad, bd, idesc, (kb > ch * KC || k4 > 0) ? 1u : 0u);
                        else
                            mma_tf32(dst, ad, bd, idesc, (kb > ch * KC || k4 > 0) ? 1u : 0u);
                    }
                    mma_commit(&empty[s]);
                }
                mma_commit(&accf[buf]);
            }
        }
    } else {
        // epilogue: warp w reads TMEM lanes 32*(w%4) .. +31
        if (alpha_dev) alpha = *alpha_dev;   // set by an earlier kernel on the stream
        const int lg = warp % 4;
        const int row = m0 + lg * 32 + lane;
        const uint32_t lane_base = (uint32_t)(lg * 32) << 16;
        if (PROMOTE) {
            float acc[TC_BN];
#pragma unroll
            for (int j = 0; j < TC_BN; ++j) acc[j] = 0.f;
            bool ok = true;
            for (int ch = 0; ch < nchunk && ok; ++ch) {
                const int buf = ch & 1;
                ok = mbar_wait(&accf[buf], (ch >> 1) & 1, abort_flag, gflag);
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                if (!ok) break;
#pragma unroll
                for (int c = 0; c < TC_BN / 32; ++c) {
                    float v[32];
                    tmem_ld32(tmem + lane_base + (uint32_t)(buf * TC_BN + c * 32), v);
#pragma unroll
                    for (int j = 0; j < 32; ++j) acc[c * 32 + j] += v[j];
                }
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acce[buf])) : "memory");
            }
            if (ok && row < M) {
#pragma unroll
                for (int c = 0; c < TC_BN / 32; ++c) {
                    float *d = D + (long long)row * ldd + n0 + c * 32;
                    int ncol = N - (n0 + c * 32);
#pragma unroll
                    for (int j = 0; j < 32; ++j)
                        if (j < ncol) d[j] = alpha * acc[c * 32 + j] + (beta != 0.f ? beta * d[j] : 0.f);
                }
            }
        } else {
            bool ok = mbar_wait(&accf[0], 0, abort_flag, gflag);
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (ok) {
                // Every MMA has completed, so the stage buffers are free: each warp
                // stages its 32 rows x 32 columns in shared memory (one row per lane,
                // as tcgen05.ld delivers them) and writes them back row-contiguous:
                // a float4 store instruction covers 4 rows x 128 B of D.
                float *stg = (float *)smem + lg * 32 * TC_EPI_PITCH;
                const int rr = lane >> 3, cq = (lane & 7) * 4;
                const bool vec = ((((uintptr_t)D) | ((uintptr_t)ldd * 4)) & 15) == 0;
                for (int c = 0; c < TC_BN / 32; ++c) {
                    float v[32];
                    tmem_ld32(tmem + lane_base + (uint32_t)(c * 32), v);
#pragma unroll
                    for (int j = 0; j < 32; j += 4)
                        *(float4 *)(stg + lane * TC_EPI_PITCH + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
                    __syncwarp();
                    const int col = n0 + c * 32 + cq;
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const int r = i * 4 + rr, grow = m0 + lg * 32 + r;
                        if (grow >= M) continue;
                        float4 a = *(const float4 *)(stg + r * TC_EPI_PITCH + cq);
                        float *d = D + (long long)grow * ldd + col;
                        if (vec && col + 3 < N) {
                            float4 o;
                            if (beta != 0.f) {
                                float4 p = *(const float4 *)d;
                                o = make_float4(alpha * a.x + beta * p.x, alpha * a.y + beta * p.y,
                                                alpha * a.z + beta * p.z, alpha * a.w + beta * p.w);
                            } else {
                                o = make_float4(alpha * a.x, alpha * a.y, alpha * a.z, alpha * a.w);
                            }
                            if (rnd) o = make_float4(tf32_rna(o.x), tf32_rna(o.y), tf32_rna(o.z), tf32_rna(o.w));
                            *(float4 *)d = o;
                        } else {
                            const float av[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
                            for (int e = 0; e < 4; ++e)
                                if (col + e < N) {
                                    float o = alpha * av[e] + (beta != 0.f ? beta * d[e] : 0.f);
                                    d[e] = rnd ? tf32_rna(o) : o;
                                }
                        }
                    }
                    __syncwarp();
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(NCOL));
}


// ---------------------------------------------------------------------------
// Persistent tcgen05 GEMM for D = alpha A Bt^T + beta D (fp32 D, TMA-able):
// one CTA per SM walks the output tiles in groups of TCP_GROUP_M row tiles
// (so the CTAs running together share A and B tiles in L2).  Roles:
//   warp 0  TMA: the D tile of each output tile (4 boxes of 32 columns, 128B
//           swizzle) into one of DBUF buffers, then the A/B k-blocks;
//   warp 1  MMA: accumulates tile i into TMEM buffer i & 1 (2 x 128 columns),
//           so tile i+1 is computed while tile i is drained;
//   warps 2-5 epilogue: TMEM -> registers, alpha acc + beta D in the swizzled
//           D buffer (conflict-free), then one thread TMA-stores the buffer.
// Every wait is bounded; on expiry the CTA raises DEV_TIMEOUT and unwinds.
// ---------------------------------------------------------------------------
constexpr int TCP_GROUP_M = 16;
constexpr int TCP_D_BYTES = TC_BM * TC_BN * 4;   // one D tile (4 boxes of 16 KB)
__host__ __device__ constexpr int tcp_smem(int stages, int dbuf)
{
    return stages * TC_STAGE_BYTES + dbuf * TCP_D_BYTES + 1024 /*align*/ + 512 /*barriers*/;
}
static_assert(tcp_smem(4, 1) <= 227 * 1024 && tcp_smem(2, 2) <= 227 * 1024,
              "persistent GEMM exceeds the shared memory of one CTA");

__device__ __forceinline__ void tcp_tile(int t, int mt, int nt, int &m0, int &n0)
{
    const int per = TCP_GROUP_M * nt;
    const int first = (t / per) * TCP_GROUP_M;
    const int gsz = min(mt - first, TCP_GROUP_M);
    const int r = t % per;
    m0 = (first + r % gsz) * TC_BM;
    n0 = (r / gsz) * TC_BN;
}

// named barrier 1 over the 128 epilogue threads that also ANDs a flag, so every
// thread takes the same branch after a bounded wait
__device__ __forceinline__ bool epi_bar_and(bool ok)
{
    uint32_t r;
    asm volatile(
        "{\n.reg .pred p, q;\nsetp.ne.u32 q, %1, 0;\nbar.red.and.pred p, 1, 128, q;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)ok)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, const void *src, int x, int y)
{
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"((uint64_t)map),
                 "r"(x), "r"(y), "r"(smem_u32(src))
                 : "memory");
}

template <int STAGES, int DBUF, bool H16 = false>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_gemm_tcp(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
               const __grid_constant__ CUtensorMap tmD, int M, int N, int K, float alpha, float beta, int rnd,
               const float *alpha_dev, int *gflag)
{
    // one k-block = one 128-byte swizzle row of each operand row: 32 fp32 or 64 fp16
    constexpr int BKE = H16 ? 2 * TC_BK : TC_BK;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *dsm = smem + STAGES * TC_STAGE_BYTES;                 // DBUF x 64 KB, 1024-aligned
    uint64_t *full = (uint64_t *)(dsm + DBUF * TCP_D_BYTES);
    uint64_t *empty = full + STAGES;
    uint64_t *tfull = empty + STAGES;     // [2] accumulator ready
    uint64_t *tempty = tfull + 2;         // [2] accumulator drained (128 arrivals)
    uint64_t *dfull = tempty + 2;         // [DBUF] D tile loaded
    uint64_t *dempty = dfull + DBUF;      // [DBUF] D buffer stored back (1 arrival)
    volatile uint32_t *tmem_slot = (volatile uint32_t *)(dempty + DBUF);
    volatile int *abort_flag = (volatile int *)(tmem_slot + 1);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int mt = (M + TC_BM - 1) / TC_BM, nt = (N + TC_BN - 1) / TC_BN, ntiles = mt * nt;
    const int nk = (K + BKE - 1) / BKE;
    const bool use_d = beta != 0.f;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        for (int b = 0; b < 2; ++b) { mbar_init(&tfull[b], 1); mbar_init(&tempty[b], 128); }
        for (int b = 0; b < DBUF; ++b) { mbar_init(&dfull[b], 1); mbar_init(&dempty[b], 1); }
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmA) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmB) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmD) : "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32((const void *)tmem_slot)),
                     "r"(2 * TC_BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            long long kg = 0;
            int li = 0;
            bool ok = true;
            // D of tile li goes into buffer li % DBUF once the store of tile li - DBUF has
            // read it: with two buffers it is requested before the tile's k-blocks,
            // with one buffer after them (so the wait overlaps this tile's MMAs)
            auto load_d = [&](int li_, int m0_, int n0_) -> bool {
                const int db = li_ % DBUF;
                if (li_ >= DBUF && !mbar_wait(&dempty[db], ((li_ / DBUF) - 1) & 1, abort_flag, gflag)) return false;
                uint8_t *dst = dsm + db * TCP_D_BYTES;
                mbar_arrive_tx(&dfull[db], TCP_D_BYTES);
#pragma unroll
                for (int cch = 0; cch < TC_BN / 32; ++cch)
                    tma_load_2d(dst + cch * (TCP_D_BYTES / 4), &tmD, &dfull[db], n0_ + cch * 32, m0_);
                return true;
            };
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++li) {
                int m0, n0;
                tcp_tile(t, mt, nt, m0, n0);
                if (use_d && DBUF > 1 && !load_d(li, m0, n0)) break;
                for (int kb = 0; kb < nk; ++kb, ++kg) {
                    const int s = (int)(kg % STAGES);
                    if (!mbar_wait(&empty[s], (int)((kg / STAGES) + 1) & 1, abort_flag, gflag)) { ok = false; break; }
                    uint8_t *sa = smem + s * TC_STAGE_BYTES;
                    mbar_arrive_tx(&full[s], TC_STAGE_BYTES);
                    tma_load_2d(sa, &tmA, &full[s], kb * BKE, m0);
                    tma_load_2d(sa + TC_A_BYTES, &tmB, &full[s], kb * BKE, n0);
                }
                if (ok && use_d && DBUF == 1 && !load_d(li, m0, n0)) break;
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = H16 ? idesc_f16(TC_BM, TC_BN) : idesc_tf32(TC_BM, TC_BN);
            long long kg = 0;
            int li = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++li) {
                const int buf = li & 1;
                if (li >= 2 && !mbar_wait(&tempty[buf], ((li >> 1) - 1) & 1, abort_flag, gflag)) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t dst = tmem + (uint32_t)(buf * TC_BN);
                for (int kb = 0; kb < nk; ++kb, ++kg) {
                    const int s = (int)(kg % STAGES);
                    if (!mbar_wait(&full[s], (int)(kg / STAGES) & 1, abort_flag, gflag)) { ok = false; break; }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t sa = smem_u32(smem + s * TC_STAGE_BYTES), sb = sa + TC_A_BYTES;
#pragma unroll
                    for (int k4 = 0; k4 < 4; ++k4) {   // 32 bytes of K per MMA: 8 tf32 or 16 fp16
                        const uint64_t ad = smem_desc_sw128(sa + k4 * 32), bd = smem_desc_sw128(sb + k4 * 32);
                        const uint32_t acc = (kb > 0 || k4 > 0) ? 1u : 0u;
                        if constexpr (H16)
                            mma_f16(dst, ad, bd, idesc, acc);
                        else
                            mma_tf32(dst, ad, bd, idesc, acc);
                    }
                    mma_commit(&empty[s]);
                }
                if (ok) mma_commit(&tfull[buf]);
            }
        }
    } else {
        if (alpha_dev) alpha = *alpha_dev;               // set by an earlier kernel on the stream
        const int lg = warp % 4, et = threadIdx.x - 64;   // epilogue thread 0..127
        const int r = lg * 32 + lane;                     // tile row of this thread
        const uint32_t lane_base = (uint32_t)(lg * 32) << 16;
        int li = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++li) {
            int m0, n0;
            tcp_tile(t, mt, nt, m0, n0);
            const int buf = li & 1, db = li % DBUF;
            bool ok = mbar_wait(&tfull[buf], (li >> 1) & 1, abort_flag, gflag);
            if (ok && use_d) ok = mbar_wait(&dfull[db], (li / DBUF) & 1, abort_flag, gflag);
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (!epi_bar_and(ok)) break;
            uint8_t *dbase = dsm + db * TCP_D_BYTES;
#pragma unroll 1
            for (int cch = 0; cch < TC_BN / 32; ++cch) {
                float v[32];
                tmem_ld32(tmem + lane_base + (uint32_t)(buf * TC_BN + cch * 32), v);
                uint8_t *rowp = dbase + cch * (TCP_D_BYTES / 4) + r * 128;
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    float4 *p = (float4 *)(rowp + ((u ^ (r & 7)) << 4));
                    float4 o;
                    if (use_d) {
                        float4 d = *p;
                        o = make_float4(alpha * v[4 * u] + beta * d.x, alpha * v[4 * u + 1] + beta * d.y,
                                        alpha * v[4 * u + 2] + beta * d.z, alpha * v[4 * u + 3] + beta * d.w);
                    } else {
                        o = make_float4(alpha * v[4 * u], alpha * v[4 * u + 1], alpha * v[4 * u + 2],
                                        alpha * v[4 * u + 3]);
                    }
                    if (rnd) o = make_float4(tf32_rna(o.x), tf32_rna(o.y), tf32_rna(o.z), tf32_rna(o.w));
                    *p = o;
                }
            }
            // the accumulator buffer is free for tile li + 2
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&tempty[buf])) : "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("bar.sync 1, 128;" ::: "memory");
            if (et == 0) {
#pragma unroll
                for (int cch = 0; cch < TC_BN / 32; ++cch)
                    tma_store_2d(&tmD, dbase + cch * (TCP_D_BYTES / 4), n0 + cch * 32, m0);
                asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&dempty[db])) : "memory");
            }
            asm volatile("bar.sync 1, 128;" ::: "memory");
        }
        if (et == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC_BN));
}

// ---------------------------------------------------------------------------
// tensor-map creation through the driver entry point (no libcuda link needed)
// ---------------------------------------------------------------------------
typedef CUresult (*PFN_encodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                    const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static std::atomic<PFN_encodeTiled> g_encode{nullptr};

static int get_encode(midas_gpu_ctx *c)
{
    if (g_encode.load(std::memory_order_acquire)) return MIDAS_OK;
    cudaDriverEntryPointQueryResult q;
    void *fn = nullptr;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
        return c->err.set(MIDAS_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled entry point unavailable");
    g_encode.store((PFN_encodeTiled)fn, std::memory_order_release);
    return MIDAS_OK;
}

// rows x K operand (ld elements per row) in 128-byte boxes along K: fp32, or fp16 when h16
static int make_map(midas_gpu_ctx *c, CUtensorMap *m, const void *base, int rows, int K, long long ld, int box_rows,
                    bool h16 = false)
{
    const int es_bytes = h16 ? 2 : 4;
    cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * es_bytes};
    cuuint32_t box[2] = {(cuuint32_t)(128 / es_bytes), (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = g_encode.load(std::memory_order_acquire)(
                          m, h16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                          (void *)base, dims, strides, box, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return c->err.set(MIDAS_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    return MIDAS_OK;
}

const char *gemm_engine() { return "tcgen05"; }

bool gemm_tc_engine() { return true; }

// algorithmic bytes of one real GEMM: A and Bt once, D written (and read when beta != 0)
static double gemm_bytes(const GemmArgs &g)
{
    return 4.0 * ((double)g.M * g.K + (double)g.N * g.K + (double)g.M * g.N * (g.beta != 0.f ? 2 : 1));
}

static int gemm_simt(midas_gpu_ctx *c, const GemmArgs &g)
{
    dim3 grd((g.N + 63) / 64, (g.M + 63) / 64);
    ++c->launches;
    int kp = kp_begin(c);
    k_gemm_simt<<<grd, 256, 0, c->stream>>>(g);
    kp_end(c, kp, MIDAS_KC_GEMM_SIMT, 2.0 * g.M * g.N * g.K, gemm_bytes(g));
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// FP16-operand persistent GEMM (A, Bt fp16 with ld in fp16 elements; D fp32)
static int gemm_tcp_h16(midas_gpu_ctx *c, const GemmArgs &g)
{
    if ((((uintptr_t)g.D) & 15) || ((g.ldd * 4) & 15))
        return c->err.set(MIDAS_ERR_ARG, "gemm fp16: D must be a 16-byte aligned TMA operand");
    const int nsm = device_sms(c);
    static PerDeviceOnce once;
    MIDAS_CUDA(c, once.run(c->device, [] {
        cudaError_t e = cudaFuncSetAttribute(k_gemm_tcp<2, 2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             tcp_smem(2, 2));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_gemm_tcp<4, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     tcp_smem(4, 1));
        return e;
    }));
    CUtensorMap ma, mb, md;
    MIDAS_TRY(make_map(c, &ma, g.A, g.M, g.K, g.lda, TC_BM, true));
    MIDAS_TRY(make_map(c, &mb, g.Bt, g.N, g.K, g.ldb, TC_BN, true));
    MIDAS_TRY(make_map(c, &md, g.D, g.M, g.N, g.ldd, TC_BM));
    const long long ntiles = (long long)((g.M + TC_BM - 1) / TC_BM) * ((g.N + TC_BN - 1) / TC_BN);
    const int grid = (int)std::min<long long>(ntiles, nsm);
    ++c->launches;
    int kp = kp_begin(c);
    if (g.K <= 512)   // the k-block count of the fp32 K <= 256 case
        k_gemm_tcp<2, 2, true><<<grid, TC_THREADS, tcp_smem(2, 2), c->stream>>>(
            ma, mb, md, g.M, g.N, g.K, g.alpha, g.beta, g.round_tf32, g.alpha_dev, c->d_flag);
    else
        k_gemm_tcp<4, 1, true><<<grid, TC_THREADS, tcp_smem(4, 1), c->stream>>>(
            ma, mb, md, g.M, g.N, g.K, g.alpha, g.beta, g.round_tf32, g.alpha_dev, c->d_flag);
    kp_end(c, kp, g.kclass, 2.0 * g.M * g.N * g.K,
           2.0 * ((double)g.M * g.K + (double)g.N * g.K) + 4.0 * (double)g.M * g.N * (g.beta != 0.f ? 2 : 1));
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

static int gemm_tc(midas_gpu_ctx *c, const GemmArgs &g, bool precise)
{
    MIDAS_TRY(get_encode(c));
    const int ldm = g.h16 ? 7 : 3;
    if ((((uintptr_t)g.A) & 15) || (((uintptr_t)g.Bt) & 15) || (g.lda & ldm) || (g.ldb & ldm))
        return c->err.set(MIDAS_ERR_ARG, "gemm_tf32: operands must be 16-byte aligned with 16-byte row strides");
    if (g.h16 && precise) {   // fp16 operands, every k-block promoted to FP32 registers
        // 6 stages (192 KB): the long-K split products (K = 6 x 3 n_j halves) keep the
        // MMA warp fed while the epilogue warps promote
        static PerDeviceOnce once_h;
        MIDAS_CUDA(c, once_h.run(c->device, [] {
            return cudaFuncSetAttribute(k_gemm_tc<true, TC_H16_STAGES, true>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, tc_smem(TC_H16_STAGES));
        }));
        if (g.a_piece && (g.a_piece % (2 * TC_BK) || 3LL * g.a_piece != g.K))
            return c->err.set(MIDAS_ERR_ARG, "gemm_tf32: two-piece A needs K = 3 pieces of whole k-blocks");
        CUtensorMap ma, mb;
        MIDAS_TRY(make_map(c, &ma, g.A, g.M, g.a_piece ? (int)(2 * g.a_piece) : g.K, g.lda, TC_BM, true));
        MIDAS_TRY(make_map(c, &mb, g.Bt, g.N, g.K, g.ldb, TC_BN, true));
        dim3 grd((g.N + TC_BN - 1) / TC_BN, (g.M + TC_BM - 1) / TC_BM);
        ++c->launches;
        int kp = kp_begin(c);
        k_gemm_tc<true, TC_H16_STAGES, true><<<grd, TC_THREADS, tc_smem(TC_H16_STAGES), c->stream>>>(
            ma, mb, g.M, g.N, g.K, g.D, g.ldd, g.alpha, g.beta, 0, c->d_flag, g.alpha_dev,
            std::max(1, std::min(g.promote_kb, 16)), (int)g.a_piece);
        kp_end(c, kp, g.kclass, 2.0 * g.M * g.N * g.K,
               2.0 * ((double)g.M * g.K + (double)g.N * g.K) + 4.0 * (double)g.M * g.N * (g.beta != 0.f ? 2 : 1));
        MIDAS_CUDA(c, cudaGetLastError());
        return MIDAS_OK;
    }
    if (g.h16) return gemm_tcp_h16(c, g);
    static PerDeviceOnce once_tc;
    MIDAS_CUDA(c, once_tc.run(c->device, [] {
        cudaError_t e = cudaFuncSetAttribute(k_gemm_tc<false, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             tc_smem(4));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_gemm_tc<false, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_smem(2));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_gemm_tc<true, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_smem(4));
        return e;
    }));
    CUtensorMap ma, mb;
    MIDAS_TRY(make_map(c, &ma, g.A, g.M, g.K, g.lda, TC_BM));
    MIDAS_TRY(make_map(c, &mb, g.Bt, g.N, g.K, g.ldb, TC_BN));
    // persistent kernel whenever D can be a TMA operand
    if (!precise && !(((uintptr_t)g.D) & 15) && !((g.ldd * 4) & 15)) {
        const int nsm = device_sms(c);
        static PerDeviceOnce once_tcp;
        MIDAS_CUDA(c, once_tcp.run(c->device, [] {
            cudaError_t e = cudaFuncSetAttribute(k_gemm_tcp<2, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 tcp_smem(2, 2));
            if (e == cudaSuccess)
                e = cudaFuncSetAttribute(k_gemm_tcp<4, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         tcp_smem(4, 1));
            return e;
        }));
        CUtensorMap md;
        MIDAS_TRY(make_map(c, &md, g.D, g.M, g.N, g.ldd, TC_BM));
        const long long ntiles = (long long)((g.M + TC_BM - 1) / TC_BM) * ((g.N + TC_BN - 1) / TC_BN);
        const int grid = (int)std::min<long long>(ntiles, nsm);
        ++c->launches;
        int kp = kp_begin(c);
        if (g.K <= 256)
            k_gemm_tcp<2, 2><<<grid, TC_THREADS, tcp_smem(2, 2), c->stream>>>(
                ma, mb, md, g.M, g.N, g.K, g.alpha, g.beta, g.round_tf32, g.alpha_dev, c->d_flag);
        else   // long K: 4 stages, one D buffer (requested after the tile's k-blocks)
            k_gemm_tcp<4, 1><<<grid, TC_THREADS, tcp_smem(4, 1), c->stream>>>(
                ma, mb, md, g.M, g.N, g.K, g.alpha, g.beta, g.round_tf32, g.alpha_dev, c->d_flag);
        kp_end(c, kp, g.kclass, 2.0 * g.M * g.N * g.K, gemm_bytes(g));
        MIDAS_CUDA(c, cudaGetLastError());
        return MIDAS_OK;
    }
    dim3 grd((g.N + TC_BN - 1) / TC_BN, (g.M + TC_BM - 1) / TC_BM);
    ++c->launches;
    int kp = kp_begin(c);
    if (precise)
        k_gemm_tc<true, 4><<<grd, TC_THREADS, tc_smem(4), c->stream>>>(ma, mb, g.M, g.N, g.K, g.D, g.ldd, g.alpha,
                                                                       g.beta, 0, c->d_flag);
    else if (g.K <= 256)
        k_gemm_tc<false, 2><<<grd, TC_THREADS, tc_smem(2), c->stream>>>(ma, mb, g.M, g.N, g.K, g.D, g.ldd, g.alpha,
                                                                        g.beta, g.round_tf32, c->d_flag);
    else
        k_gemm_tc<false, 4><<<grd, TC_THREADS, tc_smem(4), c->stream>>>(ma, mb, g.M, g.N, g.K, g.D, g.ldd, g.alpha,
                                                                        g.beta, g.round_tf32, c->d_flag);
    kp_end(c, kp, g.kclass, 2.0 * g.M * g.N * g.K, gemm_bytes(g));
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

int gemm_tf32(midas_gpu_ctx *c, const GemmArgs &g, bool precise)
{
    if (g.M <= 0 || g.N <= 0) return MIDAS_OK;
    if (g.K <= 0) return c->err.set(MIDAS_ERR_ARG, "gemm_tf32: K must be positive");
    return gemm_tc(c, g, precise);
}

// ---------------------------------------------------------------------------
// complex operand expansion
// ---------------------------------------------------------------------------
__global__ void k_expand_b(int k, int n, const float2 *B, long long rsb, long long csb, float *Bt, long long ldt)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;   // along k (contiguous in Bt rows)
    if (p >= k) return;
    for (int j = blockIdx.y; j < n; j += gridDim.y) {   // columns beyond the 65535 grid limit loop
        float2 b = B[(long long)p * rsb + (long long)j * csb];
        b = make_float2(tf32_rna(b.x), tf32_rna(b.y));   // B operand: unbiased TF32
        float *r0 = Bt + (long long)(2 * j) * ldt + 2 * p;
        float *r1 = r0 + ldt;
        r0[0] = b.x; r0[1] = -b.y;
        r1[0] = b.y; r1[1] = b.x;
    }
}

int expand_b(midas_gpu_ctx *c, int k, int n, const float2 *B, long long rsb, long long csb, float *Bt, long long ldt)
{
    if (k <= 0 || n <= 0) return MIDAS_OK;
    dim3 grd((k + 127) / 128, std::min(n, 65535));
    ++c->launches;
    k_expand_b<<<grd, 128, 0, c->stream>>>(k, n, B, rsb, csb, Bt, ldt);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// device self-test: tcgen05 vs SIMT on a ragged problem (called by tests)
// ---------------------------------------------------------------------------
__global__ void k_fill_pattern(float *p, long long n, uint32_t seed)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t h = (uint32_t)i * 2654435761u ^ seed;
    h ^= h >> 13; h *= 0x5bd1e995u; h ^= h >> 15;
    p[i] = ((h & 0xFFFF) / 32768.0f) - 1.0f;
}

__global__ void k_to_h16(float *p, __half *h, long long n, float *alpha)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i == 0) *alpha = -1.f;
    if (i >= n) return;
    const __half v = __float2half_rn(p[i]);
    h[i] = v;
    p[i] = __half2float(v);
}

int gemm_selftest(midas_gpu_ctx *c)
{
    const int M = 300, N = 200, K = 136;   // ragged in every dimension
    size_t na = (size_t)M * K, nb = (size_t)N * K, nd = (size_t)M * N;
    void *buf;
    MIDAS_TRY(ensure(c, S_T32, sizeof(float) * (na + nb + 3 * nd + 64) + sizeof(__half) * (na + nb), &buf));
    float *A = (float *)buf, *B = A + na, *D0 = B + nb, *D1 = D0 + nd, *Di = D1 + nd, *dal = Di + nd;
    __half *A16 = (__half *)(dal + 64), *B16 = A16 + na;
    ++c->launches;
    k_fill_pattern<<<(unsigned)((na + 255) / 256), 256, 0, c->stream>>>(A, (long long)na, 1u);
    ++c->launches;
    k_fill_pattern<<<(unsigned)((nb + 255) / 256), 256, 0, c->stream>>>(B, (long long)nb, 7u);
    ++c->launches;
    k_fill_pattern<<<(unsigned)((nd + 255) / 256), 256, 0, c->stream>>>(Di, (long long)nd, 11u);
    std::vector<float> h0(nd), h1(nd);
    // leg 0: fp32 operands (tf32 MMAs) against the SIMT engine; leg 1: the same
    // operands rounded to fp16, kind::f16 MMAs with alpha read from device memory
    for (int leg = 0; leg < 2; ++leg) {
        if (leg == 1) {
            c->launches += 2;
            k_to_h16<<<(unsigned)((na + 255) / 256), 256, 0, c->stream>>>(A, A16, (long long)na, dal);
            k_to_h16<<<(unsigned)((nb + 255) / 256), 256, 0, c->stream>>>(B, B16, (long long)nb, dal);
        }
        MIDAS_CUDA(c, cudaMemcpyAsync(D0, Di, sizeof(float) * nd, cudaMemcpyDeviceToDevice, c->stream));
        MIDAS_CUDA(c, cudaMemcpyAsync(D1, Di, sizeof(float) * nd, cudaMemcpyDeviceToDevice, c->stream));
        GemmArgs g{M, N, K, A, K, B, K, D0, N, -1.0f, 1.0f};
        MIDAS_TRY(gemm_simt(c, g));
        g.D = D1;
        if (leg == 1) {
            g.A = (const float *)A16;
            g.Bt = (const float *)B16;
            g.h16 = 1;
            g.alpha = 0.f;   // must come from dal
            g.alpha_dev = dal;
        }
        MIDAS_TRY(gemm_tc(c, g, false));
        MIDAS_CUDA(c, cudaMemcpyAsync(h0.data(), D0, sizeof(float) * nd, cudaMemcpyDeviceToHost, c->stream));
        MIDAS_CUDA(c, cudaMemcpyAsync(h1.data(), D1, sizeof(float) * nd, cudaMemcpyDeviceToHost, c->stream));
        MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
        MIDAS_TRY(check_flag(c, "gemm_selftest"));
        double md = 0;
        for (size_t i = 0; i < nd; ++i) md = fmax(md, fabs((double)h0[i] - (double)h1[i]));
        // leg 0, TF32 operands: |err| <= K * 2^-10 * max|a||b| ~ 0.13 worst case, typical << 0.05;
        // leg 1, exact fp16 operands: products exact, only the fp32 summation order differs
        const double tol = leg == 0 ? 0.05 : 1e-3;
        if (!(md < tol)) {
            char msg[128];
            snprintf(msg, sizeof msg, "tcgen05 GEMM self-test mismatch (%s operands): max |diff| = %g",
                     leg == 0 ? "tf32" : "fp16", md);
            return c->err.set(MIDAS_ERR_CUDA, msg);
        }
    }
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// bounded-wait check: one CTA waits on an mbarrier that nothing arrives at, with
// `limit` polls, through the same mbar_wait_n the tensor-core kernels use.  The
// wait must expire, raise DEV_TIMEOUT in the context flag and let the kernel
// return; no asynchronous copy or TMEM allocation is in flight.
// ---------------------------------------------------------------------------
__global__ void k_wait_expire(uint32_t limit, int *gflag, int *polled)
{
    __shared__ __align__(8) uint64_t bar;
    __shared__ int abort_flag;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const bool ok = mbar_wait_n(&bar, 0, &abort_flag, gflag, limit);
        *polled = ok ? 0 : 1;
    }
    __syncthreads();
}

int wait_selftest(midas_gpu_ctx *c, int limit, int *expired)
{
    if (limit <= 0 || limit > (1 << 20)) return c->err.set(MIDAS_ERR_ARG, "wait_selftest: limit outside 1..2^20");
    void *buf;
    MIDAS_TRY(ensure(c, S_T32, 256, &buf));
    int *polled = (int *)buf;
    MIDAS_CUDA(c, cudaMemsetAsync(polled, 0, sizeof(int), c->stream));
    ++c->launches;
    k_wait_expire<<<1, 32, 0, c->stream>>>((uint32_t)limit, c->d_flag, polled);
    MIDAS_CUDA(c, cudaGetLastError());
    int h = 0;
    MIDAS_CUDA(c, cudaMemcpyAsync(&h, polled, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    *expired = h;
    return check_flag(c, "wait_selftest");
}

// Time `iters` launches of one M x N x K GEMM (D = D - A Bt^T) with CUDA events on
// the context stream; returns the average device time per launch in *ms.
int gemm_bench(midas_gpu_ctx *c, int M, int N, int K, int iters, double *ms, bool f16)
{
    if (M <= 0 || N <= 0 || K <= 0 || iters <= 0) return c->err.set(MIDAS_ERR_ARG, "bench_gemm: bad sizes");
    if (f16 && K % 8) return c->err.set(MIDAS_ERR_ARG, "bench_gemm: fp16 operands need K % 8 == 0");
    size_t na = (size_t)M * K, nb = (size_t)N * K, nd = (size_t)M * N;
    void *buf;
    MIDAS_TRY(ensure(c, S_T32, sizeof(float) * (na + nb + nd + 64) + sizeof(__half) * (na + nb) + 256, &buf));
    float *A = (float *)buf, *B = A + na, *D = B + nb, *dal = D + nd;
    __half *A16 = (__half *)(dal + 64), *B16 = A16 + na;
    ++c->launches;
    k_fill_pattern<<<(unsigned)((na + 255) / 256), 256, 0, c->stream>>>(A, (long long)na, 3u);
    ++c->launches;
    k_fill_pattern<<<(unsigned)((nb + 255) / 256), 256, 0, c->stream>>>(B, (long long)nb, 5u);
    MIDAS_CUDA(c, cudaMemsetAsync(D, 0, sizeof(float) * nd, c->stream));
    GemmArgs g{M, N, K, A, K, B, K, D, N, -1.0f, 1.0f};
    if (f16) {
        c->launches += 2;
        k_to_h16<<<(unsigned)((na + 255) / 256), 256, 0, c->stream>>>(A, A16, (long long)na, dal);
        k_to_h16<<<(unsigned)((nb + 255) / 256), 256, 0, c->stream>>>(B, B16, (long long)nb, dal);
        g.A = (const float *)A16;
        g.Bt = (const float *)B16;
        g.h16 = 1;
    }
    MIDAS_TRY(gemm_tf32(c, g));   // warm-up
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, c->stream);
    for (int i = 0; i < iters; ++i) MIDAS_TRY(gemm_tf32(c, g));
    cudaEventRecord(e1, c->stream);
    cudaEventSynchronize(e1);
    float t = 0;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    MIDAS_TRY(check_flag(c, "bench_gemm"));
    *ms = t / iters;
    return MIDAS_OK;
}

}  // namespace midas
