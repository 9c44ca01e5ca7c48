// sparse.cu -- CSR form of the thresholded (SR) extended-block matrix and the
// double-float refinement residual on it (sm_103a).
//
// The reference hands the SR-thresholded block to PARDISO as a CSR matrix
// (SR_Green_s_tr_partial, src/Green_functions.f90:290-562) and PARDISO's
// refinement steps form residuals with that sparse matrix.  Here the dense
// thresholded block is factorised on the tensor cores, and the residuals of
// the refinement use the CSR form built from it: about 16 % of the entries
// survive the threshold on the voxel scatterers of interest, so the residual
// does a sixth of the dense work.
#include <cstdlib>

#include "common.cuh"
#include "kernels.cuh"

namespace midas {

// nonzeros per row of a dense row-major complex64 matrix (warp per row)
__global__ void k_csr_count(int n, const float2 *Z, long long ldz, int *cnt)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= n) return;
    const float2 *row = Z + (long long)w * ldz;
    int c = 0;
    for (int k = lane; k < n; k += 32) {
        float2 v = row[k];
        c += (v.x != 0.f || v.y != 0.f);
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if (lane == 0) cnt[w] = c;
}

// exclusive scan of cnt[0..n) into rowptr[0..n] (one CTA of 1024 threads)
__global__ void __launch_bounds__(1024) k_scan_rowptr(int n, const int *cnt, int *rowptr)
{
    __shared__ int part[32];
    __shared__ long long carry;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < n; base += 1024) {
        int v = base + tid < n ? cnt[base + tid] : 0;
        int x = v;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) part[w] = x;
        __syncthreads();
        if (w == 0) {
            int p = part[lane];
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, p, o);
                if (lane >= o) p += y;
            }
            part[lane] = p;
        }
        __syncthreads();
        int incl = x + (w > 0 ? part[w - 1] : 0);
        if (base + tid < n) rowptr[base + tid] = (int)(carry + incl - v);
        __syncthreads();
        if (tid == 1023) carry += incl;
        __syncthreads();
    }
    if (tid == 0) rowptr[n] = carry > 0x7fffffffLL ? -1 : (int)carry;   // -1: too many entries for int32
}

// column indices and values of the nonzeros, in column order (warp per row)
__global__ void k_csr_fill(int n, const float2 *Z, long long ldz, const int *rowptr, int *col, float2 *val)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= n) return;
    const float2 *row = Z + (long long)w * ldz;
    int pos = rowptr[w];
    for (int k0 = 0; k0 < n; k0 += 32) {
        int k = k0 + lane;
        float2 v = k < n ? row[k] : make_float2(0.f, 0.f);
        bool nz = (v.x != 0.f || v.y != 0.f);
        unsigned m = __ballot_sync(0xffffffffu, nz);
        if (nz) {
            int p = pos + __popc(m & ((1u << lane) - 1u));
            col[p] = k;
            val[p] = v;
        }
        pos += __popc(m);
    }
}

int csr_from_dense(midas_gpu_ctx *c, int n, const float2 *Z, long long ldz, int slot, Csr *out)
{
    void *p;
    MIDAS_TRY(ensure(c, S_RED, sizeof(int) * ((size_t)2 * n + 8), &p));
    int *cnt = (int *)p, *rp_tmp = cnt + n + 4;
    unsigned blocks = (unsigned)(((long long)n * 32 + 255) / 256);
    ++c->launches;
    k_csr_count<<<blocks, 256, 0, c->stream>>>(n, Z, ldz, cnt);
    ++c->launches;
    k_scan_rowptr<<<1, 1024, 0, c->stream>>>(n, cnt, rp_tmp);
    MIDAS_CUDA(c, cudaGetLastError());
    int nnz = 0;
    MIDAS_CUDA(c, cudaMemcpyAsync(&nnz, rp_tmp + n, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (nnz < 0) return c->err.set(MIDAS_ERR_UNSUPPORTED, "csr: more than 2^31 nonzeros");
    const size_t rp_bytes = ((sizeof(int) * ((size_t)n + 1)) + 255) & ~(size_t)255;
    const size_t col_bytes = ((sizeof(int) * (size_t)nnz) + 255) & ~(size_t)255;
    MIDAS_TRY(ensure(c, slot, rp_bytes + col_bytes + sizeof(float2) * (size_t)nnz, &p));
    out->n = n;
    out->nnz = nnz;
    out->rowptr = (int *)p;
    out->col = (int *)((char *)p + rp_bytes);
    out->val = (float2 *)((char *)p + rp_bytes + col_bytes);
    MIDAS_CUDA(c, cudaMemcpyAsync(out->rowptr, rp_tmp, sizeof(int) * ((size_t)n + 1), cudaMemcpyDeviceToDevice,
                                  c->stream));
    ++c->launches;
    k_csr_fill<<<blocks, 256, 0, c->stream>>>(n, Z, ldz, out->rowptr, out->col, out->val);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// r = B - Z (Xh + Xl) with Z in CSR form.  Xh, Xl row-major (n x m), B
// column-major float (ld n), r column-major FP64 (ld n).  A warp per row; the
// lanes run over RESID_COLS right-hand sides (blockIdx.y selects the group),
// each holding RESID_COLS / 32 double-float accumulators.  The products with
// Xh are exact (fma residue) and summed in double-float; the products with Xl
// (2^-24 smaller) are summed in FP32.
// ---------------------------------------------------------------------------
constexpr int RESID_COLS = 96;
constexpr int RESID_T = RESID_COLS / 32;

__global__ void __launch_bounds__(256) k_resid_csr_df32(int n, int m, const int *rowptr, const int *col,
                                                         const float2 *val, const float2 *Xh, const float2 *Xl,
                                                         const float2 *B, double2 *R)
{
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (i >= n) return;
    const int c0 = blockIdx.y * RESID_COLS;
    float rh[RESID_T], rl[RESID_T], ih[RESID_T], il[RESID_T], cr[RESID_T], ci[RESID_T];
#pragma unroll
    for (int t = 0; t < RESID_T; ++t) { rh[t] = rl[t] = ih[t] = il[t] = cr[t] = ci[t] = 0.f; }
    const int p1 = rowptr[i + 1];
    // the row's (column, value) pairs are read 32 at a time, one per lane, and
    // broadcast with shuffles, so the X gathers do not wait on index loads
    for (int p0 = rowptr[i]; p0 < p1; p0 += 32) {
        const int cnt = min(32, p1 - p0);
        int mk = 0;
        float2 mz = make_float2(0.f, 0.f);
        if (lane < cnt) { mk = col[p0 + lane]; mz = val[p0 + lane]; }
#pragma unroll 4
        for (int q = 0; q < cnt; ++q) {
            const int k = __shfl_sync(0xffffffffu, mk, q);
            float2 z;
            z.x = __shfl_sync(0xffffffffu, mz.x, q);
            z.y = __shfl_sync(0xffffffffu, mz.y, q);
            const float2 *xh = Xh + (long long)k * m, *xl = Xl + (long long)k * m;
#pragma unroll
            for (int t = 0; t < RESID_T; ++t) {
                const int cc = c0 + lane + 32 * t;
                if (cc < m) {
                    float2 h = xh[cc], l = xl[cc];
                    df_fma(rh[t], rl[t], z.x, h.x);
                    df_fma(rh[t], rl[t], -z.y, h.y);
                    df_fma(ih[t], il[t], z.x, h.y);
                    df_fma(ih[t], il[t], z.y, h.x);
                    cr[t] += z.x * l.x - z.y * l.y;
                    ci[t] += z.x * l.y + z.y * l.x;
                }
            }
        }
    }
#pragma unroll
    for (int t = 0; t < RESID_T; ++t) {
        const int cc = c0 + lane + 32 * t;
        if (cc < m) {
            double zr = (double)rh[t] + (double)rl[t] + (double)cr[t];
            double zi = (double)ih[t] + (double)il[t] + (double)ci[t];
            float2 b = B[(long long)cc * n + i];
            R[(long long)cc * n + i] = make_double2((double)b.x - zr, (double)b.y - zi);
        }
    }
}

// ---------------------------------------------------------------------------
// The same residual with the lanes over the row's nonzeros: a warp takes one
// row and RL_T consecutive right-hand sides; each lane walks every 32nd
// nonzero of the row (one coalesced index and value load) and accumulates its
// RL_T columns from four float4 loads of Xh and of Xl, so the per-nonzero work
// is the arithmetic alone.  The 32 lanes' double-float partial sums are then
// added by a shuffle tree of TwoSums.  m must be even (X rows start on 16-byte
// boundaries): the CBF right-hand sides come in V / H pairs.
// ---------------------------------------------------------------------------
constexpr int RL_T = 8;

// (hi, lo) += a (bh + bl): the product with bh exactly (FMA residue, TwoSum into
// hi), the product with bl (2^-24 smaller) in FP32 into lo
__device__ __forceinline__ void df_axpy(float &hi, float &lo, float a, float bh, float bl)
{
    const float p = __fmul_rn(a, bh);
    const float pe = fmaf(a, bh, -p);
    float sum, err;
    ef_two_sum(hi, p, sum, err);
    hi = sum;
    lo = fmaf(a, bl, __fadd_rn(lo, __fadd_rn(err, pe)));
}

__device__ __forceinline__ void load_row8(const float2 *X, long long base, int ncols, float2 v[RL_T])
{
    if (ncols == RL_T) {
        const float4 *q = (const float4 *)(X + base);
#pragma unroll
        for (int u = 0; u < RL_T / 2; ++u) {
            const float4 w = q[u];
            v[2 * u] = make_float2(w.x, w.y);
            v[2 * u + 1] = make_float2(w.z, w.w);
        }
    } else {
#pragma unroll
        for (int t = 0; t < RL_T; ++t) v[t] = t < ncols ? X[base + t] : make_float2(0.f, 0.f);
    }
}

__global__ void __launch_bounds__(256) k_resid_csr_df32_nz(int n, int m, const int *rowptr, const int *col,
                                                            const float2 *val, const float2 *Xh, const float2 *Xl,
                                                            const float2 *B, double2 *R)
{
    const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int ntile = (m + RL_T - 1) / RL_T;
    if (w >= (long long)n * ntile) return;
    const int i = (int)(w / ntile), c0 = (int)(w % ntile) * RL_T, ncols = min(RL_T, m - c0);
    float rh[RL_T], rl[RL_T], ih[RL_T], il[RL_T];
#pragma unroll
    for (int t = 0; t < RL_T; ++t) rh[t] = rl[t] = ih[t] = il[t] = 0.f;
    const int p1 = rowptr[i + 1];
    for (int p = rowptr[i] + lane; p < p1; p += 32) {
        const int k = col[p];
        const float2 z = val[p];
        float2 h[RL_T], l[RL_T];
        load_row8(Xh, (long long)k * m + c0, ncols, h);
        load_row8(Xl, (long long)k * m + c0, ncols, l);
#pragma unroll
        for (int t = 0; t < RL_T; ++t) {
            df_axpy(rh[t], rl[t], z.x, h[t].x, l[t].x);
            df_axpy(rh[t], rl[t], -z.y, h[t].y, l[t].y);
            df_axpy(ih[t], il[t], z.x, h[t].y, l[t].y);
            df_axpy(ih[t], il[t], z.y, h[t].x, l[t].x);
        }
    }
    // the lanes' double-float partial sums: a shuffle tree of TwoSums
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int t = 0; t < RL_T; ++t) {
            float sum, err;
            const float oh = __shfl_down_sync(0xffffffffu, rh[t], o), ol = __shfl_down_sync(0xffffffffu, rl[t], o);
            ef_two_sum(rh[t], oh, sum, err);
            rh[t] = sum;
            rl[t] = __fadd_rn(rl[t], __fadd_rn(err, ol));
            const float jh = __shfl_down_sync(0xffffffffu, ih[t], o), jl = __shfl_down_sync(0xffffffffu, il[t], o);
            ef_two_sum(ih[t], jh, sum, err);
            ih[t] = sum;
            il[t] = __fadd_rn(il[t], __fadd_rn(err, jl));
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int t = 0; t < RL_T; ++t)
            if (t < ncols) {
                const float2 b = B[(long long)(c0 + t) * n + i];
                R[(long long)(c0 + t) * n + i] = make_double2((double)b.x - ((double)rh[t] + (double)rl[t]),
                                                              (double)b.y - ((double)ih[t] + (double)il[t]));
            }
    }
}

// r -= Z d in FP32 with the same lane layout
__global__ void __launch_bounds__(256) k_csr_sub_f32_nz(int n, int m, const int *rowptr, const int *col,
                                                         const float2 *val, const float2 *D, double2 *R)
{
    const long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int ntile = (m + RL_T - 1) / RL_T;
    if (w >= (long long)n * ntile) return;
    const int i = (int)(w / ntile), c0 = (int)(w % ntile) * RL_T, ncols = min(RL_T, m - c0);
    float ar[RL_T], ai[RL_T];
#pragma unroll
    for (int t = 0; t < RL_T; ++t) ar[t] = ai[t] = 0.f;
    const int p1 = rowptr[i + 1];
    for (int p = rowptr[i] + lane; p < p1; p += 32) {
        const int k = col[p];
        const float2 z = val[p];
        float2 d[RL_T];
        load_row8(D, (long long)k * m + c0, ncols, d);
#pragma unroll
        for (int t = 0; t < RL_T; ++t) {
            ar[t] = fmaf(z.x, d[t].x, fmaf(-z.y, d[t].y, ar[t]));
            ai[t] = fmaf(z.x, d[t].y, fmaf(z.y, d[t].x, ai[t]));
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int t = 0; t < RL_T; ++t) {
            ar[t] += __shfl_down_sync(0xffffffffu, ar[t], o);
            ai[t] += __shfl_down_sync(0xffffffffu, ai[t], o);
        }
    if (lane == 0) {
#pragma unroll
        for (int t = 0; t < RL_T; ++t)
            if (t < ncols) {
                double2 *r = R + (long long)(c0 + t) * n + i;
                *r = make_double2(r->x - (double)ar[t], r->y - (double)ai[t]);
            }
    }
}

static bool csr_lanes_over_columns()
{
    static const bool v = getenv("MIDAS_CSR_COLUMN_LANES") != nullptr;
    return v;
}

int residual_csr_df32(midas_gpu_ctx *c, const Csr &Z, int m, const float2 *Xh_rm, const float2 *Xl_rm,
                      const float2 *B, double2 *R)
{
    const int n = Z.n;
    ++c->launches;
    int kp = kp_begin(c);
    if (csr_lanes_over_columns() || (m & 1)) {
        dim3 grd((unsigned)(((long long)n * 32 + 255) / 256), (m + RESID_COLS - 1) / RESID_COLS);
        k_resid_csr_df32<<<grd, 256, 0, c->stream>>>(n, m, Z.rowptr, Z.col, Z.val, Xh_rm, Xl_rm, B, R);
    } else {
        const long long warps = (long long)n * ((m + RL_T - 1) / RL_T);
        k_resid_csr_df32_nz<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, c->stream>>>(n, m, Z.rowptr, Z.col,
                                                                                           Z.val, Xh_rm, Xl_rm, B, R);
    }
    kp_end(c, kp, MIDAS_KC_RESID, 8.0 * Z.nnz * m, 12.0 * Z.nnz + 16.0 * (double)n * m * 2 + 24.0 * (double)n * m);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// r -= Z d (FP32): the residual of x + d from the residual of x, once the
// correction d is small -- its FP32 product error is then below the double-float
// accuracy the refinement needs.  d row-major (n x m), r column-major FP64.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_csr_sub_f32(int n, int m, const int *rowptr, const int *col,
                                                      const float2 *val, const float2 *D, double2 *R)
{
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (i >= n) return;
    const int c0 = blockIdx.y * RESID_COLS;
    float ar[RESID_T], ai[RESID_T];
#pragma unroll
    for (int t = 0; t < RESID_T; ++t) { ar[t] = 0.f; ai[t] = 0.f; }
    const int p1 = rowptr[i + 1];
    for (int p0 = rowptr[i]; p0 < p1; p0 += 32) {
        const int cnt = min(32, p1 - p0);
        int mk = 0;
        float2 mz = make_float2(0.f, 0.f);
        if (lane < cnt) { mk = col[p0 + lane]; mz = val[p0 + lane]; }
#pragma unroll 4
        for (int q = 0; q < cnt; ++q) {
            const int k = __shfl_sync(0xffffffffu, mk, q);
            float2 z;
            z.x = __shfl_sync(0xffffffffu, mz.x, q);
            z.y = __shfl_sync(0xffffffffu, mz.y, q);
            const float2 *dr = D + (long long)k * m;
#pragma unroll
            for (int t = 0; t < RESID_T; ++t) {
                const int cc = c0 + lane + 32 * t;
                if (cc < m) {
                    float2 d = dr[cc];
                    ar[t] = fmaf(z.x, d.x, fmaf(-z.y, d.y, ar[t]));
                    ai[t] = fmaf(z.x, d.y, fmaf(z.y, d.x, ai[t]));
                }
            }
        }
    }
#pragma unroll
    for (int t = 0; t < RESID_T; ++t) {
        const int cc = c0 + lane + 32 * t;
        if (cc < m) {
            double2 *r = R + (long long)cc * n + i;
            *r = make_double2(r->x - (double)ar[t], r->y - (double)ai[t]);
        }
    }
}

int residual_csr_update_f32(midas_gpu_ctx *c, const Csr &Z, int m, const float2 *D_rm, double2 *R)
{
    const int n = Z.n;
    ++c->launches;
    int kp = kp_begin(c);
    if (csr_lanes_over_columns() || (m & 1)) {
        dim3 grd((unsigned)(((long long)n * 32 + 255) / 256), (m + RESID_COLS - 1) / RESID_COLS);
        k_csr_sub_f32<<<grd, 256, 0, c->stream>>>(n, m, Z.rowptr, Z.col, Z.val, D_rm, R);
    } else {
        const long long warps = (long long)n * ((m + RL_T - 1) / RL_T);
        k_csr_sub_f32_nz<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, c->stream>>>(n, m, Z.rowptr, Z.col, Z.val,
                                                                                        D_rm, R);
    }
    kp_end(c, kp, MIDAS_KC_RESID, 8.0 * Z.nnz * m, 12.0 * Z.nnz + 8.0 * (double)n * m + 32.0 * (double)n * m);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

}  // namespace midas
