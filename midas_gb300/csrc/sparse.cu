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
// r = B - Z (Xh + Xl) with Z in CSR form.  Xh, Xl row-major (n rows of ldx, ldx a
// multiple of CSR_RESID_COLS), B column-major float (ld n), r column-major FP64
// (ld n).  A warp per row; the lanes run over CSR_RESID_COLS right-hand sides
// (blockIdx.y selects the group: one group's X, gathered by column index, then stays
// in L2 beside the streamed CSR entries -- with the groups of a row block side by side
// the X of both groups thrashed L2, DRAM reads 3.8 -> 34 GB on a 15k-row block, at the
// same issue-bound time), CSR_T per lane, so the per-nonzero work (the
// shuffle broadcast of the column offset and the value) is shared by 6 complex
// multiply-adds.  The products with Xh are exact (FMA TwoProduct) and summed by
// TwoSum; the products with Xl (2^-24 smaller) are added in FP32 into the same
// low word.  The padded columns of X are read but never stored.
// ---------------------------------------------------------------------------
constexpr int CSR_T = CSR_RESID_COLS / 32;

// (hi, lo) += a (bh + bl) with a exact: a bh exactly, a bl in FP32 into lo
__device__ __forceinline__ void df_fma_lo(float &hi, float &lo, float a, float bh, float bl)
{
    const float p = __fmul_rn(a, bh);
    float pe = fmaf(a, bh, -p);
    pe = fmaf(a, bl, pe);
    float s, e;
    ef_two_sum(hi, p, s, e);
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(e, pe));
}

__global__ void __launch_bounds__(256) k_resid_csr_df32(int n, int m, int ldx, const int *rowptr, const int *col,
                                                         const float2 *val, const float2 *Xh, const float2 *Xl,
                                                         const float2 *B, double2 *R)
{
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (i >= n) return;
    const int c0 = blockIdx.y * CSR_RESID_COLS + lane;
    float rh[CSR_T], rl[CSR_T], ih[CSR_T], il[CSR_T];
#pragma unroll
    for (int t = 0; t < CSR_T; ++t) rh[t] = rl[t] = ih[t] = il[t] = 0.f;
    const int p1 = rowptr[i + 1];
    const float2 *xh0 = Xh + c0, *xl0 = Xl + c0;
    // the row's (column, value) pairs are read 32 at a time, one per lane, and
    // broadcast with shuffles, so the X gathers do not wait on index loads
    for (int p0 = rowptr[i]; p0 < p1; p0 += 32) {
        const int cnt = min(32, p1 - p0);
        int mk = 0;   // row offset of X (n ldx < 2^31, checked by the launcher)
        float2 mz = make_float2(0.f, 0.f);
        if (lane < cnt) { mk = col[p0 + lane] * ldx; mz = val[p0 + lane]; }
#pragma unroll 2
        for (int q = 0; q < cnt; ++q) {
            const int k = __shfl_sync(0xffffffffu, mk, q);
            const float zx = __shfl_sync(0xffffffffu, mz.x, q), zy = __shfl_sync(0xffffffffu, mz.y, q);
            const float2 *xh = xh0 + k, *xl = xl0 + k;
            float2 h[CSR_T], l[CSR_T];
#pragma unroll
            for (int t = 0; t < CSR_T; ++t) { h[t] = xh[32 * t]; l[t] = xl[32 * t]; }
#pragma unroll
            for (int t = 0; t < CSR_T; ++t) {
                df_fma_lo(rh[t], rl[t], zx, h[t].x, l[t].x);
                df_fma_lo(rh[t], rl[t], -zy, h[t].y, l[t].y);
                df_fma_lo(ih[t], il[t], zx, h[t].y, l[t].y);
                df_fma_lo(ih[t], il[t], zy, h[t].x, l[t].x);
            }
        }
    }
#pragma unroll
    for (int t = 0; t < CSR_T; ++t) {
        const int cc = c0 + 32 * t;
        if (cc < m) {
            const float2 b = B[(long long)cc * n + i];
            R[(long long)cc * n + i] = make_double2((double)b.x - ((double)rh[t] + (double)rl[t]),
                                                    (double)b.y - ((double)ih[t] + (double)il[t]));
        }
    }
}

int residual_csr_df32(midas_gpu_ctx *c, const Csr &Z, int m, int ldx, const float2 *Xh_rm, const float2 *Xl_rm,
                      const float2 *B, double2 *R)
{
    const int n = Z.n;
    if (ldx < m || ldx % CSR_RESID_COLS) return c->err.set(MIDAS_ERR_ARG, "csr residual: bad X row stride");
    if ((long long)n * ldx >= (1LL << 31)) return c->err.set(MIDAS_ERR_UNSUPPORTED, "csr residual: X above 2^31 entries");
    ++c->launches;
    int kp = kp_begin(c);
    dim3 grd((unsigned)(((long long)n * 32 + 255) / 256), (m + CSR_RESID_COLS - 1) / CSR_RESID_COLS);
    k_resid_csr_df32<<<grd, 256, 0, c->stream>>>(n, m, ldx, Z.rowptr, Z.col, Z.val, Xh_rm, Xl_rm, B, R);
    kp_end(c, kp, MIDAS_KC_RESID, 8.0 * Z.nnz * m, 12.0 * Z.nnz + 16.0 * (double)n * m * 2 + 24.0 * (double)n * m);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

}  // namespace midas
