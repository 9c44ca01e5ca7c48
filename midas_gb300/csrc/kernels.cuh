// kernels.cuh -- internal launcher prototypes shared between translation units.
#pragma once
#include <cuda_fp16.h>

#include "common.cuh"

namespace midas {

// CUDA-event timer on a stream (device time between construction and stop()).
struct Timer {
    cudaEvent_t a, b;
    cudaStream_t s;
    explicit Timer(cudaStream_t st) : s(st) { cudaEventCreate(&a); cudaEventCreate(&b); cudaEventRecord(a, s); }
    float stop()
    {
        float ms = 0;
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(&ms, a, b);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        return ms;
    }
};

// aca.cu: one block pair of the ACA batch -- cells [r0, r0+ni) x [c0, c0+nj);
// U and V of the pair start at element offsets uoff / voff of the batch arrays.
constexpr int ACA_MAX_IT = 128;
struct AcaPair {
    int r0, ni, c0, nj;
    long long uoff, voff;
};
int aca_batch(midas_gpu_ctx *c, int npairs, const AcaPair *d_pairs, double eps, int itmax, double2 *U, double2 *V,
              int *d_rank);
int aca_uw(midas_gpu_ctx *c, int nrows, int k, int ncol, const double2 *U, const double2 *W, float2 *T, long long ldt);
int aca_run(midas_gpu_ctx *c, int row0, int nrows, int col0, int ncols, double eps, int itmax, double2 *U,
            double2 *V, int *rank);
// cbfm.cu: release the CBFM lanes of a context
void free_lanes(midas_gpu_ctx *c);

// blas.cu: one product C = A B of a batched double-float complex GEMM (element (i, k)
// of A at A[i ars + k acs], and likewise B and C); zgemm_df_batched sets kchunk, poff
// and eoff
struct ZdfJob {
    int M, N, K, kchunk;
    const double2 *A;
    long long ars, acs;
    const double2 *B;
    long long brs, bcs;
    double2 *C;
    long long crs, ccs;
    long long poff, eoff;
};
int zgemm_df_batched(midas_gpu_ctx *c, std::vector<ZdfJob> &jobs);

// sparse.cu: CSR matrix (0-based, columns ascending within a row)
struct Csr {
    int n = 0, nnz = 0;
    int *rowptr = nullptr, *col = nullptr;
    float2 *val = nullptr;
};
int csr_from_dense(midas_gpu_ctx *c, int n, const float2 *Z, long long ldz, int slot, Csr *out);
// right-hand sides per warp pass of the CSR residual; X rows are padded to a multiple
constexpr int CSR_RESID_COLS = 192;
inline int csr_resid_ldx(int m) { return (m + CSR_RESID_COLS - 1) / CSR_RESID_COLS * CSR_RESID_COLS; }
int residual_csr_df32(midas_gpu_ctx *c, const Csr &Z, int m, int ldx, const float2 *Xh_rm, const float2 *Xl_rm,
                      const float2 *B, double2 *R);

// fill.cu
int launch_set_cells(midas_gpu_ctx *c);
int launch_lat_table(midas_gpu_ctx *c);
int launch_mom_fill(midas_gpu_ctx *c, int r0, int nr, int c0, int nc, double2 *out, float2 *out32, size_t rs,
                    size_t cs);
template <typename T>
int launch_mom_rhs(midas_gpu_ctx *c, int ntr, const double *th, const double *ph, T *V, size_t rs, size_t cs);
template <typename T>
int launch_incident4(midas_gpu_ctx *c, int ncell, const int *idx, int ntr, const double *th, const double *ph, T *E,
                     size_t rs, size_t cs);
template <typename T>
int launch_incident_sph(midas_gpu_ctx *c, int ncell, const int *idx, int ntr, const double *th, const double *ph,
                        T *E, size_t rs, size_t cs);
template <typename T>
int launch_block_fill4(midas_gpu_ctx *c, int n1, const int *idx1, int n2, const int *idx2, int mode, double thr,
                       int homog, T *out, size_t rs, size_t cs);
// Z(idx1 rows, idx2 cols) (mode 0) written as the split-TF32 A operand (hi | hi | lo), or
// with A3h as the fp16 [hi | lo] operand (lda3 = h16_arow(3 n2) halves, pieces scaled by hscale)
int launch_block_fill4_a3(midas_gpu_ctx *c, int n1, const int *idx1, int n2, const int *idx2, float *A3,
                          long long lda3, __half *A3h = nullptr, float hscale = 1.f);
// upper bound of |Z| over the lattice-table fill (0 when the fill is direct)
int fill4_bound(midas_gpu_ctx *c, double *bound);
int sr_ladder(midas_gpu_ctx *c, int s_n, const int *d_idx, int first_cell, int homog, double res_sr, double *fsr_out,
              long long *nnz_out, int want_all, double *all_nnz, double *all_fn, double *fnz_out);

// gemm.cu : D[M x N] = alpha * A[M x K] * Bt[N x K]^T + beta * D   (all fp32, row-major,
// K contiguous for A and Bt).  Complex products use the real embedding: A is the
// interleaved complex matrix (K = 2k), Bt the expanded operand (N = 2n, see expand_b).
struct GemmArgs {
    int M, N, K;
    const float *A; long long lda;
    const float *Bt; long long ldb;
    float *D; long long ldd;
    float alpha, beta;
    int round_tf32 = 0;   // store D rounded to TF32 (final L / U factor entries)
    int kclass = MIDAS_KC_GEMM_TC;   // kernel class for the profiler
    int h16 = 0;                     // A, Bt are fp16 (__half*, ld in fp16 elements): kind::f16 MMAs
    const float *alpha_dev = nullptr;   // when set, alpha is read from device memory at launch
    int promote_kb = 2;   // h16 precise products: k-blocks (64 products each) per FP32 promotion
    long long a_piece = 0;   // h16 precise products: A is [hi | lo] of a_piece elements each, K = 3 a_piece
};

// fp16 split operands.  A row of the A operand holds the hi piece, then the lo piece, of
// its K complex entries (re, im interleaved), each piece h16_piece(K) complex entries (a
// multiple of 32, so that a piece is whole 64-half k-blocks; the tail is zero).  B3 rows
// hold [hi | lo | hi] pieces of the same width, and the GEMM reads A's hi piece twice:
// hi.hi + hi.lo + lo.hi.
__host__ __device__ inline long long h16_piece(long long K) { return (K + 31) / 32 * 32; }
__host__ __device__ inline long long h16_arow(long long K) { return 4 * h16_piece(K); }   // halves per A row
__host__ __device__ inline long long h16_brow(long long K) { return 6 * h16_piece(K); }   // halves per B3 row: the GEMM's K
bool gemm_tc_engine();   // the tcgen05 engine is selected (required for h16 operands)
// precise = periodic promotion of the tensor-core partial sums to FP32 registers
int gemm_tf32(midas_gpu_ctx *c, const GemmArgs &g, bool precise = false);
// expand a complex k x n operand B (element (p,j) at B[p*rsb + j*csb], complex64) into
// Bt (2n x 2k floats, row stride ldt): rows 2j = (Br, -Bi), 2j+1 = (Bi, Br) along p.
int expand_b(midas_gpu_ctx *c, int k, int n, const float2 *B, long long rsb, long long csb, float *Bt,
             long long ldt);
// which GEMM engine is active ("tcgen05" or "simt")
const char *gemm_engine();
int gemm_selftest(midas_gpu_ctx *c);
int wait_selftest(midas_gpu_ctx *c, int limit, int *expired);
int gemm_bench(midas_gpu_ctx *c, int M, int N, int K, int iters, double *ms, bool f16 = false);

// dense.cu
constexpr int LU_MB = 256;   // macro block of the triangular solves
struct DenseLU {
    int n = 0, nb = 64, nblk = 0, nmac = 0;
    float2 *A = nullptr;     // n x n row-major, overwritten by L\U
    long long lda = 0;
    float2 *Linv = nullptr;  // nblk blocks of nb x nb (row-major), unit-lower inverses
    float2 *Uinv = nullptr;  // nblk blocks of nb x nb, upper inverses
    float2 *MLinvT = nullptr;   // nmac inverses of the LU_MB x LU_MB diagonal blocks of L, transposed
    float2 *MUinvT = nullptr;   // the same for U
};
// bytes of the diagonal-block inverses (slot S_LINV)
inline size_t lu_inv_bytes(int n)
{
    const size_t nblk = (size_t)(n + 63) / 64, nmac = (size_t)(n + LU_MB - 1) / LU_MB;
    return sizeof(float2) * (nblk * 64 * 64 * 2 + nmac * LU_MB * LU_MB * 2);
}
int lu_factor_nopiv(midas_gpu_ctx *c, DenseLU &lu);
// solve LU X = R in place; R is n x nrhs column-major complex64 (ld = n)
// Panel width of the two-level factorisation: the trailing update reads and
// writes the whole trailing matrix once per panel, so wide panels cut that
// traffic; narrow ones keep the sequential in-panel work short on small systems.
inline int lu_panel_width(int n) { return n >= 32768 ? 1024 : n >= 16384 ? 512 : 256; }
inline size_t lu_bexp2_bytes(int n) { return sizeof(float) * (size_t)2 * n * 2 * lu_panel_width(n); }   // slot S_BEXP2
int lu_solve(midas_gpu_ctx *c, const DenseLU &lu, float2 *R, int nrhs);
size_t lu_solve_scratch_bytes(int n, int nrhs);   // device scratch lu_solve takes from slot S_SOLVE
size_t lu_h16_scratch_bytes(int n);               // FP16 trailing-update panels, slot S_H16
// mixed-precision solve of Z x = b: Z64 row-major FP64 (n % 64 == 0), lu factored;
// b/x are n x nrhs column-major FP64.  Z64 is overwritten with its double-float
// split (float4 per element), which the refinement residuals read.
int ir_solve(midas_gpu_ctx *c, const DenseLU &lu, double2 *Z64, long long ldz, const double2 *b, double2 *x,
             int nrhs, midas_gpu_info *info);
int zgesv_fp64(midas_gpu_ctx *c, int n, int nrhs, double2 *Acol, double2 *Bcol, midas_gpu_info *info);
void destroy_cusolver(void *h);
// Mixed solve of a system whose FP64 row-major matrix Z64 and complex64 copy Z32
// (np x np, padded to 64) are filled; b/x are np x nrhs column-major (ld np).
// Both matrices are consumed (Z32 holds the factors, Z64 the split).
int mixed_solve_lattice(midas_gpu_ctx *c, int np, float2 *Z32, const double2 *b, double2 *x, int nrhs,
                        midas_gpu_info *info);
int mixed_solve(midas_gpu_ctx *c, int np, float2 *Z32, double2 *Z64, const double2 *b, double2 *x, int nrhs,
                midas_gpu_info *info, DenseLU *lu_out = nullptr);

// refinement residuals on the FP32 cores (resid.cu)
size_t resid_scratch_bytes(int n, int nrhs);   // slot S_RPART
// bound on |fl(Zh d) - Z d| / (|Z|_inf |d|_inf) of the FP32 product of resid_dense
double resid_update_error_factor(midas_gpu_ctx *c, int n, int nrhs);
// Z64 (row-major, ldz) -> float4 (hi.re, hi.im, lo.re, lo.im) in place; ||Z||_inf
int z_split_inplace(midas_gpu_ctx *c, double2 *Z64, long long ldz, int n, double *znorm);
// r = base - Z X for X = x (double-float, df) or X = d (complex64, FP32 product);
// r32 = fl32(r); rmax[j] = max over column j of max(|Re r|, |Im r|) (atomicMax of
// the FP64 bits, caller zeroes).  base may alias r.  n % 64 == 0.
int resid_dense(midas_gpu_ctx *c, int n, int nrhs, const float4 *Zs, long long ldz, bool df, const double2 *x,
                const float2 *d, const double2 *base, double2 *r, float2 *r32, unsigned long long *rmax);

}  // namespace midas
