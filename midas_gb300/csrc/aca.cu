// aca.cu -- partial-pivot adaptive cross approximation of CBFM block pairs (sm_103a).
//
// Calcul_MatrixZij_ACA (src/Calcul_ACA_matrices.f90:6-219) approximates the
// off-diagonal impedance block Z_ij (3 n_i x 3 n_j) by U V with U (3 n_i x k)
// and V (k x 3 n_j), building one row and one column of Z per step with
// computeBlockRow / computeBlockCol (src/Green_functions.f90:905-1225).  The
// steps of one block pair are sequential; the pairs are independent, so one
// CTA runs the whole ACA of one pair and a single launch covers every pair of
// the partition.
//
// Reproducibility: the row/column entries use the complex(4) element
// arithmetic of the block fills, the residual updates R = Z - sum_l U V are
// FP64 with every operation rounded (no FMA) and summed in the reference's
// order, and the pivot searches return the first index of the largest |R|
// (|R| rounded as the oracle rounds it) -- so the pivots, and hence U and V,
// are those of the sequential algorithm.
// Only the Frobenius-norm recursion (used for the stopping test) is summed in
// a different order.
#include "common.cuh"
#include "green.cuh"
#include "kernels.cuh"

namespace midas {

constexpr int ACA_THREADS = 256;
constexpr int ACA_WARPS = ACA_THREADS / 32;

__device__ __forceinline__ double2 zdiv_rn(double2 a, double2 b)
{
    double d = __dadd_rn(__dmul_rn(b.x, b.x), __dmul_rn(b.y, b.y));
    return make_double2(__ddiv_rn(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), d),
                        __ddiv_rn(__dsub_rn(__dmul_rn(a.y, b.x), __dmul_rn(a.x, b.y)), d));
}

// (value, index) maximum over the block; ties go to the lower index.  Every
// thread receives the winning index.
__device__ int block_argmax(double v, int idx, double *sv, int *si)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        double ov = __shfl_down_sync(0xffffffffu, v, o);
        int oi = __shfl_down_sync(0xffffffffu, idx, o);
        if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
    }
    if (lane == 0) { sv[w] = v; si[w] = idx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double bv = sv[0];
        int bi = si[0];
        for (int k = 1; k < ACA_WARPS; ++k)
            if (sv[k] > bv || (sv[k] == bv && si[k] < bi)) { bv = sv[k]; bi = si[k]; }
        si[ACA_WARPS] = bi;
    }
    __syncthreads();
    int r = si[ACA_WARPS];
    __syncthreads();
    return r;
}

__device__ double block_sum(double v, double *sv)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sv[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int k = 0; k < ACA_WARPS; ++k) t += sv[k];
        sv[ACA_WARPS] = t;
    }
    __syncthreads();
    double r = sv[ACA_WARPS];
    __syncthreads();
    return r;
}

// complex(4) dyad F of the cell pair (o, s), from the lattice table or directly
template <bool LAT>
__device__ __forceinline__ void dyad_pair(int o, int s, const double *x, const double *y, const double *z, double k0,
                                          double Pi, const Lat &lat, const float2 *tab4, float2 F[6])
{
    if (LAT) {
        size_t sl = lat.slot(o, s);
#pragma unroll
        for (int c = 0; c < 6; ++c) F[c] = tab4[6 * sl + c];
    } else {
        dyadF4(x[o] - x[s], y[o] - y[s], z[o] - z[s], k0, Pi, F);
    }
}

// One CTA per block pair.  U: column-major nrows x itmax (U[l*nrows + r]);
// V: row-major itmax x ncols (V[l*ncols + j]).  rank[p] = the reference's
// nb_iter_out (itmax + 1 when the tolerance was not reached).
template <bool LAT>
__global__ void __launch_bounds__(ACA_THREADS) k_aca_batch(const AcaPair *pairs, const double *x, const double *y,
                                                           const double *z, const float2 *fk4, double k0, double Pi,
                                                           Lat lat, const float2 *tab4, double eps, int itmax,
                                                           double2 *U, double2 *V, int *rank)
{
    const AcaPair P = pairs[blockIdx.x];
    const int nrows = 3 * P.ni, ncols = 3 * P.nj, tid = threadIdx.x;
    double2 *Up = U + P.uoff;
    double2 *Vp = V + P.voff;
    __shared__ int Ir[ACA_MAX_IT + 2], Jc[ACA_MAX_IT + 2];
    __shared__ double2 coef[ACA_MAX_IT];
    __shared__ double sv[ACA_WARPS + 1];
    __shared__ int si[ACA_WARPS + 1];
    __shared__ double s_prev;
    if (tid == 0) { Ir[0] = 0; s_prev = 0.0; }
    __syncthreads();
    int kk = 0, k_out = itmax + 1;
    for (;;) {
        const int ik = Ir[kk];
        // ---- residual row ik -> V(kk, :) (unnormalised) and its pivot column
        if (tid < kk) coef[tid] = Up[(size_t)tid * nrows + ik];
        __syncthreads();
        {
            const int io = P.r0 + ik / 3, pc = ik % 3;
            double best = -1.0;
            int bidx = 0x7fffffff;
            for (int s = tid; s < P.nj; s += ACA_THREADS) {
                const int sc = P.c0 + s;
                float2 F[6];
                dyad_pair<LAT>(io, sc, x, y, z, k0, Pi, lat, tab4, F);
                const float2 fk = fk4[sc];
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const int j = 3 * s + q;
                    float2 g = zmul4_rn(F[comp6(pc, q)], fk);
                    double2 acc = make_double2(0.0, 0.0);
                    for (int l = 0; l < kk; ++l) {
                        double2 p = zmul8_rn(coef[l], Vp[(size_t)l * ncols + j]);
                        acc.x = __dadd_rn(acc.x, p.x);
                        acc.y = __dadd_rn(acc.y, p.y);
                    }
                    double2 R = make_double2(__dsub_rn(-(double)g.x, acc.x), __dsub_rn(-(double)g.y, acc.y));
                    Vp[(size_t)kk * ncols + j] = R;
                    bool used = false;
                    for (int l = 0; l < kk; ++l) used |= (Jc[l] == j);
                    double a = used ? 0.0 : absd8(R);
                    if (a > best) { best = a; bidx = j; }
                }
            }
            const int jk = block_argmax(best, bidx, sv, si);
            if (tid == 0) Jc[kk] = jk;
            const double2 piv = Vp[(size_t)kk * ncols + jk];
            __syncthreads();   // every thread has read the pivot before any row entry is overwritten
            for (int j = tid; j < ncols; j += ACA_THREADS) {
                double2 *e = Vp + (size_t)kk * ncols + j;
                *e = zdiv_rn(*e, piv);
            }
        }
        __syncthreads();
        const int jk = Jc[kk];
        // ---- residual column jk -> U(:, kk)
        if (tid < kk) coef[tid] = Vp[(size_t)tid * ncols + jk];
        __syncthreads();
        double nu2 = 0.0;
        {
            const int sc = P.c0 + jk / 3, qc = jk % 3;
            const float2 fk = fk4[sc];
            for (int i = tid; i < P.ni; i += ACA_THREADS) {
                float2 F[6];
                dyad_pair<LAT>(P.r0 + i, sc, x, y, z, k0, Pi, lat, tab4, F);
#pragma unroll
                for (int p = 0; p < 3; ++p) {
                    const int r = 3 * i + p;
                    float2 g = zmul4_rn(F[comp6(p, qc)], fk);
                    double2 acc = make_double2(0.0, 0.0);
                    for (int l = 0; l < kk; ++l) {
                        double2 t = zmul8_rn(coef[l], Up[(size_t)l * nrows + r]);
                        acc.x = __dadd_rn(acc.x, t.x);
                        acc.y = __dadd_rn(acc.y, t.y);
                    }
                    double2 R = make_double2(__dsub_rn(-(double)g.x, acc.x), __dsub_rn(-(double)g.y, acc.y));
                    Up[(size_t)kk * nrows + r] = R;
                    double a = absd8(R);
                    nu2 += a * a;
                }
            }
        }
        double nv2 = 0.0;
        for (int j = tid; j < ncols; j += ACA_THREADS) {
            double a = absd8(Vp[(size_t)kk * ncols + j]);
            nv2 += a * a;
        }
        __syncthreads();   // U(:, kk) complete
        nu2 = block_sum(nu2, sv);
        nv2 = block_sum(nv2, sv);
        // sum_{l<kk} |U(:,l) . U(:,kk)| |V(kk,:) . V(l,:)| (plain products, no conjugate), a warp per l
        double suv = 0.0;
        {
            const int lane = tid & 31, w = tid >> 5;
            for (int l = w; l < kk; l += ACA_WARPS) {
                double2 su = make_double2(0, 0), sw = make_double2(0, 0);
                for (int r = lane; r < nrows; r += 32) {
                    double2 t = zmul8(Up[(size_t)l * nrows + r], Up[(size_t)kk * nrows + r]);
                    su.x += t.x; su.y += t.y;
                }
                for (int j = lane; j < ncols; j += 32) {
                    double2 t = zmul8(Vp[(size_t)kk * ncols + j], Vp[(size_t)l * ncols + j]);
                    sw.x += t.x; sw.y += t.y;
                }
                for (int o = 16; o > 0; o >>= 1) {
                    su.x += __shfl_down_sync(0xffffffffu, su.x, o);
                    su.y += __shfl_down_sync(0xffffffffu, su.y, o);
                    sw.x += __shfl_down_sync(0xffffffffu, sw.x, o);
                    sw.y += __shfl_down_sync(0xffffffffu, sw.y, o);
                }
                if (lane == 0) suv += absd8(su) * absd8(sw);
            }
        }
        suv = block_sum(suv, sv);
        const double nu = sqrt(nu2), nv = sqrt(nv2);
        const double prev = s_prev;
        const double nf = sqrt(prev * prev + 2 * suv + nu * nu * (nv * nv));
        const double res = (nu * nv) / nf;
        __syncthreads();
        if (tid == 0) s_prev = nf;
        if (kk > 0 && res <= eps) { k_out = kk + 1; break; }
        if (kk + 1 >= itmax) { k_out = itmax + 1; break; }
        // ---- next pivot row: largest |R(:, jk)| among the rows not used yet
        {
            double best = -1.0;
            int bidx = 0x7fffffff;
            for (int r = tid; r < nrows; r += ACA_THREADS) {
                bool used = false;
                for (int l = 0; l <= kk; ++l) used |= (Ir[l] == r);
                double2 u = Up[(size_t)kk * nrows + r];
                double a = used ? 0.0 : absd8(u);
                if (a > best) { best = a; bidx = r; }
            }
            const int inext = block_argmax(best, bidx, sv, si);
            if (tid == 0) Ir[kk + 1] = inext;
        }
        __syncthreads();
        ++kk;
    }
    if (tid == 0) rank[blockIdx.x] = k_out;
}

// V (row-major itmax x ncols) -> column-major (Vc[j*itmax + l])
__global__ void k_aca_vt(const double2 *V, int itmax, int ncols, double2 *Vc)
{
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)itmax * ncols) return;
    int l = (int)(t / ncols), j = (int)(t % ncols);
    Vc[(size_t)j * itmax + l] = V[t];
}

// T(r, c) = sum_{l<k} U(r, l) W(l, c) in FP64, stored rounded to complex64 at
// T[r*ldt + c] (the reduced-matrix work array of the CBFM assembly)
__global__ void k_aca_uw(int nrows, int k, int ncol, const double2 *U, const double2 *W, float2 *T, long long ldt)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    int c = blockIdx.y;
    if (r >= nrows) return;
    double2 acc = make_double2(0, 0);
    for (int l = 0; l < k; ++l) {
        double2 u = U[(size_t)l * nrows + r], w = W[(size_t)l * ncol + c];
        acc.x += u.x * w.x - u.y * w.y;
        acc.y += u.x * w.y + u.y * w.x;
    }
    T[(size_t)r * ldt + c] = make_float2((float)acc.x, (float)acc.y);
}

int aca_batch(midas_gpu_ctx *c, int npairs, const AcaPair *d_pairs, double eps, int itmax, double2 *U, double2 *V,
              int *d_rank)
{
    if (npairs <= 0) return MIDAS_OK;
    if (itmax < 2 || itmax > ACA_MAX_IT) return c->err.set(MIDAS_ERR_ARG, "aca: itmax must be in [2, 128]");
    Lat l;
    l.ijk = c->lat_ijk;
    l.dim0 = c->lat_dim[0]; l.dim1 = c->lat_dim[1]; l.dim2 = c->lat_dim[2];
    l.sp0 = (c->lat_dim[0] - 1) / 2; l.sp1 = (c->lat_dim[1] - 1) / 2; l.sp2 = (c->lat_dim[2] - 1) / 2;
    const bool lat = c->opts.fill_mode == MIDAS_FILL_FAST && c->lattice && c->lat_tab4;
    ++c->launches;
    int kp = kp_begin(c);
    if (lat)
        k_aca_batch<true><<<npairs, ACA_THREADS, 0, c->stream>>>(d_pairs, c->x, c->y, c->z, c->fk4, c->k0, c->pi, l,
                                                                 c->lat_tab4, eps, itmax, U, V, d_rank);
    else
        k_aca_batch<false><<<npairs, ACA_THREADS, 0, c->stream>>>(d_pairs, c->x, c->y, c->z, c->fk4, c->k0, c->pi, l,
                                                                  nullptr, eps, itmax, U, V, d_rank);
    kp_end(c, kp, MIDAS_KC_OTHER, 0.0, 0.0);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

int aca_uw(midas_gpu_ctx *c, int nrows, int k, int ncol, const double2 *U, const double2 *W, float2 *T, long long ldt)
{
    if (nrows <= 0 || ncol <= 0) return MIDAS_OK;
    dim3 grd((nrows + 127) / 128, ncol);
    ++c->launches;
    k_aca_uw<<<grd, 128, 0, c->stream>>>(nrows, k, ncol, U, W, T, ldt);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// single block pair (the midas_gpu_aca entry point): U column-major nrows x itmax,
// V column-major itmax x ncols
int aca_run(midas_gpu_ctx *c, int row0, int nrows, int col0, int ncols, double eps, int itmax, double2 *U,
            double2 *V, int *rank)
{
    if (itmax < 2 || itmax > ACA_MAX_IT) return c->err.set(MIDAS_ERR_ARG, "aca: itmax must be in [2, 128]");
    if (row0 < col0 + ncols && col0 < row0 + nrows)
        return c->err.set(MIDAS_ERR_ARG, "aca: row and column blocks overlap (ACA applies to distinct blocks)");
    void *p;
    const size_t vbytes = sizeof(double2) * (size_t)itmax * ncols;
    MIDAS_TRY(ensure(c, S_IN5, sizeof(AcaPair) + 256 + vbytes, &p));
    AcaPair *dp = (AcaPair *)p;
    int *drank = (int *)((char *)p + sizeof(AcaPair));
    double2 *Vr = (double2 *)((char *)p + 256);
    AcaPair h{row0 / 3, nrows / 3, col0 / 3, ncols / 3, 0, 0};
    MIDAS_CUDA(c, cudaMemcpyAsync(dp, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
    MIDAS_CUDA(c, cudaMemsetAsync(U, 0, sizeof(double2) * (size_t)nrows * itmax, c->stream));
    MIDAS_CUDA(c, cudaMemsetAsync(Vr, 0, vbytes, c->stream));
    MIDAS_TRY(aca_batch(c, 1, dp, eps, itmax, U, Vr, drank));
    long long tot = (long long)itmax * ncols;
    ++c->launches;
    k_aca_vt<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(Vr, itmax, ncols, V);
    MIDAS_CUDA(c, cudaGetLastError());
    MIDAS_CUDA(c, cudaMemcpyAsync(rank, drank, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    return MIDAS_OK;
}

}  // namespace midas
