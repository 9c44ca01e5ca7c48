// krylov.cu -- restarted GMRES on the FFT lattice operator (sm_103a).
//
// The MoM system Z E = E_inc of compute_Green_s_tr_single_element
// (src/Compute_EFields_MoM.f90:433-598) for cells on one lattice, solved without
// forming Z: every product is the FFT operator of fft.cu (FP64).  The
// reference solves the same system with a dense LU (PZGESV,
// src/Compute_EFields_MoM.f90:153-198); the Krylov path is what makes systems of
// ~1e5 unknowns solvable from an initial guess (a learned predictor's output)
// in seconds, with the dense solve as its fallback and judge.
//
// All right-hand sides advance in lockstep, so each Arnoldi step is one batched
// FFT product.  Orthogonalisation is classical Gram-Schmidt applied twice
// (CGS2), with deterministic two-stage reductions; the small Hessenberg
// least-squares problems (Givens rotations) run on the host.  Every restart
// recomputes the true residual b - Z x in FP64, and convergence is accepted on
// that true residual only.  Optional right preconditioner: the inverse of the
// matrix diagonal, 1 / (1 - Znnpp) per cell (Jacobi), or the learned network of
// nn.cu, which is not linear and makes the method flexible GMRES (FGMRES: the
// preconditioned vectors P(v_j) are kept and x += sum_j P(v_j) y_j).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace midas {

constexpr int KR_THREADS = 256;
constexpr int KR_CHUNK = 4096;   // rows per reduction block

__device__ __forceinline__ double2 kr_cmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 kr_cjmul(double2 a, double2 b)   // conj(a) b
{
    return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

// partial[(k * nv + i) * nblk + blk] = sum over the block's rows of conj(V_i,k) w_k
// V: vectors i = 0..nv-1, each N x ncol column-major (ld N), vector stride vs
__global__ void __launch_bounds__(KR_THREADS) k_kr_dots(int N, int ncol, int nv, const double2 *V, long long vs,
                                                        const double2 *W, double2 *partial)
{
    __shared__ double2 red[KR_THREADS / 32];
    const int k = blockIdx.y, blk = blockIdx.x, nblk = gridDim.x;
    const int r0 = blk * KR_CHUNK, r1 = min(N, r0 + KR_CHUNK);
    const double2 *w = W + (long long)k * N;
    for (int i = 0; i < nv; ++i) {
        const double2 *v = V + i * vs + (long long)k * N;
        double2 s = make_double2(0, 0);
        for (int r = r0 + threadIdx.x; r < r1; r += KR_THREADS) {
            const double2 t = kr_cjmul(v[r], w[r]);
            s.x += t.x;
            s.y += t.y;
        }
        for (int o = 16; o > 0; o >>= 1) {
            s.x += __shfl_down_sync(0xffffffffu, s.x, o);
            s.y += __shfl_down_sync(0xffffffffu, s.y, o);
        }
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double2 t = make_double2(0, 0);
            for (int q = 0; q < KR_THREADS / 32; ++q) { t.x += red[q].x; t.y += red[q].y; }
            partial[((long long)k * nv + i) * nblk + blk] = t;
        }
        __syncthreads();
    }
}

// out[k * nv + i] = sum over blocks of partial (fixed order: deterministic)
__global__ void k_kr_reduce(int n_out, int nblk, const double2 *partial, double2 *out)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_out) return;
    double2 s = make_double2(0, 0);
    for (int b = 0; b < nblk; ++b) {
        s.x += partial[(long long)t * nblk + b].x;
        s.y += partial[(long long)t * nblk + b].y;
    }
    out[t] = s;
}

// W_k += sgn * sum_i V_i,k h[k * ldh + i]  (h in device memory), for active columns
__global__ void k_kr_axpy(int N, int ncol, int nv, const double2 *V, long long vs, const double2 *h, int ldh,
                          double sgn, const int *active, double2 *W)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (t >= N || (active && !active[k])) return;
    double2 acc = make_double2(0, 0);
    for (int i = 0; i < nv; ++i) {
        const double2 c = h[(long long)k * ldh + i];
        const double2 v = V[i * vs + (long long)k * N + t];
        const double2 p = kr_cmul(v, c);
        acc.x += p.x;
        acc.y += p.y;
    }
    double2 *w = W + (long long)k * N + t;
    *w = make_double2(w->x + sgn * acc.x, w->y + sgn * acc.y);
}

// V_k = W_k * s[k] (real scale per column)
__global__ void k_kr_scale(int N, const double2 *W, const double *s, double2 *V)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (t >= N) return;
    const double2 w = W[(long long)k * N + t];
    V[(long long)k * N + t] = make_double2(w.x * s[k], w.y * s[k]);
}

// Y_k = D^-1 X_k with D = 1 - Znnpp per cell (3 rows per cell)
__global__ void k_kr_jacobi(int ncell, int ncol, const double2 *znnpp, const double2 *X, double2 *Y)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (t >= 3LL * ncell) return;
    const double2 d = make_double2(1.0 - znnpp[t / 3].x, -znnpp[t / 3].y);
    const double den = d.x * d.x + d.y * d.y;
    const double2 x = X[(long long)k * 3 * ncell + t];
    Y[(long long)k * 3 * ncell + t] = make_double2((x.x * d.x + x.y * d.y) / den, (x.y * d.x - x.x * d.y) / den);
}

struct Kr {
    midas_gpu_ctx *c;
    int N, ncol;
    double2 *partial, *hdev;
    int nblk;
    // conj(V_i)^T W for i < nv, every column: returns host h[k * nv + i]
    int dots(const double2 *V, long long vs, int nv, const double2 *W, std::vector<std::complex<double>> &h)
    {
        ++c->launches;
        k_kr_dots<<<dim3(nblk, ncol), KR_THREADS, 0, c->stream>>>(N, ncol, nv, V, vs, W, partial);
        const int nout = ncol * nv;
        ++c->launches;
        k_kr_reduce<<<(nout + 127) / 128, 128, 0, c->stream>>>(nout, nblk, partial, hdev);
        MIDAS_CUDA(c, cudaGetLastError());
        h.resize(nout);
        MIDAS_CUDA(c, cudaMemcpyAsync(h.data(), hdev, sizeof(double2) * nout, cudaMemcpyDeviceToHost, c->stream));
        MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
        return MIDAS_OK;
    }
};

static unsigned kr_blocks(long long n) { return (unsigned)((n + KR_THREADS - 1) / KR_THREADS); }

// GMRES(restart) for Z X = B, B and X column-major (3n x ncol, ld 3n), X holds the
// initial guess on entry.  Returns the iterations (Arnoldi steps) and the final
// true relative residual max_k ||b_k - Z x_k|| / ||b_k||.
int gmres_lattice(midas_gpu_ctx *c, int ncol, const double2 *B, double2 *X, int restart, int maxit, double tol,
                  bool jacobi, int *iters, double *relres, midas_gpu_nn *net)
{
    if (net) jacobi = false;   // the network's prediction contains the Jacobi term
    MIDAS_TRY(lattice_fft_prepare(c));
    const int N = 3 * c->n;
    const int m = std::max(1, restart);
    const long long vs = (long long)N * ncol;   // one Krylov vector for every column
    const int nblk = (N + KR_CHUNK - 1) / KR_CHUNK;
    void *p;
    const size_t vbytes = sizeof(double2) * (size_t)vs;
    const int nz = net ? m : 0;   // flexible GMRES keeps the preconditioned vectors P(v_j)
    MIDAS_TRY(ensure(c, S_KRYLOV, vbytes * (m + 1 + nz) + 3 * vbytes + sizeof(double2) * ((size_t)ncol * (m + 2) * nblk +
                                                                                     (size_t)ncol * (m + 2) + 64) +
                                      sizeof(double) * ncol + sizeof(int) * ncol + 4096,
                      &p));
    char *base = (char *)p;
    auto take = [&](size_t bytes) { char *q = base; base += (bytes + 255) & ~(size_t)255; return q; };
    double2 *V = (double2 *)take(vbytes * (m + 1));
    double2 *Zp = net ? (double2 *)take(vbytes * m) : nullptr;
    double2 *W = (double2 *)take(vbytes), *R = (double2 *)take(vbytes), *Tz = (double2 *)take(vbytes);
    double2 *partial = (double2 *)take(sizeof(double2) * (size_t)ncol * (m + 2) * nblk);
    double2 *hdev = (double2 *)take(sizeof(double2) * ((size_t)ncol * (m + 2) + 64));
    double *sdev = (double *)take(sizeof(double) * ncol);
    int *adev = (int *)take(sizeof(int) * ncol);
    Kr kr{c, N, ncol, partial, hdev, nblk};
    const dim3 gv(kr_blocks(N), ncol);
    using cd = std::complex<double>;
    std::vector<cd> hv;
    // ||b_k||
    std::vector<double> bn(ncol), rn(ncol);
    MIDAS_TRY(kr.dots(B, 0, 1, B, hv));
    for (int k = 0; k < ncol; ++k) bn[k] = sqrt(std::max(hv[k].real(), 0.0));
    int total = 0;
    double worst = 1e300;
    std::vector<int> active(ncol, 1);
    std::vector<double> scale(ncol);
    std::vector<cd> H((size_t)ncol * (m + 1) * m), g((size_t)ncol * (m + 1)), cs((size_t)ncol * m),
        sn((size_t)ncol * m), y((size_t)ncol * m);
    while (true) {
        // true residual R = B - Z X (FP64)
        MIDAS_TRY(lattice_matvec(c, ncol, X, N, B, N, R, N, S_LFFT));
        MIDAS_TRY(kr.dots(R, 0, 1, R, hv));
        worst = 0;
        for (int k = 0; k < ncol; ++k) {
            rn[k] = sqrt(std::max(hv[k].real(), 0.0));
            const double rel = bn[k] > 0 ? rn[k] / bn[k] : rn[k];
            worst = std::max(worst, rel);
            active[k] = rel > tol;
        }
        if (c->opts.verbose)
            fprintf(stderr, "[midas] gmres: %d iterations, true relative residual %.3e\n", total, worst);
        if (!(worst == worst)) return c->err.set(MIDAS_ERR_NOT_CONVERGED, "gmres: NaN residual");
        if (worst <= tol || total >= maxit) break;
        // v0 = r / ||r||
        for (int k = 0; k < ncol; ++k) scale[k] = rn[k] > 0 ? 1.0 / rn[k] : 0.0;
        MIDAS_CUDA(c, cudaMemcpyAsync(sdev, scale.data(), sizeof(double) * ncol, cudaMemcpyHostToDevice, c->stream));
        MIDAS_CUDA(c, cudaMemcpyAsync(adev, active.data(), sizeof(int) * ncol, cudaMemcpyHostToDevice, c->stream));
        ++c->launches;
        k_kr_scale<<<gv, KR_THREADS, 0, c->stream>>>(N, R, sdev, V);
        std::fill(g.begin(), g.end(), cd(0));
        for (int k = 0; k < ncol; ++k) g[(size_t)k * (m + 1)] = rn[k];
        int j;
        bool inner_done = false;
        for (j = 0; j < m && total < maxit && !inner_done; ++j, ++total) {
            const double2 *vj = V + j * vs;
            // W = Z M^-1 v_j
            const double2 *zin = vj;
            if (net) {
                MIDAS_TRY(nn_prec_apply(c, net, ncol, vj, N, Zp + j * vs, N));
                zin = Zp + j * vs;
            } else if (jacobi) {
                ++c->launches;
                k_kr_jacobi<<<dim3(kr_blocks(N), ncol), KR_THREADS, 0, c->stream>>>(c->n, ncol, c->znnpp, vj, Tz);
                zin = Tz;
            }
            MIDAS_TRY(lattice_matvec(c, ncol, zin, N, nullptr, 0, W, N, S_LFFT));
            // CGS2: h = V^H w twice
            std::vector<cd> hsum((size_t)ncol * (j + 1), cd(0));
            for (int pass = 0; pass < 2; ++pass) {
                MIDAS_TRY(kr.dots(V, vs, j + 1, W, hv));
                for (size_t q = 0; q < hsum.size(); ++q) hsum[q] += hv[q];
                MIDAS_CUDA(c, cudaMemcpyAsync(hdev, hv.data(), sizeof(double2) * hv.size(), cudaMemcpyHostToDevice,
                                              c->stream));
                ++c->launches;
                k_kr_axpy<<<gv, KR_THREADS, 0, c->stream>>>(N, ncol, j + 1, V, vs, hdev, j + 1, -1.0, adev, W);
            }
            MIDAS_TRY(kr.dots(W, 0, 1, W, hv));
            std::vector<double> hn(ncol);
            for (int k = 0; k < ncol; ++k) {
                hn[k] = sqrt(std::max(hv[k].real(), 0.0));
                scale[k] = hn[k] > 0 ? 1.0 / hn[k] : 0.0;
            }
            MIDAS_CUDA(c, cudaMemcpyAsync(sdev, scale.data(), sizeof(double) * ncol, cudaMemcpyHostToDevice, c->stream));
            ++c->launches;
            k_kr_scale<<<gv, KR_THREADS, 0, c->stream>>>(N, W, sdev, V + (j + 1) * vs);
            MIDAS_CUDA(c, cudaGetLastError());
            // Hessenberg column j, previous rotations, new rotation, residual estimate
            double est = 0;
            for (int k = 0; k < ncol; ++k) {
                if (!active[k]) continue;
                cd *Hk = &H[(size_t)k * (m + 1) * m];
                for (int i = 0; i <= j; ++i) Hk[(size_t)j * (m + 1) + i] = hsum[(size_t)k * (j + 1) + i];
                Hk[(size_t)j * (m + 1) + j + 1] = hn[k];
                for (int i = 0; i < j; ++i) {
                    const cd a = Hk[(size_t)j * (m + 1) + i], b = Hk[(size_t)j * (m + 1) + i + 1];
                    const cd cc = cs[(size_t)k * m + i], ss = sn[(size_t)k * m + i];
                    Hk[(size_t)j * (m + 1) + i] = std::conj(cc) * a + std::conj(ss) * b;
                    Hk[(size_t)j * (m + 1) + i + 1] = -ss * a + cc * b;
                }
                const cd a = Hk[(size_t)j * (m + 1) + j], b = Hk[(size_t)j * (m + 1) + j + 1];
                const double den = sqrt(std::norm(a) + std::norm(b));
                const cd cc = den > 0 ? a / den : cd(1), ss = den > 0 ? b / den : cd(0);
                cs[(size_t)k * m + j] = cc;
                sn[(size_t)k * m + j] = ss;
                Hk[(size_t)j * (m + 1) + j] = den;
                Hk[(size_t)j * (m + 1) + j + 1] = 0;
                cd *gk = &g[(size_t)k * (m + 1)];
                gk[j + 1] = -ss * gk[j];
                gk[j] = std::conj(cc) * gk[j];
                est = std::max(est, std::abs(gk[j + 1]) / (bn[k] > 0 ? bn[k] : 1.0));
            }
            inner_done = est <= 0.5 * tol;
        }
        // x += M^-1 V y with H y = g (upper triangular, j x j)
        std::fill(y.begin(), y.end(), cd(0));
        for (int k = 0; k < ncol; ++k) {
            if (!active[k]) continue;
            const cd *Hk = &H[(size_t)k * (m + 1) * m];
            const cd *gk = &g[(size_t)k * (m + 1)];
            for (int i = j - 1; i >= 0; --i) {
                cd s = gk[i];
                for (int l = i + 1; l < j; ++l) s -= Hk[(size_t)l * (m + 1) + i] * y[(size_t)k * m + l];
                y[(size_t)k * m + i] = s / Hk[(size_t)i * (m + 1) + i];
            }
        }
        MIDAS_CUDA(c, cudaMemcpyAsync(hdev, y.data(), sizeof(double2) * (size_t)ncol * m, cudaMemcpyHostToDevice,
                                      c->stream));
        if (net) {   // x += sum_j P(v_j) y_j
            ++c->launches;
            k_kr_axpy<<<gv, KR_THREADS, 0, c->stream>>>(N, ncol, j, Zp, vs, hdev, m, 1.0, adev, X);
        } else if (jacobi) {
            MIDAS_CUDA(c, cudaMemsetAsync(W, 0, vbytes, c->stream));
            ++c->launches;
            k_kr_axpy<<<gv, KR_THREADS, 0, c->stream>>>(N, ncol, j, V, vs, hdev, m, 1.0, adev, W);
            ++c->launches;
            k_kr_jacobi<<<dim3(kr_blocks(N), ncol), KR_THREADS, 0, c->stream>>>(c->n, ncol, c->znnpp, W, Tz);
            // X += Tz (scale 1), active columns only: Tz is zero for the others
            std::vector<cd> ones((size_t)ncol, cd(1));
            MIDAS_CUDA(c, cudaMemcpyAsync(hdev, ones.data(), sizeof(double2) * ncol, cudaMemcpyHostToDevice, c->stream));
            ++c->launches;
            k_kr_axpy<<<gv, KR_THREADS, 0, c->stream>>>(N, ncol, 1, Tz, 0, hdev, 1, 1.0, adev, X);
        } else {
            ++c->launches;
            k_kr_axpy<<<gv, KR_THREADS, 0, c->stream>>>(N, ncol, j, V, vs, hdev, m, 1.0, adev, X);
        }
        MIDAS_CUDA(c, cudaGetLastError());
    }
    MIDAS_TRY(check_flag(c, "gmres"));
    *iters = total;
    *relres = worst;
    if (worst > tol) {
        char msg[160];
        snprintf(msg, sizeof msg, "gmres: true relative residual %.3e after %d iterations (tolerance %.1e)", worst,
                 total, tol);
        return c->err.set(MIDAS_ERR_NOT_CONVERGED, msg);
    }
    return MIDAS_OK;
}

}  // namespace midas
