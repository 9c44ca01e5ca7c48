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
// least-squares problems (Givens rotations, the back-substitution) run on the
// device too, so an Arnoldi step costs the host one read of the residual
// estimates.  Every restart
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
constexpr int KR_CHUNK = 1024;   // rows per reduction block

__device__ __forceinline__ double2 kr_cmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 kr_cjmul(double2 a, double2 b)   // conj(a) b
{
    return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

// partial[(k * nv + i) * nblk + blk] = sum over the block's rows of conj(V_i,k) w_k
// V: vectors i = 0..nv-1, each N x ncol column-major (ld N), vector stride vs; one
// CTA per (row block, column, vector), so the products run at full occupancy
// (with jd, nv = *jd + 1: the Arnoldi index read from device memory, so that one
// captured graph of an Arnoldi step serves every step; blocks beyond nv exit)
__global__ void __launch_bounds__(KR_THREADS) k_kr_dots(int N, int ncol, int nv, const double2 *V, long long vs,
                                                        const double2 *W, double2 *partial, const int *jd = nullptr)
{
    __shared__ double2 red[KR_THREADS / 32];
    if (jd) nv = *jd + 1;
    const int k = blockIdx.y, blk = blockIdx.x, nblk = gridDim.x, i = blockIdx.z;
    if (i >= nv) return;
    const int r0 = blk * KR_CHUNK, r1 = min(N, r0 + KR_CHUNK);
    const double2 *w = W + (long long)k * N;
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
}

// out[k * nv + i] = sum over blocks of partial (fixed order: deterministic); with
// acc, the sum is also added into acc[k * lda + i]
__global__ void k_kr_reduce(int n_out, int nblk, const double2 *partial, double2 *out, int nv, double2 *acc,
                            int lda, int first, const int *jd = nullptr)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (jd) {   // n_out is the column count times the largest nv
        n_out = n_out / nv * (*jd + 1);
        nv = *jd + 1;
    }
    if (t >= n_out) return;
    double2 s = make_double2(0, 0);
    for (int b = 0; b < nblk; ++b) {
        s.x += partial[(long long)t * nblk + b].x;
        s.y += partial[(long long)t * nblk + b].y;
    }
    out[t] = s;
    if (acc) {
        double2 *a = acc + (long long)(t / nv) * lda + t % nv;
        *a = first ? s : make_double2(a->x + s.x, a->y + s.y);
    }
}

// W_k += sgn * sum_i V_i,k h[k * ldh + i]  (h in device memory), for active columns
__global__ void k_kr_axpy(int N, int ncol, int nv, const double2 *V, long long vs, const double2 *h, int ldh,
                          double sgn, const int *active, double2 *W, const int *jd = nullptr)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (jd) nv = ldh = *jd + 1;
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

// V_k = W_k / sqrt(n2[k].x) (n2 = the column's squared norm from k_kr_reduce; 0 for a zero column)
__global__ void k_kr_normalise(int N, const double2 *W, const double2 *n2, double2 *V, const int *jd = nullptr,
                               long long vs = 0)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (t >= N) return;
    if (jd) V += (long long)(*jd + 1) * vs;   // into Krylov slot j + 1
    const double nn = sqrt(fmax(n2[k].x, 0.0));
    const double sc = nn > 0 ? 1.0 / nn : 0.0;
    const double2 w = W[(long long)k * N + t];
    V[(long long)k * N + t] = make_double2(w.x * sc, w.y * sc);
}

__device__ __forceinline__ double2 kr_conjmul(double2 a, double2 b)   // conj(a) b
{
    return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

// Arnoldi step j of every active column on the device: Hessenberg column j from the
// CGS2 sums hc (ld ldh) and the norm |w|, the previous Givens rotations, a new one,
// the rotated right-hand side g, and est[k] = |g_{j+1}| / |b_k| (0 for inactive
// columns).  H: column j of matrix k at H[(k (m+1)) m + j (m+1) + i].
__global__ void k_kr_givens(int ncol, const int *jd, int m, const double2 *hc, int ldh, const double2 *n2,
                            const int *active, const double *bn, double2 *H, double2 *g, double2 *cs, double2 *sn,
                            double *est)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ncol) return;
    const int j = *jd;
    if (!active[k]) { est[k] = 0.0; return; }
    double2 *Hk = H + (long long)k * (m + 1) * m + (long long)j * (m + 1);
    for (int i = 0; i <= j; ++i) Hk[i] = hc[(long long)k * ldh + i];
    Hk[j + 1] = make_double2(sqrt(fmax(n2[k].x, 0.0)), 0.0);
    double2 *csk = cs + (long long)k * m, *snk = sn + (long long)k * m;
    for (int i = 0; i < j; ++i) {
        const double2 a = Hk[i], b = Hk[i + 1], cc = csk[i], ss = snk[i];
        const double2 t1 = kr_conjmul(cc, a), t2 = kr_conjmul(ss, b);
        const double2 u1 = kr_cmul(ss, a), u2 = kr_cmul(cc, b);
        Hk[i] = make_double2(t1.x + t2.x, t1.y + t2.y);
        Hk[i + 1] = make_double2(u2.x - u1.x, u2.y - u1.y);
    }
    const double2 a = Hk[j], b = Hk[j + 1];
    const double den = sqrt(a.x * a.x + a.y * a.y + b.x * b.x + b.y * b.y);
    const double2 cc = den > 0 ? make_double2(a.x / den, a.y / den) : make_double2(1.0, 0.0);
    const double2 ss = den > 0 ? make_double2(b.x / den, b.y / den) : make_double2(0.0, 0.0);
    csk[j] = cc;
    snk[j] = ss;
    Hk[j] = make_double2(den, 0.0);
    Hk[j + 1] = make_double2(0.0, 0.0);
    double2 *gk = g + (long long)k * (m + 1);
    const double2 gj = gk[j], t = kr_cmul(ss, gj);
    gk[j + 1] = make_double2(-t.x, -t.y);
    gk[j] = kr_conjmul(cc, gj);
    est[k] = sqrt(gk[j + 1].x * gk[j + 1].x + gk[j + 1].y * gk[j + 1].y) / (bn[k] > 0 ? bn[k] : 1.0);
}

// y = H^-1 g (upper triangular, nj x nj) per active column, into y[k * m + i]
__global__ void k_kr_backsolve(int ncol, int nj, int m, const double2 *H, const double2 *g, const int *active,
                               double2 *y)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ncol) return;
    double2 *yk = y + (long long)k * m;
    if (!active[k]) {
        for (int i = 0; i < nj; ++i) yk[i] = make_double2(0.0, 0.0);
        return;
    }
    const double2 *Hk = H + (long long)k * (m + 1) * m, *gk = g + (long long)k * (m + 1);
    for (int i = nj - 1; i >= 0; --i) {
        double2 sacc = gk[i];
        for (int l = i + 1; l < nj; ++l) {
            const double2 p = kr_cmul(Hk[(long long)l * (m + 1) + i], yk[l]);
            sacc = make_double2(sacc.x - p.x, sacc.y - p.y);
        }
        const double2 d = Hk[(long long)i * (m + 1) + i];
        const double den = d.x * d.x + d.y * d.y;
        yk[i] = make_double2((sacc.x * d.x + sacc.y * d.y) / den, (sacc.y * d.x - sacc.x * d.y) / den);
    }
}

// out = Krylov slot *jd + off of V (or in = out into that slot of V when put)
__global__ void k_kr_slot(long long tot, double2 *V, long long vs, const int *jd, int off, double2 *buf, int put)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= tot) return;
    double2 *v = V + (long long)(*jd + off) * vs + t;
    if (put) *v = buf[t];
    else buf[t] = *v;
}

__global__ void k_kr_next(int *jd) { *jd += 1; }

// g_k = (|r_k|, 0, ..., 0)
__global__ void k_kr_g0(int ncol, int m, const double2 *r2, double2 *g)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncol * (m + 1)) return;
    const int k = t / (m + 1), i = t % (m + 1);
    g[t] = i == 0 ? make_double2(sqrt(fmax(r2[k].x, 0.0)), 0.0) : make_double2(0.0, 0.0);
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
    // the same on the device only: out[k * nv + i], optionally accumulated into acc (ld lda)
    int dots_dev(const double2 *V, long long vs, int nv, const double2 *W, double2 *out, double2 *acc = nullptr,
                 int lda = 0, bool first = true, const int *jd = nullptr)
    {
        ++c->launches;
        k_kr_dots<<<dim3(nblk, ncol, nv), KR_THREADS, 0, c->stream>>>(N, ncol, nv, V, vs, W, partial, jd);
        const int nout = ncol * nv;   // with jd: nv is the largest count
        ++c->launches;
        k_kr_reduce<<<(nout + 127) / 128, 128, 0, c->stream>>>(nout, nblk, partial, out, nv, acc, lda, first ? 1 : 0,
                                                               jd);
        MIDAS_CUDA(c, cudaGetLastError());
        return MIDAS_OK;
    }
    int dots(const double2 *V, long long vs, int nv, const double2 *W, std::vector<std::complex<double>> &h)
    {
        MIDAS_TRY(dots_dev(V, vs, nv, W, hdev));
        const int nout = ncol * nv;
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
// X_k += T_k for the active columns
__global__ void k_kr_add(int N, const double2 *T, const int *active, double2 *X)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int k = blockIdx.y;
    if (t >= N || !active[k]) return;
    const double2 v = T[(long long)k * N + t];
    double2 *x = X + (long long)k * N + t;
    *x = make_double2(x->x + v.x, x->y + v.y);
}

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
    // the Arnoldi bookkeeping lives on the device: Hessenberg matrices, rotations,
    // rotated right-hand sides, the CGS2 sums and the y of each column
    const size_t hb = sizeof(double2) * (size_t)ncol * (m + 1) * m, gb = sizeof(double2) * (size_t)ncol * (m + 1),
                 rb = sizeof(double2) * (size_t)ncol * m;
    MIDAS_TRY(ensure(c, S_KRYLOV, vbytes * (m + 1 + nz) + 3 * vbytes + sizeof(double2) * ((size_t)ncol * (m + 2) * nblk +
                                                                                     (size_t)ncol * (m + 2) + 64) +
                                      hb + 2 * gb + 3 * rb + sizeof(double2) * ncol + 2 * sizeof(double) * ncol +
                                      sizeof(int) * ncol + vbytes + 17 * 256,
                      &p));
    char *base = (char *)p;
    auto take = [&](size_t bytes) { char *q = base; base += (bytes + 255) & ~(size_t)255; return q; };
    double2 *V = (double2 *)take(vbytes * (m + 1));
    double2 *Zp = net ? (double2 *)take(vbytes * m) : nullptr;
    double2 *W = (double2 *)take(vbytes), *R = (double2 *)take(vbytes), *Tz = (double2 *)take(vbytes);
    double2 *partial = (double2 *)take(sizeof(double2) * (size_t)ncol * (m + 2) * nblk);
    double2 *hdev = (double2 *)take(sizeof(double2) * ((size_t)ncol * (m + 2) + 64));
    double2 *Hd = (double2 *)take(hb), *gd = (double2 *)take(gb), *hc = (double2 *)take(gb);
    double2 *csd = (double2 *)take(rb), *snd = (double2 *)take(rb), *yd = (double2 *)take(rb);
    double2 *n2d = (double2 *)take(sizeof(double2) * ncol);
    double *estd = (double *)take(sizeof(double) * ncol), *bnd = (double *)take(sizeof(double) * ncol);
    int *adev = (int *)take(sizeof(int) * ncol);
    double2 *Stage = (double2 *)take(vbytes);   // v_j, copied out of the Krylov basis
    int *jd = (int *)take(sizeof(int));          // the Arnoldi index, on the device
    Kr kr{c, N, ncol, partial, hdev, nblk};
    const dim3 gv(kr_blocks(N), ncol);
    const unsigned gc = (unsigned)((ncol + 127) / 128);
    using cd = std::complex<double>;
    std::vector<cd> hv;
    // ||b_k||
    std::vector<double> bn(ncol), rn(ncol), hest(ncol);
    MIDAS_TRY(kr.dots(B, 0, 1, B, hv));
    for (int k = 0; k < ncol; ++k) bn[k] = sqrt(std::max(hv[k].real(), 0.0));
    MIDAS_CUDA(c, cudaMemcpyAsync(bnd, bn.data(), sizeof(double) * ncol, cudaMemcpyHostToDevice, c->stream));
    int total = 0;
    double worst = 1e300;
    std::vector<int> active(ncol, 1);
    const long long tot = (long long)N * ncol;
    const unsigned gt = (unsigned)((tot + KR_THREADS - 1) / KR_THREADS);
    // One Arnoldi step, the index j read from (and advanced in) device memory:
    // W = Z M^-1 v_j, CGS2 against v_0..v_j, v_{j+1} = W / |W|, the Hessenberg
    // column, rotations and residual estimates.
    auto step = [&]() -> int {
        const double2 *zin = Stage;
        ++c->launches;
        k_kr_slot<<<gt, KR_THREADS, 0, c->stream>>>(tot, V, vs, jd, 0, Stage, 0);
        if (net) {
            MIDAS_TRY(nn_prec_apply(c, net, ncol, Stage, N, Tz, N));
            ++c->launches;
            k_kr_slot<<<gt, KR_THREADS, 0, c->stream>>>(tot, Zp, vs, jd, 0, Tz, 1);   // P(v_j) kept
            zin = Tz;
        } else if (jacobi) {
            ++c->launches;
            k_kr_jacobi<<<dim3(kr_blocks(N), ncol), KR_THREADS, 0, c->stream>>>(c->n, ncol, c->znnpp, Stage, Tz);
            zin = Tz;
        }
        MIDAS_TRY(lattice_matvec(c, ncol, zin, N, nullptr, 0, W, N, S_LFFT));
        for (int pass = 0; pass < 2; ++pass) {   // CGS2, the sums collected in hc
            MIDAS_TRY(kr.dots_dev(V, vs, m + 1, W, hdev, hc, m + 1, pass == 0, jd));
            ++c->launches;
            k_kr_axpy<<<gv, KR_THREADS, 0, c->stream>>>(N, ncol, m + 1, V, vs, hdev, m + 1, -1.0, adev, W, jd);
        }
        MIDAS_TRY(kr.dots_dev(W, 0, 1, W, n2d));
        c->launches += 3;
        k_kr_normalise<<<gv, KR_THREADS, 0, c->stream>>>(N, W, n2d, V, jd, vs);
        k_kr_givens<<<gc, 128, 0, c->stream>>>(ncol, jd, m, hc, m + 1, n2d, adev, bnd, Hd, gd, csd, snd, estd);
        k_kr_next<<<1, 1, 0, c->stream>>>(jd);
        MIDAS_CUDA(c, cudaGetLastError());
        return MIDAS_OK;
    };
    // Steps after the first (which sets up every buffer) replay one captured graph
    // of step(); not while per-kernel profiling events are being recorded.
    const bool use_graph = !c->kprof.on;
    cudaGraphExec_t gexec = nullptr;
    long long glaunches = 0;
    struct ExecGuard {
        cudaGraphExec_t *e;
        ~ExecGuard() { if (*e) cudaGraphExecDestroy(*e); }
    } exec_guard{&gexec};
    auto capture = [&]() -> int {
        const long long l0 = c->launches;
        MIDAS_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        const int st = step();
        cudaGraph_t graph = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(c->stream, &graph);
        if (st != MIDAS_OK) {
            if (graph) cudaGraphDestroy(graph);
            return st;
        }
        if (ee != cudaSuccess || !graph) return c->err.set(MIDAS_ERR_CUDA, "gmres: Arnoldi-step capture failed");
        const cudaError_t ei = cudaGraphInstantiate(&gexec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) {
            gexec = nullptr;
            return c->err.set(MIDAS_ERR_CUDA, "gmres: Arnoldi-step graph instantiation failed");
        }
        glaunches = c->launches - l0;
        c->launches = l0;
        return MIDAS_OK;
    };
    while (true) {
        // true residual R = B - Z X (FP64)
        MIDAS_TRY(lattice_matvec(c, ncol, X, N, B, N, R, N, S_LFFT));
        MIDAS_TRY(kr.dots(R, 0, 1, R, hv));   // leaves |r_k|^2 in hdev as well
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
        MIDAS_CUDA(c, cudaMemcpyAsync(adev, active.data(), sizeof(int) * ncol, cudaMemcpyHostToDevice, c->stream));
        // v0 = r / ||r||, g = (||r||, 0, ...)
        c->launches += 2;
        k_kr_normalise<<<gv, KR_THREADS, 0, c->stream>>>(N, R, hdev, V);
        k_kr_g0<<<(unsigned)((ncol * (m + 1) + 127) / 128), 128, 0, c->stream>>>(ncol, m, hdev, gd);
        MIDAS_CUDA(c, cudaMemsetAsync(jd, 0, sizeof(int), c->stream));
        int j;
        bool inner_done = false;
        for (j = 0; j < m && total < maxit && !inner_done; ++j, ++total) {
            if (j == 0 || !use_graph) {
                MIDAS_TRY(step());
            } else {
                if (!gexec) MIDAS_TRY(capture());
                MIDAS_CUDA(c, cudaGraphLaunch(gexec, c->stream));
                c->launches += glaunches;
            }
            MIDAS_CUDA(c, cudaMemcpyAsync(hest.data(), estd, sizeof(double) * ncol, cudaMemcpyDeviceToHost, c->stream));
            MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
            double est = 0;
            for (int k = 0; k < ncol; ++k) {
                if (!(hest[k] == hest[k])) return c->err.set(MIDAS_ERR_NOT_CONVERGED, "gmres: NaN in the Arnoldi process");
                est = std::max(est, hest[k]);
            }
            inner_done = est <= 0.5 * tol;
        }
        // x += M^-1 V y with H y = g (upper triangular, j x j), y on the device
        ++c->launches;
        k_kr_backsolve<<<gc, 128, 0, c->stream>>>(ncol, j, m, Hd, gd, adev, yd);
        if (net) {   // x += sum_j P(v_j) y_j
            ++c->launches;
            k_kr_axpy<<<gv, KR_THREADS, 0, c->stream>>>(N, ncol, j, Zp, vs, yd, m, 1.0, adev, X);
        } else if (jacobi) {
            MIDAS_CUDA(c, cudaMemsetAsync(W, 0, vbytes, c->stream));
            c->launches += 3;
            k_kr_axpy<<<gv, KR_THREADS, 0, c->stream>>>(N, ncol, j, V, vs, yd, m, 1.0, adev, W);
            k_kr_jacobi<<<dim3(kr_blocks(N), ncol), KR_THREADS, 0, c->stream>>>(c->n, ncol, c->znnpp, W, Tz);
            k_kr_add<<<gv, KR_THREADS, 0, c->stream>>>(N, Tz, adev, X);
        } else {
            ++c->launches;
            k_kr_axpy<<<gv, KR_THREADS, 0, c->stream>>>(N, ncol, j, V, vs, yd, m, 1.0, adev, X);
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
