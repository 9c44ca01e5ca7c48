// midas_gpu.cu -- C ABI of the GB300 MIDAS hot path (see include/midas_gpu.h).
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>

#include "common.cuh"
#include "kernels.cuh"

namespace midas {

int launch_cext_cabs(midas_gpu_ctx *c, int ntr, const double *th, const double *ph, const double2 *E, double *cext,
                     double *cabs);
int launch_smatrix(midas_gpu_ctx *c, int nrx, const double *rth, const double *rph, int ntr, const double2 *E,
                   double2 *S);
int scattering_quantities(midas_gpu_ctx *c, int quad_tr, int quad_rx, int ntr_theta, int ntr_phi,
                          const double *tr_theta, const double *tr_phi, int nrx_theta, int nrx_phi, int nrx_tot,
                          const double *rx_theta, const double *rx_phi, const double *S, const double *cext,
                          const double *cabs, double dm, double k0, int cext_intfields, const double *w_tr,
                          const double *w_rx, double *q_dir, double *q_avg);
template <typename TA, typename TB>
int zgemm_x3(midas_gpu_ctx *c, int M, int N, int K, const TA *A, long long ars, long long acs, int conjA,
             const TB *B, long long brs, long long bcs, float *D, long long ldd, float alpha, float beta);
int heev_dev(midas_gpu_ctx *c, int batch, int m, double2 *A, long long lda, long long sa, double2 *H, double2 *V,
             long long sv, double *W);
int cbfm_run(midas_gpu_ctx *c, int nblocks, const int *blk_offsets, const int *ext_offsets, const int *ext_idx,
             int ncbf, const double *cbf_theta, const double *cbf_phi, double thr_cbf, double res_sr, int flags,
             double eps_aca, int aca_itmax, int ntr, const double *theta, const double *phi, double2 *E, int *K,
             midas_gpu_info *info);
int aca_run(midas_gpu_ctx *c, int row0, int nrows, int col0, int ncols, double eps, int itmax, double2 *U,
            double2 *V, int *rank);

int ensure(midas_gpu_ctx *ctx, int slot, size_t bytes, void **out)
{
    if (slot < 0 || slot >= (int)ctx->pool.size()) return ctx->err.set(MIDAS_ERR_ARG, "bad pool slot");
    DBuf &b = ctx->pool[slot];
    if (b.bytes < bytes && ctx->no_alloc) {
        char m[160];
        snprintf(m, sizeof m, "pool slot %d holds %zu bytes but %zu were requested on the allocation-free path", slot,
                 b.bytes, bytes);
        return ctx->err.set(MIDAS_ERR_ALLOC, m);
    }
    if (b.bytes < bytes) {
        if (b.p) { cudaStreamSynchronize(ctx->stream); cudaFree(b.p); b.p = nullptr; b.bytes = 0; }
        size_t want = bytes + bytes / 8 + 256;
        cudaError_t e = cudaMalloc(&b.p, want);
        if (e != cudaSuccess) {
            cudaGetLastError();
            char m[128];
            snprintf(m, sizeof m, "cudaMalloc(%zu bytes) failed in pool slot %d", want, slot);
            return ctx->err.set(MIDAS_ERR_ALLOC, m);
        }
        b.bytes = want;
    }
    *out = b.p;
    return MIDAS_OK;
}

bool is_device_ptr(const void *p)
{
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int to_device(midas_gpu_ctx *ctx, const void *p, size_t bytes, int slot, const void **out)
{
    if (is_device_ptr(p)) { *out = p; return MIDAS_OK; }
    void *d;
    MIDAS_TRY(ensure(ctx, slot, bytes, &d));
    MIDAS_CUDA(ctx, cudaMemcpyAsync(d, p, bytes, cudaMemcpyHostToDevice, ctx->stream));
    *out = d;
    return MIDAS_OK;
}

int device_sms(midas_gpu_ctx *c)
{
    static std::atomic<int> cache[64];
    std::atomic<int> &slot = cache[c->device & 63];
    int v = slot.load(std::memory_order_relaxed);
    if (v > 0) return v;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess || v <= 0) {
        cudaGetLastError();
        return 152;
    }
    slot.store(v, std::memory_order_relaxed);
    return v;
}

int side_stream(midas_gpu_ctx *c, cudaStream_t *out)
{
    if (!c->side) {
        int prio = 0;
        MIDAS_CUDA(c, cudaStreamGetPriority(c->stream, &prio));
        MIDAS_CUDA(c, cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, prio));
        MIDAS_CUDA(c, cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
        MIDAS_CUDA(c, cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
    }
    *out = c->side;
    return MIDAS_OK;
}

void destroy_side(midas_gpu_ctx *c)
{
    if (c->side) {
        cudaStreamSynchronize(c->side);
        cudaStreamDestroy(c->side);
    }
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    c->side = nullptr;
    c->ev_fork = c->ev_join = nullptr;
}

int kp_begin(midas_gpu_ctx *c)
{
    KProf &k = c->kprof;
    if (!k.on) return -1;
    while (k.ev.size() < k.used + 2) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) { cudaGetLastError(); k.on = false; return -1; }
        k.ev.push_back(e);
    }
    int i = (int)k.used;
    k.used += 2;
    if (cudaEventRecord(k.ev[i], c->stream) != cudaSuccess) { cudaGetLastError(); return -1; }
    return i;
}

void kp_end(midas_gpu_ctx *c, int e0, int cls, double flops, double bytes)
{
    if (e0 < 0) return;
    KProf &k = c->kprof;
    if (cudaEventRecord(k.ev[e0 + 1], c->stream) != cudaSuccess) { cudaGetLastError(); return; }
    k.rec.push_back({cls, e0, flops, bytes});
}

int kp_flush(midas_gpu_ctx *c)
{
    KProf &k = c->kprof;
    if (k.rec.empty()) { k.used = 0; return MIDAS_OK; }
    MIDAS_CUDA(c, cudaEventSynchronize(k.ev[k.rec.back().e0 + 1]));
    for (const auto &r : k.rec) {
        float ms = 0;
        MIDAS_CUDA(c, cudaEventElapsedTime(&ms, k.ev[r.e0], k.ev[r.e0 + 1]));
        k.ms[r.cls] += ms;
        k.flops[r.cls] += r.flops;
        k.bytes[r.cls] += r.bytes;
        k.n[r.cls] += 1;
    }
    k.rec.clear();
    k.used = 0;
    return MIDAS_OK;
}

int check_flag(midas_gpu_ctx *ctx, const char *where)
{
    int h = 0;
    MIDAS_CUDA(ctx, cudaMemcpyAsync(&h, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MIDAS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    MIDAS_TRY(kp_flush(ctx));
    if (h == 0) return MIDAS_OK;
    MIDAS_CUDA(ctx, cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
    std::string w(where);
    if (h & DEV_TIMEOUT) return ctx->err.set(MIDAS_ERR_DEVICE_TIMEOUT, w + ": bounded device wait expired");
    if (h & DEV_ZERO_PIVOT) return ctx->err.set(MIDAS_ERR_SINGULAR, w + ": SINGULAR MATRIX (zero pivot)");
    return ctx->err.set(MIDAS_ERR_CUDA, w + ": device error flag set");
}

// copy a device result to a caller pointer (host or device)
static int copy_out(midas_gpu_ctx *c, void *dst, const void *src, size_t bytes)
{
    if (dst == src) return MIDAS_OK;
    MIDAS_CUDA(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    return MIDAS_OK;
}

// index arrays: convert to 0-based device ints in `slot`
__global__ void k_rebase(const int *in, int *out, int n, int base)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[i] - base;
}

static int idx_to_device(midas_gpu_ctx *c, const int *idx, int n, int slot, const int **out)
{
    const void *d;
    MIDAS_TRY(to_device(c, idx, sizeof(int) * (size_t)n, slot, &d));
    if (c->opts.index_base == 0) { *out = (const int *)d; return MIDAS_OK; }
    void *o;
    MIDAS_TRY(ensure(c, slot == S_IN0 ? S_IN4 : S_IN5, sizeof(int) * (size_t)n, &o));
    ++c->launches;
    k_rebase<<<(n + 255) / 256, 256, 0, c->stream>>>((const int *)d, (int *)o, n, c->opts.index_base);
    MIDAS_CUDA(c, cudaGetLastError());
    *out = (const int *)o;
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// uniform-lattice detection (host): every centroid = o + (i, j, k) d
// ---------------------------------------------------------------------------
static void detect_lattice(midas_gpu_ctx *c, const std::vector<double> &x, const std::vector<double> &y,
                           const std::vector<double> &z, const std::vector<double> &sc)
{
    c->lattice = 0;
    int n = (int)x.size();
    if (n < 2) return;
    double d = sc[0];
    for (int i = 1; i < n; ++i)
        if (sc[i] != d) return;
    if (!(d > 0)) return;
    std::vector<int> ijk(3 * (size_t)n);
    const std::vector<double> *v[3] = {&x, &y, &z};
    for (int a = 0; a < 3; ++a) {
        double o = (*v[a])[0];
        int lo = 0, hi = 0;
        for (int i = 0; i < n; ++i) {
            double q = ((*v[a])[i] - o) / d;
            double r = std::nearbyint(q);
            if (fabs(q - r) > 1e-7) return;
            int ii = (int)r;
            ijk[3 * (size_t)i + a] = ii;
            lo = std::min(lo, ii);
            hi = std::max(hi, ii);
        }
        c->lat_o[a] = o;
        c->lat_lo[a] = lo;
        c->lat_hi[a] = hi;
        c->lat_dim[a] = 2 * (hi - lo) + 1;
    }
    size_t tot = (size_t)c->lat_dim[0] * c->lat_dim[1] * c->lat_dim[2];
    if (tot > (size_t)64 << 20) return;   // offset table would exceed ~6 GB: keep direct evaluation
    if (cudaMalloc(&c->lat_ijk, sizeof(int) * ijk.size()) != cudaSuccess) { cudaGetLastError(); return; }
    cudaMemcpyAsync(c->lat_ijk, ijk.data(), sizeof(int) * ijk.size(), cudaMemcpyHostToDevice, c->stream);
    c->lat_d = d;
    c->lattice = 1;
}

static void free_cells(midas_gpu_ctx *c)
{
    void *ptrs[] = {c->x, c->y, c->z, c->sc, c->an, c->kappa, c->eps, c->che, c->znnpp, c->fk4, c->fk8,
                    c->lat_ijk, c->lat_tab4, c->lat_tab8};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    c->x = c->y = c->z = c->sc = c->an = c->kappa = nullptr;
    c->eps = c->che = c->znnpp = c->fk8 = nullptr;
    c->fk4 = nullptr;
    c->lat_ijk = nullptr;
    c->lat_tab4 = nullptr;
    c->lat_tab8 = nullptr;
    c->lattice = 0;
    c->n = 0;
}

static int need_cells(midas_gpu_ctx *c)
{
    if (c->n <= 0) return c->err.set(MIDAS_ERR_STATE, "no cells: call midas_gpu_set_cells first");
    return MIDAS_OK;
}

// ensure the lattice offset tables exist (FAST fill mode)
static int need_tables(midas_gpu_ctx *c)
{
    if (c->opts.fill_mode != MIDAS_FILL_FAST || !c->lattice || c->lat_tab4) return MIDAS_OK;
    size_t tot = (size_t)c->lat_dim[0] * c->lat_dim[1] * c->lat_dim[2];
    MIDAS_CUDA(c, cudaMalloc(&c->lat_tab4, sizeof(float2) * 6 * tot));
    MIDAS_CUDA(c, cudaMalloc(&c->lat_tab8, sizeof(double2) * 6 * tot));
    return launch_lat_table(c);
}

}  // namespace midas

using namespace midas;

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

void midas_gpu_default_opts(midas_gpu_opts *o)
{
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->struct_size = sizeof(midas_gpu_opts);
    o->device = 0;
    o->index_base = 0;
    o->solve_mode = MIDAS_SOLVE_MIXED;
    o->fill_mode = MIDAS_FILL_FAITHFUL;
    o->ir_max_iter = 30;
    o->ir_tol = 1e-13;
    o->verbose = 0;
}

int midas_gpu_init(const midas_gpu_opts *opts, midas_gpu_ctx **out)
{
    if (!out) return MIDAS_ERR_ARG;
    *out = nullptr;
    midas_gpu_opts o;
    midas_gpu_default_opts(&o);
    if (opts) {
        if (opts->struct_size != (int)sizeof(midas_gpu_opts)) return MIDAS_ERR_ARG;
        o = *opts;
    }
    if (o.index_base != 0 && o.index_base != 1) return MIDAS_ERR_ARG;
    if (o.solve_mode != MIDAS_SOLVE_MIXED && o.solve_mode != MIDAS_SOLVE_FP64) return MIDAS_ERR_ARG;
    if (o.fill_mode != MIDAS_FILL_FAITHFUL && o.fill_mode != MIDAS_FILL_FAST) return MIDAS_ERR_ARG;
    // The CBFM pipeline drives ~20 streams (lanes, their side streams, eigen-solve and
    // finisher streams).  With the default 8 hardware work queues streams share queues,
    // and a long kernel (an eigen-solve, ~50 ms on one SM) holds up the kernels queued
    // behind it from other streams.  Takes effect only if this process has no CUDA
    // context yet; an explicit setting is kept.
    setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || o.device < 0 || o.device >= ndev) {
        cudaGetLastError();
        return MIDAS_ERR_CUDA;
    }
    if (cudaSetDevice(o.device) != cudaSuccess) return MIDAS_ERR_CUDA;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, o.device) != cudaSuccess) return MIDAS_ERR_CUDA;
    if (prop.major != 10 || prop.minor != 3) return MIDAS_ERR_UNSUPPORTED;   // built for sm_103a only
    midas_gpu_ctx *c = new midas_gpu_ctx();
    c->opts = o;
    c->device = o.device;
    c->pi = ref_pi_host();
    c->pool.resize(S_NSLOTS);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&c->d_flag, sizeof(int)) != cudaSuccess ||
        cudaMemset(c->d_flag, 0, sizeof(int)) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return MIDAS_ERR_CUDA;
    }
    *out = c;
    return MIDAS_OK;
}

int midas_gpu_free(midas_gpu_ctx *c)
{
    if (!c) return MIDAS_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    free_cells(c);
    lattice_fft_release(c);
    for (auto &b : c->pool)
        if (b.p) cudaFree(b.p);
    if (c->d_flag) cudaFree(c->d_flag);
    if (c->cusolver) destroy_cusolver(c->cusolver);
    free_lanes(c);
    destroy_side(c);
    for (cudaEvent_t e : c->kprof.ev) cudaEventDestroy(e);
    cudaStreamDestroy(c->stream);
    delete c;
    return MIDAS_OK;
}

const char *midas_gpu_last_error(const midas_gpu_ctx *c)
{
    if (!c) return "null context";
    return c->err.msg.c_str();
}

int midas_gpu_set_cells(midas_gpu_ctx *c, int n, const double *xc, const double *yc, const double *zc,
                        const double *sc, const double *eps_re, const double *eps_im, double k0)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    if (n <= 0 || !xc || !yc || !zc || !sc || !eps_re || !eps_im || !(k0 > 0))
        return c->err.set(MIDAS_ERR_ARG, "set_cells: bad arguments");
    cudaSetDevice(c->device);
    free_cells(c);
    std::vector<double> hx(n), hy(n), hz(n), hs(n), er(n), ei(n);
    MIDAS_CUDA(c, cudaMemcpy(hx.data(), xc, sizeof(double) * n, cudaMemcpyDefault));
    MIDAS_CUDA(c, cudaMemcpy(hy.data(), yc, sizeof(double) * n, cudaMemcpyDefault));
    MIDAS_CUDA(c, cudaMemcpy(hz.data(), zc, sizeof(double) * n, cudaMemcpyDefault));
    MIDAS_CUDA(c, cudaMemcpy(hs.data(), sc, sizeof(double) * n, cudaMemcpyDefault));
    MIDAS_CUDA(c, cudaMemcpy(er.data(), eps_re, sizeof(double) * n, cudaMemcpyDefault));
    MIDAS_CUDA(c, cudaMemcpy(ei.data(), eps_im, sizeof(double) * n, cudaMemcpyDefault));
    std::vector<double2> he(n);
    for (int i = 0; i < n; ++i) he[i] = make_double2(er[i], ei[i]);
    MIDAS_CUDA(c, cudaMalloc(&c->x, sizeof(double) * n));
    MIDAS_CUDA(c, cudaMalloc(&c->y, sizeof(double) * n));
    MIDAS_CUDA(c, cudaMalloc(&c->z, sizeof(double) * n));
    MIDAS_CUDA(c, cudaMalloc(&c->sc, sizeof(double) * n));
    MIDAS_CUDA(c, cudaMalloc(&c->an, sizeof(double) * n));
    MIDAS_CUDA(c, cudaMalloc(&c->kappa, sizeof(double) * n));
    MIDAS_CUDA(c, cudaMalloc(&c->eps, sizeof(double2) * n));
    MIDAS_CUDA(c, cudaMalloc(&c->che, sizeof(double2) * n));
    MIDAS_CUDA(c, cudaMalloc(&c->znnpp, sizeof(double2) * n));
    MIDAS_CUDA(c, cudaMalloc(&c->fk8, sizeof(double2) * n));
    MIDAS_CUDA(c, cudaMalloc(&c->fk4, sizeof(float2) * n));
    MIDAS_CUDA(c, cudaMemcpyAsync(c->x, hx.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    MIDAS_CUDA(c, cudaMemcpyAsync(c->y, hy.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    MIDAS_CUDA(c, cudaMemcpyAsync(c->z, hz.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    MIDAS_CUDA(c, cudaMemcpyAsync(c->sc, hs.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    MIDAS_CUDA(c, cudaMemcpyAsync(c->eps, he.data(), sizeof(double2) * n, cudaMemcpyHostToDevice, c->stream));
    c->n = n;
    c->k0 = k0;
    MIDAS_TRY(launch_set_cells(c));
    detect_lattice(c, hx, hy, hz, hs);
    ++c->cells_version;   // the lattice FFT spectra of the previous cells are stale
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    return MIDAS_OK;
}

int midas_gpu_get_cell_params(midas_gpu_ctx *c, double *a_n, double *che, double *znnpp, double *kappa)
{
    if (!c) return MIDAS_ERR_ARG;
    MIDAS_TRY(need_cells(c));
    size_t n = c->n;
    if (a_n) MIDAS_CUDA(c, cudaMemcpy(a_n, c->an, sizeof(double) * n, cudaMemcpyDefault));
    if (che) MIDAS_CUDA(c, cudaMemcpy(che, c->che, sizeof(double2) * n, cudaMemcpyDefault));
    if (znnpp) MIDAS_CUDA(c, cudaMemcpy(znnpp, c->znnpp, sizeof(double2) * n, cudaMemcpyDefault));
    if (kappa) MIDAS_CUDA(c, cudaMemcpy(kappa, c->kappa, sizeof(double) * n, cudaMemcpyDefault));
    return MIDAS_OK;
}

int midas_gpu_mom_fill(midas_gpu_ctx *c, int r0, int nr, int c0, int nc, double *Z)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    MIDAS_TRY(need_cells(c));
    int N = 3 * c->n;
    if (!Z || r0 < 0 || c0 < 0 || nr <= 0 || nc <= 0 || r0 + nr > N || c0 + nc > N)
        return c->err.set(MIDAS_ERR_ARG, "mom_fill: block outside the 3n x 3n matrix");
    MIDAS_TRY(need_tables(c));
    size_t bytes = sizeof(double2) * (size_t)nr * nc;
    double2 *out = (double2 *)Z;
    if (!is_device_ptr(Z)) {
        void *p;
        MIDAS_TRY(ensure(c, S_OUT0, bytes, &p));
        out = (double2 *)p;
    }
    MIDAS_TRY(launch_mom_fill(c, r0, nr, c0, nc, out, nullptr, 1, (size_t)nr));
    return copy_out(c, Z, out, bytes);
}

int midas_gpu_mom_rhs(midas_gpu_ctx *c, int ntr, const double *theta, const double *phi, double *V)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    MIDAS_TRY(need_cells(c));
    if (ntr <= 0 || !theta || !phi || !V) return c->err.set(MIDAS_ERR_ARG, "mom_rhs: bad arguments");
    const void *th, *ph;
    MIDAS_TRY(to_device(c, theta, sizeof(double) * ntr, S_IN0, &th));
    MIDAS_TRY(to_device(c, phi, sizeof(double) * ntr, S_IN1, &ph));
    size_t N = 3 * (size_t)c->n, bytes = sizeof(double2) * N * 2 * ntr;
    double2 *out = (double2 *)V;
    if (!is_device_ptr(V)) {
        void *p;
        MIDAS_TRY(ensure(c, S_OUT0, bytes, &p));
        out = (double2 *)p;
    }
    MIDAS_TRY(launch_mom_rhs<double2>(c, ntr, (const double *)th, (const double *)ph, out, 1, N));
    return copy_out(c, V, out, bytes);
}

int midas_gpu_incident_field(midas_gpu_ctx *c, int ncell, const int *idx, int ntr, const double *theta,
                             const double *phi, double *E)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    MIDAS_TRY(need_cells(c));
    if (ntr <= 0 || !theta || !phi || !E || (idx && ncell <= 0)) return c->err.set(MIDAS_ERR_ARG, "incident_field");
    if (!idx) ncell = c->n;
    const int *didx = nullptr;
    if (idx) MIDAS_TRY(idx_to_device(c, idx, ncell, S_IN2, &didx));
    const void *th, *ph;
    MIDAS_TRY(to_device(c, theta, sizeof(double) * ntr, S_IN0, &th));
    MIDAS_TRY(to_device(c, phi, sizeof(double) * ntr, S_IN1, &ph));
    size_t N = 3 * (size_t)ncell, bytes = sizeof(double2) * N * 2 * ntr;
    double2 *out = (double2 *)E;
    if (!is_device_ptr(E)) {
        void *p;
        MIDAS_TRY(ensure(c, S_OUT0, bytes, &p));
        out = (double2 *)p;
    }
    MIDAS_TRY(launch_incident4<double2>(c, ncell, didx, ntr, (const double *)th, (const double *)ph, out, 1, N));
    return copy_out(c, E, out, bytes);
}

int midas_gpu_incident_field_spherical(midas_gpu_ctx *c, int ncell, const int *idx, int ntr, const double *theta,
                                       const double *phi, double *E)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    MIDAS_TRY(need_cells(c));
    if (ntr <= 0 || !theta || !phi || !E || (idx && ncell <= 0))
        return c->err.set(MIDAS_ERR_ARG, "incident_field_spherical");
    if (!idx) ncell = c->n;
    const int *didx = nullptr;
    if (idx) MIDAS_TRY(idx_to_device(c, idx, ncell, S_IN2, &didx));
    const void *th, *ph;
    MIDAS_TRY(to_device(c, theta, sizeof(double) * ntr, S_IN0, &th));
    MIDAS_TRY(to_device(c, phi, sizeof(double) * ntr, S_IN1, &ph));
    size_t N = 3 * (size_t)ncell, bytes = sizeof(double2) * N * 2 * ntr;
    double2 *out = (double2 *)E;
    if (!is_device_ptr(E)) {
        void *p;
        MIDAS_TRY(ensure(c, S_OUT0, bytes, &p));
        out = (double2 *)p;
    }
    MIDAS_TRY(launch_incident_sph<double2>(c, ncell, didx, ntr, (const double *)th, (const double *)ph, out, 1, N));
    return copy_out(c, E, out, bytes);
}

int midas_gpu_block_fill(midas_gpu_ctx *c, int n1, const int *idx1, int n2, const int *idx2, double *Z)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    MIDAS_TRY(need_cells(c));
    if (n1 <= 0 || n2 <= 0 || !idx1 || !idx2 || !Z) return c->err.set(MIDAS_ERR_ARG, "block_fill");
    MIDAS_TRY(need_tables(c));
    const int *d1, *d2;
    MIDAS_TRY(idx_to_device(c, idx1, n1, S_IN0, &d1));
    MIDAS_TRY(idx_to_device(c, idx2, n2, S_IN1, &d2));
    size_t bytes = sizeof(double2) * 9 * (size_t)n1 * n2;
    double2 *out = (double2 *)Z;
    if (!is_device_ptr(Z)) {
        void *p;
        MIDAS_TRY(ensure(c, S_OUT0, bytes, &p));
        out = (double2 *)p;
    }
    MIDAS_TRY(launch_block_fill4<double2>(c, n1, d1, n2, d2, 0, 0.0, 0, out, 1, 3 * (size_t)n1));
    return copy_out(c, Z, out, bytes);
}

int midas_gpu_sr_fill(midas_gpu_ctx *c, int s, const int *idx, double fsr, int homog, double *Z, long long *nnz,
                      double *fn)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    MIDAS_TRY(need_cells(c));
    if (s <= 0 || !idx || !(fsr > 0)) return c->err.set(MIDAS_ERR_ARG, "sr_fill");
    MIDAS_TRY(need_tables(c));
    const int *d;
    MIDAS_TRY(idx_to_device(c, idx, s, S_IN0, &d));
    int first;
    MIDAS_CUDA(c, cudaMemcpyAsync(&first, d, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (first < 0 || first >= c->n) return c->err.set(MIDAS_ERR_ARG, "sr_fill: cell index out of range");
    // nnz / fn for this fSR through the ladder scan (the ladder always contains the reference's values)
    double all_nnz[11], all_fn[11], fnz;
    double fsr_sel;
    long long nz;
    MIDAS_TRY(sr_ladder(c, s, d, first, homog, 1e300, &fsr_sel, &nz, 1, all_nnz, all_fn, &fnz));
    static const double ladder[11] = {1e2, 1e3, 2e3, 3e3, 4e3, 5e3, 6e3, 7e3, 8e3, 9e3, 1e4};
    int j = -1;
    for (int k = 0; k < 11; ++k)
        if (ladder[k] == fsr) j = k;
    if (nnz) *nnz = j >= 0 ? (long long)all_nnz[j] : -1;
    if (fn) *fn = j >= 0 ? all_fn[j] : -1;
    if (Z) {
        double2 zn;
        MIDAS_CUDA(c, cudaMemcpy(&zn, c->znnpp + first, sizeof(double2), cudaMemcpyDeviceToHost));
        double thr = hypot(1 - zn.x, -zn.y) / fsr;
        size_t bytes = sizeof(double2) * 9 * (size_t)s * s;
        double2 *out = (double2 *)Z;
        if (!is_device_ptr(Z)) {
            void *p;
            MIDAS_TRY(ensure(c, S_OUT0, bytes, &p));
            out = (double2 *)p;
        }
        MIDAS_TRY(launch_block_fill4<double2>(c, s, d, s, d, 1, thr, homog, out, 1, 3 * (size_t)s));
        MIDAS_TRY(copy_out(c, Z, out, bytes));
    }
    return MIDAS_OK;
}

int midas_gpu_set_fsr(midas_gpu_ctx *c, int s, const int *idx, int homog, double res_sr, double *fsr,
                      long long *nnz)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    MIDAS_TRY(need_cells(c));
    if (s <= 0 || !idx || !fsr) return c->err.set(MIDAS_ERR_ARG, "set_fsr");
    MIDAS_TRY(need_tables(c));
    const int *d;
    MIDAS_TRY(idx_to_device(c, idx, s, S_IN0, &d));
    int first;
    MIDAS_CUDA(c, cudaMemcpyAsync(&first, d, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (first < 0 || first >= c->n) return c->err.set(MIDAS_ERR_ARG, "set_fsr: cell index out of range");
    if (!(res_sr > 0)) res_sr = (double)1e-2f;
    return sr_ladder(c, s, d, first, homog, res_sr, fsr, nnz, 0, nullptr, nullptr, nullptr);
}

int midas_gpu_aca(midas_gpu_ctx *c, int row0, int nrows, int col0, int ncols, double eps, int itmax, double *U,
                  double *V, int *rank)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    MIDAS_TRY(need_cells(c));
    int N = 3 * c->n;
    if (row0 < 0 || col0 < 0 || nrows <= 0 || ncols <= 0 || row0 % 3 || col0 % 3 || nrows % 3 || ncols % 3 ||
        row0 + nrows > N || col0 + ncols > N || itmax < 2 || !U || !V || !rank)
        return c->err.set(MIDAS_ERR_ARG, "aca: bad block");
    cudaSetDevice(c->device);
    MIDAS_TRY(need_tables(c));
    size_t bu = sizeof(double2) * (size_t)nrows * itmax, bv = sizeof(double2) * (size_t)itmax * ncols;
    void *pu, *pv;
    MIDAS_TRY(ensure(c, S_OUT0, bu, &pu));
    MIDAS_TRY(ensure(c, S_OUT1, bv, &pv));
    MIDAS_TRY(aca_run(c, row0, nrows, col0, ncols, eps, itmax, (double2 *)pu, (double2 *)pv, rank));
    MIDAS_TRY(copy_out(c, U, pu, bu));
    return copy_out(c, V, pv, bv);
}

// ---------------------------------------------------------------------------
// dense solves
// ---------------------------------------------------------------------------
}  // extern "C"

namespace midas {

__global__ void k_pad_identity(double2 *Z64, float2 *Z32, long long ld, int n0, int np)
{
    int i = n0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    if (Z64) Z64[(long long)i * ld + i] = make_double2(1, 0);
    if (Z32) Z32[(long long)i * ld + i] = make_float2(1, 0);
}

// column-major complex128 (n x n, ld n) -> row-major FP64 and complex64 (np x np)
__global__ void k_transpose_in(const double2 *A, int n, double2 *Z64, float2 *Z32, long long ld)
{
    __shared__ double2 t[32][33];
    int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        int col = bx + j, row = by + threadIdx.x;
        if (row < n && col < n) t[j][threadIdx.x] = A[(long long)col * n + row];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        int row = by + j, col = bx + threadIdx.x;
        if (row < n && col < n) {
            double2 v = t[threadIdx.x][j];
            Z64[(long long)row * ld + col] = v;
            Z32[(long long)row * ld + col] = make_float2((float)v.x, (float)v.y);
        }
    }
}

// copy n x nrhs column-major (ld n) into (ld np) with zero padding
__global__ void k_copy_pad(const double2 *src, int n, int np, int nrhs, double2 *dst)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long tot = (long long)np * nrhs;
    if (i >= tot) return;
    int r = (int)(i % np), k = (int)(i / np);
    dst[i] = r < n ? src[(long long)k * n + r] : make_double2(0, 0);
}
__global__ void k_copy_unpad(const double2 *src, int n, int np, int nrhs, double2 *dst)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long tot = (long long)n * nrhs;
    if (i >= tot) return;
    int r = (int)(i % n), k = (int)(i / n);
    dst[i] = src[(long long)k * np + r];
}

}  // namespace midas

extern "C" {

int midas_gpu_dense_solve(midas_gpu_ctx *c, int n, int nrhs, const double *A, double *B, midas_gpu_info *info)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    auto t0 = std::chrono::steady_clock::now();
    if (n <= 0 || nrhs <= 0 || !A || !B) return c->err.set(MIDAS_ERR_ARG, "dense_solve: bad arguments");
    cudaSetDevice(c->device);
    if (info) memset(info, 0, sizeof(*info));
    int st;
    if (c->opts.solve_mode == MIDAS_SOLVE_FP64) {
        void *pa, *pb;
        MIDAS_TRY(ensure(c, S_Z64, sizeof(double2) * (size_t)n * n, &pa));
        MIDAS_TRY(ensure(c, S_RHS64, sizeof(double2) * (size_t)n * nrhs, &pb));
        MIDAS_CUDA(c, cudaMemcpyAsync(pa, A, sizeof(double2) * (size_t)n * n, cudaMemcpyDefault, c->stream));
        MIDAS_CUDA(c, cudaMemcpyAsync(pb, B, sizeof(double2) * (size_t)n * nrhs, cudaMemcpyDefault, c->stream));
        Timer tf(c->stream);
        st = zgesv_fp64(c, n, nrhs, (double2 *)pa, (double2 *)pb, info);
        if (info) info->t_factor_ms = tf.stop();
        if (st == MIDAS_OK) st = copy_out(c, B, pb, sizeof(double2) * (size_t)n * nrhs);
    } else {
        int np = (n + 63) / 64 * 64;
        const void *dA;
        MIDAS_TRY(to_device(c, A, sizeof(double2) * (size_t)n * n, S_IN3, &dA));
        void *p64, *p32, *pb, *px, *pbin;
        MIDAS_TRY(ensure(c, S_Z64, sizeof(double2) * (size_t)np * np, &p64));
        MIDAS_TRY(ensure(c, S_Z32, sizeof(float2) * (size_t)np * np, &p32));
        MIDAS_CUDA(c, cudaMemsetAsync(p64, 0, sizeof(double2) * (size_t)np * np, c->stream));
        MIDAS_CUDA(c, cudaMemsetAsync(p32, 0, sizeof(float2) * (size_t)np * np, c->stream));
        dim3 blk(32, 8), grd((n + 31) / 32, (n + 31) / 32);
        ++c->launches;
        k_transpose_in<<<grd, blk, 0, c->stream>>>((const double2 *)dA, n, (double2 *)p64, (float2 *)p32, np);
        if (np > n) { ++c->launches; k_pad_identity<<<1, 64, 0, c->stream>>>((double2 *)p64, (float2 *)p32, np, n, np); }
        MIDAS_TRY(to_device(c, B, sizeof(double2) * (size_t)n * nrhs, S_IN2, (const void **)&pbin));
        MIDAS_TRY(ensure(c, S_RHS64, sizeof(double2) * (size_t)np * nrhs, &pb));
        MIDAS_TRY(ensure(c, S_X64, sizeof(double2) * (size_t)np * nrhs, &px));
        long long tot = (long long)np * nrhs;
        ++c->launches;
        k_copy_pad<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>((const double2 *)pbin, n, np, nrhs,
                                                                         (double2 *)pb);
        MIDAS_CUDA(c, cudaGetLastError());
        st = mixed_solve(c, np, (float2 *)p32, (double2 *)p64, (const double2 *)pb, (double2 *)px, nrhs,
                                info);
        if (st == MIDAS_OK) {
            void *pout;
            MIDAS_TRY(ensure(c, S_OUT0, sizeof(double2) * (size_t)n * nrhs, &pout));
            long long t2 = (long long)n * nrhs;
            ++c->launches;
            k_copy_unpad<<<(unsigned)((t2 + 255) / 256), 256, 0, c->stream>>>((const double2 *)px, n, np, nrhs,
                                                                              (double2 *)pout);
            st = copy_out(c, B, pout, sizeof(double2) * (size_t)n * nrhs);
        }
    }
    if (info) {
        info->status = st;
        info->t_total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return st;
}

int midas_gpu_mom_solve(midas_gpu_ctx *c, int ntr, const double *theta, const double *phi, double *E,
                        midas_gpu_info *info)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    auto t0 = std::chrono::steady_clock::now();
    MIDAS_TRY(need_cells(c));
    if (ntr <= 0 || !theta || !phi || !E) return c->err.set(MIDAS_ERR_ARG, "mom_solve: bad arguments");
    cudaSetDevice(c->device);
    if (info) memset(info, 0, sizeof(*info));
    MIDAS_TRY(need_tables(c));
    const void *th, *ph;
    MIDAS_TRY(to_device(c, theta, sizeof(double) * ntr, S_IN0, &th));
    MIDAS_TRY(to_device(c, phi, sizeof(double) * ntr, S_IN1, &ph));
    const int n = 3 * c->n, nrhs = 2 * ntr;
    int st;
    if (c->opts.solve_mode == MIDAS_SOLVE_FP64) {
        void *pa, *pb;
        MIDAS_TRY(ensure(c, S_Z64, sizeof(double2) * (size_t)n * n, &pa));
        MIDAS_TRY(ensure(c, S_RHS64, sizeof(double2) * (size_t)n * nrhs, &pb));
        Timer tf(c->stream);
        MIDAS_TRY(launch_mom_fill(c, 0, n, 0, n, (double2 *)pa, nullptr, 1, (size_t)n));   // column-major
        MIDAS_TRY(launch_mom_rhs<double2>(c, ntr, (const double *)th, (const double *)ph, (double2 *)pb, 1, n));
        float tfill = tf.stop();
        Timer tl(c->stream);
        st = zgesv_fp64(c, n, nrhs, (double2 *)pa, (double2 *)pb, info);
        float tlu = tl.stop();
        if (info) { info->t_fill_ms = tfill; info->t_factor_ms = tlu; }
        if (st == MIDAS_OK) st = copy_out(c, E, pb, sizeof(double2) * (size_t)n * nrhs);
    } else if (lattice_fft_preferred(c, (n + 63) / 64 * 64)) {
        // cells on a compact lattice: the residuals come from the FFT operator, so
        // only the complex64 matrix (the factorisation's operand) is formed
        int np = (n + 63) / 64 * 64;
        void *p32, *pb, *px;
        MIDAS_TRY(ensure(c, S_Z32, sizeof(float2) * (size_t)np * np, &p32));
        MIDAS_TRY(ensure(c, S_RHS64, sizeof(double2) * (size_t)np * nrhs, &pb));
        MIDAS_TRY(ensure(c, S_X64, sizeof(double2) * (size_t)np * nrhs, &px));
        Timer tf(c->stream);
        if (np > n) {
            MIDAS_CUDA(c, cudaMemsetAsync(p32, 0, sizeof(float2) * (size_t)np * np, c->stream));
            ++c->launches;
            k_pad_identity<<<1, 64, 0, c->stream>>>(nullptr, (float2 *)p32, np, n, np);
            MIDAS_CUDA(c, cudaMemsetAsync(pb, 0, sizeof(double2) * (size_t)np * nrhs, c->stream));
        }
        MIDAS_TRY(launch_mom_fill(c, 0, n, 0, n, nullptr, (float2 *)p32, (size_t)np, 1));   // row-major
        MIDAS_TRY(launch_mom_rhs<double2>(c, ntr, (const double *)th, (const double *)ph, (double2 *)pb, 1, np));
        float tfill = tf.stop();
        if (info) info->t_fill_ms = tfill;
        st = mixed_solve_lattice(c, np, (float2 *)p32, (const double2 *)pb, (double2 *)px, nrhs, info);
        if (st == MIDAS_OK) {
            void *pout;
            MIDAS_TRY(ensure(c, S_OUT0, sizeof(double2) * (size_t)n * nrhs, &pout));
            long long t2 = (long long)n * nrhs;
            ++c->launches;
            k_copy_unpad<<<(unsigned)((t2 + 255) / 256), 256, 0, c->stream>>>((const double2 *)px, n, np, nrhs,
                                                                              (double2 *)pout);
            st = copy_out(c, E, pout, sizeof(double2) * (size_t)n * nrhs);
        }
    } else {
        int np = (n + 63) / 64 * 64;
        void *p64, *p32, *pb, *px;
        MIDAS_TRY(ensure(c, S_Z64, sizeof(double2) * (size_t)np * np, &p64));
        MIDAS_TRY(ensure(c, S_Z32, sizeof(float2) * (size_t)np * np, &p32));
        MIDAS_TRY(ensure(c, S_RHS64, sizeof(double2) * (size_t)np * nrhs, &pb));
        MIDAS_TRY(ensure(c, S_X64, sizeof(double2) * (size_t)np * nrhs, &px));
        Timer tf(c->stream);
        if (np > n) {
            // padding: zero the pad rows / columns, unit diagonal
            MIDAS_CUDA(c, cudaMemsetAsync(p64, 0, sizeof(double2) * (size_t)np * np, c->stream));
            MIDAS_CUDA(c, cudaMemsetAsync(p32, 0, sizeof(float2) * (size_t)np * np, c->stream));
            ++c->launches;
            k_pad_identity<<<1, 64, 0, c->stream>>>((double2 *)p64, (float2 *)p32, np, n, np);
            MIDAS_CUDA(c, cudaMemsetAsync(pb, 0, sizeof(double2) * (size_t)np * nrhs, c->stream));
        }
        MIDAS_TRY(launch_mom_fill(c, 0, n, 0, n, (double2 *)p64, (float2 *)p32, (size_t)np, 1));   // row-major
        MIDAS_TRY(launch_mom_rhs<double2>(c, ntr, (const double *)th, (const double *)ph, (double2 *)pb, 1, np));
        float tfill = tf.stop();
        if (info) info->t_fill_ms = tfill;
        st = mixed_solve(c, np, (float2 *)p32, (double2 *)p64, (const double2 *)pb, (double2 *)px, nrhs,
                                info);
        if (st == MIDAS_OK) {
            void *pout;
            MIDAS_TRY(ensure(c, S_OUT0, sizeof(double2) * (size_t)n * nrhs, &pout));
            long long t2 = (long long)n * nrhs;
            ++c->launches;
            k_copy_unpad<<<(unsigned)((t2 + 255) / 256), 256, 0, c->stream>>>((const double2 *)px, n, np, nrhs,
                                                                              (double2 *)pout);
            st = copy_out(c, E, pout, sizeof(double2) * (size_t)n * nrhs);
        }
    }
    if (info) {
        info->status = st;
        info->t_total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return st;
}

int midas_gpu_lattice_matvec(midas_gpu_ctx *c, int nrhs, const double *X, double *Y)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    MIDAS_TRY(need_cells(c));
    if (nrhs <= 0 || !X || !Y) return c->err.set(MIDAS_ERR_ARG, "lattice_matvec: bad arguments");
    cudaSetDevice(c->device);
    const size_t N = 3 * (size_t)c->n, bytes = sizeof(double2) * N * nrhs;
    const void *dx;
    MIDAS_TRY(to_device(c, X, bytes, S_IN3, &dx));
    double2 *out = (double2 *)Y;
    if (!is_device_ptr(Y)) {
        void *p;
        MIDAS_TRY(ensure(c, S_OUT0, bytes, &p));
        out = (double2 *)p;
    }
    MIDAS_TRY(lattice_matvec(c, nrhs, (const double2 *)dx, (long long)N, nullptr, 0, out, (long long)N, S_LFFT));
    MIDAS_TRY(copy_out(c, Y, out, bytes));
    return check_flag(c, "lattice_matvec");
}

static int gmres_solve(midas_gpu_ctx *c, midas_gpu_nn *net, int ntr, const double *theta, const double *phi,
                       const double *E0, int restart, int maxit, double tol, int flags, double *E, midas_gpu_info *info)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    auto t0 = std::chrono::steady_clock::now();
    MIDAS_TRY(need_cells(c));
    if (ntr <= 0 || !theta || !phi || !E || restart <= 0 || restart > 500 || maxit <= 0 || !(tol > 0))
        return c->err.set(MIDAS_ERR_ARG, "gmres_solve: bad arguments");
    if (!lattice_fft_fits(c)) return c->err.set(MIDAS_ERR_UNSUPPORTED, "gmres_solve: cells are not on a lattice");
    cudaSetDevice(c->device);
    if (info) memset(info, 0, sizeof(*info));
    const int n = 3 * c->n, nrhs = 2 * ntr;
    const size_t bytes = sizeof(double2) * (size_t)n * nrhs;
    const void *th, *ph;
    MIDAS_TRY(to_device(c, theta, sizeof(double) * ntr, S_IN0, &th));
    MIDAS_TRY(to_device(c, phi, sizeof(double) * ntr, S_IN1, &ph));
    void *pb, *px;
    MIDAS_TRY(ensure(c, S_RHS64, bytes, &pb));
    MIDAS_TRY(ensure(c, S_X64, bytes, &px));
    MIDAS_TRY(launch_mom_rhs<double2>(c, ntr, (const double *)th, (const double *)ph, (double2 *)pb, 1, n));
    if (E0) MIDAS_CUDA(c, cudaMemcpyAsync(px, E0, bytes, cudaMemcpyDefault, c->stream));
    else MIDAS_CUDA(c, cudaMemsetAsync(px, 0, bytes, c->stream));
    int iters = 0;
    double rel = 0;
    Timer ts(c->stream);
    int st = gmres_lattice(c, nrhs, (const double2 *)pb, (double2 *)px, restart, maxit, tol,
                           (flags & MIDAS_GMRES_JACOBI) != 0, &iters, &rel, net);
    const float tsol = ts.stop();
    const int cst = copy_out(c, E, px, bytes);
    if (st == MIDAS_OK) st = cst;
    if (info) {
        info->status = st;
        info->ir_iters = iters;
        info->backward_error = rel;
        info->t_solve_ms = tsol;
        info->t_total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return st;
}

int midas_gpu_gmres_solve(midas_gpu_ctx *c, int ntr, const double *theta, const double *phi, const double *E0,
                          int restart, int maxit, double tol, int flags, double *E, midas_gpu_info *info)
{
    return gmres_solve(c, nullptr, ntr, theta, phi, E0, restart, maxit, tol, flags, E, info);
}

int midas_gpu_fgmres_solve(midas_gpu_ctx *c, midas_gpu_nn *net, int ntr, const double *theta, const double *phi,
                           const double *E0, int restart, int maxit, double tol, double *E, midas_gpu_info *info)
{
    if (!c) return MIDAS_ERR_ARG;
    if (!net) return c->err.set(MIDAS_ERR_ARG, "fgmres_solve: no network");
    return gmres_solve(c, net, ntr, theta, phi, E0, restart, maxit, tol, 0, E, info);
}

int midas_gpu_cbfm_solve(midas_gpu_ctx *c, int nblocks, const int *blk_offsets, const int *ext_offsets,
                         const int *ext_idx, int ncbf, const double *cbf_theta, const double *cbf_phi, double thr_cbf,
                         double res_sr, int flags, double eps_aca, int aca_itmax, int ntr, const double *theta,
                         const double *phi, double *E, int *K, midas_gpu_info *info)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    MIDAS_TRY(need_cells(c));
    if (nblocks <= 0 || !blk_offsets || !ext_offsets || ncbf <= 0 || !cbf_theta || !cbf_phi || ntr <= 0 || !theta ||
        !phi || !E)
        return c->err.set(MIDAS_ERR_ARG, "cbfm_solve: bad arguments");
    cudaSetDevice(c->device);
    MIDAS_TRY(need_tables(c));
    return cbfm_run(c, nblocks, blk_offsets, ext_offsets, ext_idx, ncbf, cbf_theta, cbf_phi, thr_cbf, res_sr, flags,
                    eps_aca, aca_itmax, ntr, theta, phi, (double2 *)E, K, info);
}

int midas_gpu_cext_cabs(midas_gpu_ctx *c, int ntr, const double *theta, const double *phi, const double *E,
                        double *cext, double *cabs)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    MIDAS_TRY(need_cells(c));
    if (ntr <= 0 || !theta || !phi || !E || !cext || !cabs) return c->err.set(MIDAS_ERR_ARG, "cext_cabs");
    const void *th, *ph, *dE;
    MIDAS_TRY(to_device(c, theta, sizeof(double) * ntr, S_IN0, &th));
    MIDAS_TRY(to_device(c, phi, sizeof(double) * ntr, S_IN1, &ph));
    MIDAS_TRY(to_device(c, E, sizeof(double2) * 3 * (size_t)c->n * 2 * ntr, S_IN2, &dE));
    void *p;
    MIDAS_TRY(ensure(c, S_OUT0, sizeof(double) * 2 * ntr, &p));
    double *d = (double *)p;
    MIDAS_TRY(launch_cext_cabs(c, ntr, (const double *)th, (const double *)ph, (const double2 *)dE, d, d + ntr));
    MIDAS_TRY(copy_out(c, cext, d, sizeof(double) * ntr));
    return copy_out(c, cabs, d + ntr, sizeof(double) * ntr);
}

int midas_gpu_smatrix(midas_gpu_ctx *c, int nrx, const double *rx_theta, const double *rx_phi, int ntr,
                      const double *E, double *S)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    MIDAS_TRY(need_cells(c));
    if (nrx <= 0 || ntr <= 0 || !rx_theta || !rx_phi || !E || !S) return c->err.set(MIDAS_ERR_ARG, "smatrix");
    const void *th, *ph, *dE;
    MIDAS_TRY(to_device(c, rx_theta, sizeof(double) * nrx, S_IN0, &th));
    MIDAS_TRY(to_device(c, rx_phi, sizeof(double) * nrx, S_IN1, &ph));
    MIDAS_TRY(to_device(c, E, sizeof(double2) * 3 * (size_t)c->n * 2 * ntr, S_IN2, &dE));
    size_t bytes = sizeof(double2) * (size_t)nrx * 4 * ntr;
    double2 *out = (double2 *)S;
    if (!is_device_ptr(S)) {
        void *p;
        MIDAS_TRY(ensure(c, S_OUT0, bytes, &p));
        out = (double2 *)p;
    }
    MIDAS_TRY(launch_smatrix(c, nrx, (const double *)th, (const double *)ph, ntr, (const double2 *)dE, out));
    return copy_out(c, S, out, bytes);
}

int midas_gpu_scattering_quantities(midas_gpu_ctx *c, int quad_tr, int quad_rx, int ntr_theta, int ntr_phi,
                                    const double *tr_theta, const double *tr_phi, int nrx_theta, int nrx_phi,
                                    int nrx_tot, const double *rx_theta, const double *rx_phi, const double *S,
                                    const double *cext, const double *cabs, double dm, double k0, int cext_intfields,
                                    const double *w_tr, const double *w_rx, double *q_dir, double *q_avg)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    return scattering_quantities(c, quad_tr, quad_rx, ntr_theta, ntr_phi, tr_theta, tr_phi, nrx_theta, nrx_phi,
                                 nrx_tot, rx_theta, rx_phi, S, cext, cabs, dm, k0, cext_intfields, w_tr, w_rx,
                                 q_dir, q_avg);
}

// internal hooks used by the tests
int midas_gpu_gemm_selftest(midas_gpu_ctx *c)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    return gemm_selftest(c);
}

const char *midas_gpu_gemm_engine(void) { return gemm_engine(); }

int midas_gpu_wait_selftest(midas_gpu_ctx *c, int limit, int *expired)
{
    if (!c || !expired) return MIDAS_ERR_ARG;
    c->err = Err();
    return wait_selftest(c, limit, expired);
}

int midas_gpu_heev(midas_gpu_ctx *c, int m, const double *A, double *W, double *V)
{
    if (!c || m <= 0 || !A || !W || !V) return MIDAS_ERR_ARG;
    c->err = Err();
    void *p;
    MIDAS_TRY(ensure(c, S_OUT0, sizeof(double2) * 3 * (size_t)m * m + sizeof(double) * m + 512, &p));
    double2 *dA = (double2 *)p, *dV = dA + (size_t)m * m, *dH = dV + (size_t)m * m;
    double *dW = (double *)(dH + (size_t)m * m);
    MIDAS_CUDA(c, cudaMemcpyAsync(dA, A, sizeof(double2) * (size_t)m * m, cudaMemcpyDefault, c->stream));
    MIDAS_TRY(heev_dev(c, 1, m, dA, m, (long long)m * m, dH, dV, (long long)m * m, dW));
    MIDAS_CUDA(c, cudaMemcpyAsync(W, dW, sizeof(double) * m, cudaMemcpyDefault, c->stream));
    MIDAS_CUDA(c, cudaMemcpyAsync(V, dV, sizeof(double2) * (size_t)m * m, cudaMemcpyDefault, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    return check_flag(c, "heev");
}

int midas_gpu_zgemm_x3(midas_gpu_ctx *c, int M, int N, int K, const double *A, const double *B, double *D)
{
    if (!c || M <= 0 || N <= 0 || K <= 0 || !A || !B || !D) return MIDAS_ERR_ARG;
    c->err = Err();
    void *p;
    size_t na = (size_t)M * K, nb = (size_t)K * N, nd = (size_t)M * N;
    MIDAS_TRY(ensure(c, S_OUT0, sizeof(double2) * (na + nb) + sizeof(float2) * nd + 1024, &p));
    double2 *dA = (double2 *)p, *dB = dA + na;
    float2 *dD = (float2 *)(dB + nb);
    MIDAS_CUDA(c, cudaMemcpyAsync(dA, A, sizeof(double2) * na, cudaMemcpyDefault, c->stream));
    MIDAS_CUDA(c, cudaMemcpyAsync(dB, B, sizeof(double2) * nb, cudaMemcpyDefault, c->stream));
    MIDAS_TRY(zgemm_x3<double2, double2>(c, M, N, K, dA, K, 1, 0, dB, N, 1, (float *)dD, 2LL * N, 1.f, 0.f));
    std::vector<float2> h(nd);
    MIDAS_CUDA(c, cudaMemcpyAsync(h.data(), dD, sizeof(float2) * nd, cudaMemcpyDeviceToHost, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i < nd; ++i) { D[2 * i] = h[i].x; D[2 * i + 1] = h[i].y; }
    return check_flag(c, "zgemm_x3");
}

int midas_gpu_bench_gemm(midas_gpu_ctx *c, int M, int N, int K, int iters, double *ms)
{
    if (!c || !ms) return MIDAS_ERR_ARG;
    c->err = Err();
    return gemm_bench(c, M, N, K, iters, ms);
}

int midas_gpu_bench_gemm_ex(midas_gpu_ctx *c, int M, int N, int K, int iters, int f16, double *ms)
{
    if (!c || !ms) return MIDAS_ERR_ARG;
    c->err = Err();
    return gemm_bench(c, M, N, K, iters, ms, f16 != 0);
}

long long midas_gpu_launch_count(const midas_gpu_ctx *c) { return c ? c->launches : 0; }

int midas_gpu_profile(midas_gpu_ctx *c, int enable)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    cudaSetDevice(c->device);
    MIDAS_TRY(kp_flush(c));
    KProf &k = c->kprof;
    if (enable) {
        for (int i = 0; i < MIDAS_KC_COUNT; ++i) { k.ms[i] = k.flops[i] = k.bytes[i] = 0; k.n[i] = 0; }
    }
    k.on = enable != 0;
    return MIDAS_OK;
}

int midas_gpu_profile_query(midas_gpu_ctx *c, int kclass, double *ms, double *flops, double *bytes,
                            long long *launches)
{
    if (!c || kclass < 0 || kclass >= MIDAS_KC_COUNT) return MIDAS_ERR_ARG;
    c->err = Err();
    cudaSetDevice(c->device);
    MIDAS_TRY(kp_flush(c));
    const KProf &k = c->kprof;
    if (ms) *ms = k.ms[kclass];
    if (flops) *flops = k.flops[kclass];
    if (bytes) *bytes = k.bytes[kclass];
    if (launches) *launches = k.n[kclass];
    return MIDAS_OK;
}

void *midas_gpu_stream(const midas_gpu_ctx *c) { return c ? (void *)c->stream : nullptr; }

int midas_gpu_wait_event(midas_gpu_ctx *c, void *event)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    if (!event) return c->err.set(MIDAS_ERR_ARG, "wait_event: null event");
    MIDAS_CUDA(c, cudaStreamWaitEvent(c->stream, (cudaEvent_t)event, 0));
    return MIDAS_OK;
}

int midas_gpu_record_event(midas_gpu_ctx *c, void *event)
{
    if (!c) return MIDAS_ERR_ARG;
    c->err = Err();
    if (!event) return c->err.set(MIDAS_ERR_ARG, "record_event: null event");
    MIDAS_CUDA(c, cudaEventRecord((cudaEvent_t)event, c->stream));
    return MIDAS_OK;
}

}  // extern "C"
