// noalloc.cu -- dense complex solve that allocates no device memory.
//
// Some callers cannot call cudaMalloc: plug-ins that run inside a host
// application which owns and caps all device memory (the host hands out
// buffers, and an allocation behind its back can fail or break its
// accounting), and real-time paths where an allocation could block on the
// driver.  For them midas_gpu_dense_solve_noalloc() solves A X = B with the
// same mixed-precision LU + FP64 refinement as midas_gpu_dense_solve(), taking
// every byte of device scratch from one file-scope static __device__ array of
// NOALLOC_BYTES.  That array is part of the loaded library: every GPU that
// loads it holds the 24 MiB until the process exits, and all calls share it.
// The context it builds on the host stack has `no_alloc` set, so a scratch
// request larger than its carved slot fails with MIDAS_ERR_ALLOC instead of
// reaching cudaMalloc.
//
// The call is synchronous: it waits on the caller's stream and reads the
// refinement's convergence test on the host, as midas_gpu_dense_solve() does.
// A call on a stream that is being captured returns MIDAS_ERR_ARG before it
// issues any work, so the caller's capture is left intact.
//
// Limits: n <= NOALLOC_NMAX (512) unknowns and nrhs <= NOALLOC_RMAX (32)
// right-hand sides; larger requests return MIDAS_ERR_ARG before any device work.
// The array keeps the previous call's contents, so every region that must
// start at zero is cleared on each call.  Calls that overlap on the GPU (two
// host threads, or two streams) race on the shared array and must be
// serialised by the caller.  The first call on a device looks up the array's
// device address with cudaGetSymbolAddress (with that device current) and
// caches it; a cached address that no longer names device memory (after a
// cudaDeviceReset) is looked up again.
#include <cstring>

#include "common.cuh"
#include "kernels.cuh"

namespace midas {

constexpr int NOALLOC_NMAX = 512;
constexpr int NOALLOC_RMAX = 32;
constexpr size_t NOALLOC_BYTES = (size_t)24 << 20;   // n = 512, nrhs = 32 needs 19.2 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

// Device address of the scratch array, per device.  In host code the array's name
// is only a host-side stand-in: kernels must be given this address instead.
// Atomic entries, because two host threads may make their first call at once
// (both then look up the same address).
static std::atomic<void *> g_noalloc_addr[64];

static int noalloc_scratch_address(int device, void **out)
{
    void *p = g_noalloc_addr[device].load(std::memory_order_acquire);
    if (p && is_device_ptr(p)) { *out = p; return MIDAS_OK; }
    p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) { cudaGetLastError(); return MIDAS_ERR_CUDA; }
    g_noalloc_addr[device].store(p, std::memory_order_release);
    *out = p;
    return MIDAS_OK;
}

__global__ void k_na_transpose(const double2 *A, int n, double2 *Z64, float2 *Z32, long long ld)
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

__global__ void k_na_pad(double2 *Z64, float2 *Z32, long long ld, int n0, int np)
{
    int i = n0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    Z64[(long long)i * ld + i] = make_double2(1, 0);
    Z32[(long long)i * ld + i] = make_float2(1, 0);
}

__global__ void k_na_copy(const double2 *src, long long lds, double2 *dst, long long ldd, int rows, int rows_out,
                          int nrhs)
{
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)rows_out * nrhs) return;
    int r = (int)(i % rows_out), k = (int)(i / rows_out);
    dst[(long long)k * ldd + r] = r < rows ? src[(long long)k * lds + r] : make_double2(0, 0);
}

// carve a region of the scratch array for a pool slot (the slot reports exactly
// its capacity, so the shared ensure() never needs to grow it)
struct Carver {
    char *base;
    size_t top, cap;
    bool ok = true;
    void *take(size_t bytes)
    {
        top = (top + 255) & ~(size_t)255;
        if (top + bytes > cap) { ok = false; return nullptr; }
        void *p = base + top;
        top += bytes;
        return p;
    }
};

}  // namespace midas

using namespace midas;

extern "C" int midas_gpu_dense_solve_noalloc(int device, void *stream, int n, int nrhs, const double *A, double *B,
                                             double *backward_error)
{
    if (n <= 0 || nrhs <= 0 || !A || !B) return MIDAS_ERR_ARG;
    if (n > NOALLOC_NMAX || nrhs > NOALLOC_RMAX) return MIDAS_ERR_ARG;   // beyond the static scratch
    if (device < 0 || device >= 64) return MIDAS_ERR_ARG;
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) { cudaGetLastError(); return MIDAS_ERR_CUDA; }
    if (cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); return MIDAS_ERR_CUDA; }
    struct Restore {
        int d;
        ~Restore() { if (d >= 0) cudaSetDevice(d); }
    } restore{prev};
    {
        // refuse a capturing stream before issuing anything on it: the solve waits on
        // the stream and reads convergence on the host, neither of which a capture allows
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing((cudaStream_t)stream, &cs) != cudaSuccess) { cudaGetLastError(); return MIDAS_ERR_ARG; }
        if (cs != cudaStreamCaptureStatusNone) return MIDAS_ERR_ARG;
    }
    void *scratch = nullptr;
    if (noalloc_scratch_address(device, &scratch) != MIDAS_OK) return MIDAS_ERR_CUDA;
    // a context that lives on the host stack; its scratch slots point into the array
    midas_gpu_ctx c;
    midas_gpu_default_opts(&c.opts);
    c.opts.device = device;
    c.device = device;
    c.stream = (cudaStream_t)stream;
    c.allow_side = false;   // no stream or event creation on this path
    c.no_alloc = true;      // a slot request beyond its carve is an error, not a cudaMalloc
    c.pi = ref_pi_host();
    c.pool.resize(S_NSLOTS);
    const int np = (n + 63) / 64 * 64;
    Carver cv{(char *)scratch, 0, NOALLOC_BYTES};
    c.d_flag = (int *)cv.take(256);
    auto slot = [&](int s, size_t bytes) {
        c.pool[s].p = cv.take(bytes);
        c.pool[s].bytes = bytes;
    };
    const size_t nn = (size_t)np * nrhs;
    slot(S_Z64, sizeof(double2) * (size_t)np * np);
    slot(S_Z32, sizeof(float2) * (size_t)np * np);
    slot(S_LINV, lu_inv_bytes(np));
    slot(S_BEXP, sizeof(float) * (size_t)128 * 128);   // expanded 64 x 64 U^-1
    slot(S_BEXP2, lu_bexp2_bytes(np));
    slot(S_RHS64, sizeof(double2) * nn);
    slot(S_X64, sizeof(double2) * nn);
    slot(S_R64, sizeof(double2) * nn);
    slot(S_T32B, sizeof(float2) * nn);
    slot(S_T32, sizeof(float2) * nn);
    slot(S_RED, sizeof(unsigned long long) * 4 * (size_t)nrhs + 64);
    slot(S_SOLVE, lu_solve_scratch_bytes(np, nrhs));
    slot(S_RPART, resid_scratch_bytes(np, nrhs));
    slot(S_H16, lu_h16_scratch_bytes(np));
    slot(S_IN3, sizeof(double2) * (size_t)n * n);      // staging of A when it is host memory
    slot(S_IN2, sizeof(double2) * (size_t)n * nrhs);   // staging of B / output
    if (!cv.ok) return MIDAS_ERR_ARG;
    int st = MIDAS_OK;
    do {
        cudaStream_t s = c.stream;
        if (cudaMemsetAsync(c.d_flag, 0, sizeof(int), s) != cudaSuccess) { st = MIDAS_ERR_CUDA; break; }
        const double2 *dA = (const double2 *)A;
        if (!is_device_ptr(A)) {
            if (cudaMemcpyAsync(c.pool[S_IN3].p, A, sizeof(double2) * (size_t)n * n, cudaMemcpyHostToDevice, s) !=
                cudaSuccess) { st = MIDAS_ERR_CUDA; break; }
            dA = (const double2 *)c.pool[S_IN3].p;
        }
        const bool Bdev = is_device_ptr(B);
        double2 *dB = (double2 *)B;
        if (!Bdev) {
            if (cudaMemcpyAsync(c.pool[S_IN2].p, B, sizeof(double2) * (size_t)n * nrhs, cudaMemcpyHostToDevice, s) !=
                cudaSuccess) { st = MIDAS_ERR_CUDA; break; }
            dB = (double2 *)c.pool[S_IN2].p;
        }
        double2 *Z64 = (double2 *)c.pool[S_Z64].p, *b = (double2 *)c.pool[S_RHS64].p, *x = (double2 *)c.pool[S_X64].p;
        float2 *Z32 = (float2 *)c.pool[S_Z32].p;
        // the previous call's matrices are still in the array: clear before filling
        if (cudaMemsetAsync(Z64, 0, sizeof(double2) * (size_t)np * np, s) != cudaSuccess ||
            cudaMemsetAsync(Z32, 0, sizeof(float2) * (size_t)np * np, s) != cudaSuccess) { st = MIDAS_ERR_CUDA; break; }
        dim3 blk(32, 8), grd((n + 31) / 32, (n + 31) / 32);
        k_na_transpose<<<grd, blk, 0, s>>>(dA, n, Z64, Z32, np);
        if (np > n) k_na_pad<<<1, 64, 0, s>>>(Z64, Z32, np, n, np);
        long long tot = (long long)np * nrhs;
        k_na_copy<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(dB, n, b, np, n, np, nrhs);
        if (cudaGetLastError() != cudaSuccess) { st = MIDAS_ERR_CUDA; break; }
        DenseLU lu;
        lu.n = np;
        lu.A = Z32;
        lu.lda = np;
        st = lu_factor_nopiv(&c, lu);
        if (st == MIDAS_OK) st = check_flag(&c, "noalloc lu");
        midas_gpu_info info;
        memset(&info, 0, sizeof(info));
        if (st == MIDAS_OK) st = ir_solve(&c, lu, Z64, np, b, x, nrhs, &info);
        if (st != MIDAS_OK) break;
        long long t2 = (long long)n * nrhs;
        k_na_copy<<<(unsigned)((t2 + 255) / 256), 256, 0, s>>>(x, np, dB, n, np, n, nrhs);
        if (!Bdev && cudaMemcpyAsync(B, dB, sizeof(double2) * (size_t)n * nrhs, cudaMemcpyDeviceToHost, s) !=
                         cudaSuccess) { st = MIDAS_ERR_CUDA; break; }
        if (cudaStreamSynchronize(s) != cudaSuccess) { st = MIDAS_ERR_CUDA; break; }
        if (backward_error) *backward_error = info.backward_error;
    } while (0);
    // every slot points into the static array: nothing to free
    for (auto &d : c.pool) { d.p = nullptr; d.bytes = 0; }
    return st;
}
