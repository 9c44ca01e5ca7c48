// common.cuh -- shared definitions of the GB300 MIDAS library (internal).
#pragma once
#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/midas_gpu.h"

namespace midas {

// ---------------------------------------------------------------------------
// status plumbing: every internal call returns a midas_status; the first
// failure message is kept on the context.
// ---------------------------------------------------------------------------
struct Err {
    int code = MIDAS_OK;
    std::string msg;
    int set(int c, const std::string &m) {
        if (code == MIDAS_OK) { code = c; msg = m; }
        return c;
    }
};

#define MIDAS_CUDA(ctx, expr)                                                                      \
    do {                                                                                           \
        cudaError_t _e = (expr);                                                                   \
        if (_e != cudaSuccess)                                                                     \
            return (ctx)->err.set(_e == cudaErrorMemoryAllocation ? MIDAS_ERR_ALLOC : MIDAS_ERR_CUDA, \
                                  std::string(#expr) + ": " + cudaGetErrorString(_e));             \
    } while (0)

#define MIDAS_TRY(...)                   \
    do {                                 \
        int _s = (__VA_ARGS__);          \
        if (_s != MIDAS_OK) return _s;   \
    } while (0)

// Device error flags (written by kernels that hit a bounded wait or a bad pivot).
enum DevErr : int { DEV_OK = 0, DEV_TIMEOUT = 1, DEV_ZERO_PIVOT = 2, DEV_BAD_ARG = 4 };

// FP32 -> TF32 with round-to-nearest (ties away): the tensor cores read only the
// top 19 bits of an FP32 operand (truncation, a one-sided error), so values that
// feed them repeatedly are stored pre-rounded to keep the errors unbiased.
__device__ __forceinline__ float tf32_rna(float x)
{
    uint32_t u;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(x));
    return __uint_as_float(u);
}

// Error-free transformations in FP32 for double-float (hi + lo) accumulation:
// Knuth's TwoSum and the FMA TwoProduct.  The _rn intrinsics are never
// contracted, so a product cannot be fused into the following sum (which would
// make s differ from hi + p and break the exactness the pair relies on).
__device__ __forceinline__ void ef_two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (hi, lo) += a * b exactly up to the FP32 rounding of lo (TwoProduct + TwoSum).
__device__ __forceinline__ void df_fma(float &hi, float &lo, float a, float b)
{
    const float p = __fmul_rn(a, b);
    const float pe = fmaf(a, b, -p);
    float s, e;
    ef_two_sum(hi, p, s, e);
    hi = s;
    lo += e + pe;
}

// (hi, lo) += (ah + al)(bh + bl): ah*bh exactly, the cross terms in FP32 (they
// are 2^-24 of the product), al*bl dropped (2^-48).
__device__ __forceinline__ void df_fma(float &hi, float &lo, float ah, float bh, float al, float bl)
{
    const float p = __fmul_rn(ah, bh);
    float pe = fmaf(ah, bh, -p);
    pe = fmaf(ah, bl, pe);
    pe = fmaf(al, bh, pe);
    float s, e;
    ef_two_sum(hi, p, s, e);
    hi = s;
    lo += e + pe;
}

// Reference Pi = Acos(-1.) evaluated in single precision (src/Initialization.f90:39).
inline double ref_pi_host() { return (double)acosf(-1.0f); }

// ---------------------------------------------------------------------------
// device buffers
// ---------------------------------------------------------------------------
struct DBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

// ---------------------------------------------------------------------------
// per-kernel-class device timing (roofline reports): CUDA events recorded on
// the context stream around each instrumented launch while profiling is on
// ---------------------------------------------------------------------------
struct KProf {
    bool on = false;
    std::vector<cudaEvent_t> ev;   // event pool, grown on demand
    size_t used = 0;
    struct Rec { int cls, e0; double flops, bytes; };
    std::vector<Rec> rec;
    double ms[MIDAS_KC_COUNT] = {}, flops[MIDAS_KC_COUNT] = {}, bytes[MIDAS_KC_COUNT] = {};
    long long n[MIDAS_KC_COUNT] = {};
};

// FFT form of the MoM operator on a voxel lattice (fft.cu): grid sizes and the
// dyad spectra of the current cells
struct LatticeFft {
    int L[3] = {0, 0, 0}, n[3] = {0, 0, 0};
    long long npts = 0;
    double2 *G6 = nullptr;   // 6 spectra of the FP64 dyads, npts each
    double2 *G6c4 = nullptr; // 6 spectra of the complex(4)-rounded dyads
    int *lo = nullptr;       // lattice lower corner (device copy)
    long long version = -1;  // cells version the spectra belong to
};

}  // namespace midas

// The context (opaque in the C ABI).
struct midas_gpu_ctx {
    midas_gpu_opts opts;
    int device = 0;
    cudaStream_t stream = nullptr;
    midas::Err err;
    double pi = 0;
    // cells
    int n = 0;
    double k0 = 0;
    double *x = nullptr, *y = nullptr, *z = nullptr, *sc = nullptr, *an = nullptr, *kappa = nullptr;
    double2 *eps = nullptr, *che = nullptr, *znnpp = nullptr;
    float2 *fk4 = nullptr;   // f_kapChe rounded to complex(4), per cell
    double2 *fk8 = nullptr;  // f_kapChe in complex(8), per cell
    // uniform-lattice description of the cells (fast fills)
    int lattice = 0;         // 1 when all cells sit on one grid of pitch d
    double lat_d = 0, lat_o[3] = {0, 0, 0};
    int lat_lo[3] = {0, 0, 0}, lat_hi[3] = {0, 0, 0};
    int *lat_ijk = nullptr;  // 3 ints per cell
    float2 *lat_tab4 = nullptr;    // complex(4) dyad table per lattice offset (6 comps)
    double2 *lat_tab8 = nullptr;   // FP64 dyad table per lattice offset (6 comps)
    int lat_dim[3] = {0, 0, 0};
    long long cells_version = 0;   // incremented by every midas_gpu_set_cells
    midas::LatticeFft lfft;
    // scratch pool (grow-only, reused across calls)
    std::vector<midas::DBuf> pool;
    int *d_flag = nullptr;   // device error flag
    long long launches = 0;  // kernels launched on this context
    midas::KProf kprof;
    // lanes: child contexts (own stream and scratch pool, the cells aliased)
    // that run independent CBFM blocks concurrently
    std::vector<midas_gpu_ctx *> lanes;
    std::vector<midas_gpu_ctx *> aux;   // the CBFM pipeline's finisher and eigen-solve contexts
    // side stream (created on first use, same priority as `stream`) for work that
    // only joins later, e.g. the solve's diagonal-block inverses during the LU
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    bool allow_side = true;   // false for the allocation-free entry point
    // true for the allocation-free entry point: its slots are carved from a static
    // array, and a request beyond a slot's capacity is an error, never a cudaMalloc
    bool no_alloc = false;
    void *cusolver = nullptr;
    void *cublas = nullptr;
};

namespace midas {

// One-time per-device setup (kernel attributes) that several host threads -- the
// CBFM lanes -- may reach at once: f runs until it succeeds once on a device; a
// race only repeats the idempotent call.
struct PerDeviceOnce {
    std::atomic<unsigned long long> mask{0};
    template <typename F>
    cudaError_t run(int device, F f)
    {
        const unsigned long long bit = 1ull << (device & 63);
        if (mask.load(std::memory_order_acquire) & bit) return cudaSuccess;
        const cudaError_t e = f();
        if (e == cudaSuccess) mask.fetch_or(bit, std::memory_order_acq_rel);
        return e;
    }
};

// Number of SMs of a device (cached per device, thread-safe).
int device_sms(midas_gpu_ctx *ctx);

// Scratch allocation helpers (pool slot i grows as needed).
int ensure(midas_gpu_ctx *ctx, int slot, size_t bytes, void **out);

// Kernel-class timing: kp_begin records a start event (returns -1 when profiling
// is off), kp_end the stop event with the launch's algorithmic flops and bytes;
// kp_flush waits for the recorded events and accumulates them per class.
int kp_begin(midas_gpu_ctx *ctx);
void kp_end(midas_gpu_ctx *ctx, int e0, int cls, double flops, double bytes);
int kp_flush(midas_gpu_ctx *ctx);

// The context's side stream and fork/join events (created on first use).
int side_stream(midas_gpu_ctx *ctx, cudaStream_t *out);
void destroy_side(midas_gpu_ctx *ctx);

// Is p a device (or managed) pointer?
bool is_device_ptr(const void *p);

// Copy-in helper: returns a device pointer holding `bytes` of p (p itself when it
// already lives on the device); uses pool slot `slot`.
int to_device(midas_gpu_ctx *ctx, const void *p, size_t bytes, int slot, const void **out);

// Device error flag check after a kernel sequence.
int check_flag(midas_gpu_ctx *ctx, const char *where);

// Lattice FFT operator (fft.cu): Y = Z X, or Y = B - Z X when B is given.
int lattice_fft_prepare(midas_gpu_ctx *c, bool c4 = false);
bool lattice_fft_fits(const midas_gpu_ctx *c);   // cells on a lattice of <= 256 cells per axis
bool lattice_fft_preferred(const midas_gpu_ctx *c, long long np);   // FFT residuals cheaper than dense ones
void lattice_fft_release(midas_gpu_ctx *c);
int lattice_matvec(midas_gpu_ctx *c, int nrhs, const double2 *X, long long ldx, const double2 *B, long long ldb,
                   double2 *Y, long long ldy, int slot, bool c4 = false);

// Restarted GMRES on the lattice operator (krylov.cu); X holds the initial guess.
// With net, flexible GMRES right-preconditioned by the network (nn.cu).
int gmres_lattice(midas_gpu_ctx *c, int ncol, const double2 *B, double2 *X, int restart, int maxit, double tol,
                  bool jacobi, int *iters, double *relres, midas_gpu_nn *net = nullptr);
// Zout = P(V): the network preconditioner on unit-norm cell vectors (nn.cu)
int nn_prec_apply(midas_gpu_ctx *c, midas_gpu_nn *net, int ncol, const double2 *V, long long ldv, double2 *Zout,
                  long long ldz);

// Scene preparation on the device (prep.cu); outputs in device memory.
int voxelise_sphere(midas_gpu_ctx *c, double dm, double sc, long long cap, double *x, double *y, double *z,
                    long long *ncell);
int voxelise_spheres(midas_gpu_ctx *c, int nsph, const double *centres, double a, int cells_per_diameter,
                     long long cap, double *x, double *y, double *z, long long *ncell, double *edge);
int box_partition(midas_gpu_ctx *c, int n, const double *x, const double *y, const double *z, int nx, int ny, int nz,
                  int *perm, int *blk_offsets, int *nblocks);
int extend_blocks(midas_gpu_ctx *c, int n, const double *x, const double *y, const double *z, int nb,
                  const int *offs_host, double ext_length, double sc, int *ext_offsets, long long cap, int *ext_idx,
                  long long *ntotal);

// Pool slots (fixed roles).  A pointer taken from a slot stays valid only until the
// next ensure() on the same slot, so a caller never holds a slot that a callee grows.
enum Slot : int {
    S_IN0 = 0, S_IN1, S_IN2, S_IN3, S_IN4, S_IN5, S_OUT0, S_OUT1,
    S_Z32, S_Z64, S_LINV, S_UINV, S_BEXP, S_BEXP2, S_RHS64, S_X64, S_R64, S_T32, S_T32B, S_RED,
    S_CBF0, S_CBF1, S_CBF2, S_CBF3, S_CBF4, S_CBF5, S_CBF6, S_CBF7, S_CBF8, S_CBF9, S_RED2, S_EINC,
    S_ACA, S_SOLVE, S_CSR, S_RPART, S_H16, S_HEEV, S_ZDF, S_QWS, S_SPH, S_LFFT, S_KRYLOV, S_PREP, S_CREF, S_NN, S_NSLOTS
};

}  // namespace midas
