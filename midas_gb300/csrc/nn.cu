// nn.cu -- the learned initial guess of the Krylov solve (sm_103a): a small 3-D
// convolutional network trained and evaluated by this library's own kernels.
//
// The network maps, on a G^3 voxel grid, the per-voxel contrast chi = eps - 1
// (real, imaginary), the incident field (three complex components), their
// products chi E_inc and the scatterer mask -- 16 input channels -- to the
// scattered part of the internal field, 6 output channels; the prediction is
// E = E_inc + mask * net(...).  Four 3 x 3 x 3 convolutions with zero padding,
// 16 -> 32 -> 32 -> 32 -> 6 channels (the last padded to 8), ReLU between them.
// The products chi E_inc are inputs because a ReLU stack represents a product
// of two inputs only coarsely, and the internal field is, to first order, that
// product rescaled.  The reference has no learned component; the dense LU /
// CBFM solve stays the fallback and the judge of its error, and the Krylov
// solve it starts checks its residual in FP64.
//
// Arithmetic: every convolution is an fp16 im2col (channel-last activations,
// the 27 neighbour offsets x input channels contiguous) multiplied on the
// tensor cores by the fp16 weights (tcgen05.mma kind::f16, FP32 accumulation in
// tensor memory) through the library's persistent GEMM.  Backward:
//   dX = im2col(dZ) * W'^T   with W'[ci][o][co] = W[co][-o][ci] (the transposed
//                            convolution is a convolution with flipped taps),
//   dW = dZ^T * im2col(X)    (K = the voxels of the batch; operands transposed
//                            so K is contiguous),
//   db = column sums of dZ.
// Gradients are scaled per layer into the fp16 range before they become GEMM
// operands (scale 2^(10 - ceil(log2 max|dZ|)), kept on the device); the GEMM
// reads the inverse scale as its alpha from device memory.  Master weights and
// Adam moments are FP32.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace midas {

constexpr int NN_LAYERS = 4;
constexpr int NN_CIN0 = 16;   // input channels
constexpr int NN_COUT = 6;    // output channels (complex field)
static const int NN_CI[NN_LAYERS] = {16, 32, 32, 32};
static const int NN_CO[NN_LAYERS] = {32, 32, 32, 8};   // last layer: 6 real + 2 zero rows

}  // namespace midas

struct midas_gpu_nn {
    int device = 0, grid = 0;
    float *W[midas::NN_LAYERS] = {}, *b[midas::NN_LAYERS] = {};            // FP32 master parameters
    float *gW[midas::NN_LAYERS] = {}, *gb[midas::NN_LAYERS] = {};          // gradients
    float *mW[midas::NN_LAYERS] = {}, *vW[midas::NN_LAYERS] = {};          // Adam moments
    float *mb[midas::NN_LAYERS] = {}, *vb[midas::NN_LAYERS] = {};
    __half *W16[midas::NN_LAYERS] = {}, *Wf16[midas::NN_LAYERS] = {};      // fp16 copies: W and flipped W'
    long long step = 0;
};

namespace midas {

static int nn_wcount(int l) { return NN_CO[l] * 27 * NN_CI[l]; }

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
// A[r][o * C + c] = X[neighbour(r, o)][c] (0 outside the grid); 8 fp16 per thread
__global__ void k_nn_im2col(const __half *X, int B, int G, int C, __half *A)
{
    const int C8 = C / 8;
    const long long V = (long long)G * G * G;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long tot = B * V * 27 * C8;
    if (t >= tot) return;
    const int c8 = (int)(t % C8);
    const int o = (int)((t / C8) % 27);
    const long long r = t / (27LL * C8);
    const long long v = r % V, bb = r / V;
    const int x = (int)(v % G), y = (int)((v / G) % G), z = (int)(v / ((long long)G * G));
    const int xn = x + o % 3 - 1, yn = y + (o / 3) % 3 - 1, zn = z + o / 9 - 1;
    uint4 val = make_uint4(0, 0, 0, 0);
    if (xn >= 0 && xn < G && yn >= 0 && yn < G && zn >= 0 && zn < G) {
        const long long rn = bb * V + ((long long)zn * G + yn) * G + xn;
        val = *(const uint4 *)(X + rn * C + c8 * 8);
    }
    *(uint4 *)(A + r * (27LL * C) + o * C + c8 * 8) = val;
}

// AT[o * C + c][r] = X[neighbour(r, o)][c]  (the transposed im2col of dW = dZ^T im2col(X))
__global__ void k_nn_im2col_t(const __half *X, int B, int G, int C, __half *AT)
{
    const long long V = (long long)G * G * G, M = B * V;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= M * 27 * C) return;
    const long long r = t % M;
    const int oc = (int)(t / M), o = oc / C, c = oc % C;
    const long long v = r % V, bb = r / V;
    const int x = (int)(v % G), y = (int)((v / G) % G), z = (int)(v / ((long long)G * G));
    const int xn = x + o % 3 - 1, yn = y + (o / 3) % 3 - 1, zn = z + o / 9 - 1;
    __half val = __float2half(0.f);
    if (xn >= 0 && xn < G && yn >= 0 && yn < G && zn >= 0 && zn < G)
        val = X[(bb * V + ((long long)zn * G + yn) * G + xn) * C + c];
    AT[(long long)oc * M + r] = val;
}

// Z = D + b (in place); X16 = fp16(relu(Z))
__global__ void k_nn_bias_relu(long long M, int C, float *D, const float *b, __half *X16)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= M * C) return;
    const float z = D[t] + b[t % C];
    D[t] = z;
    X16[t] = __float2half(fmaxf(z, 0.f));
}

__global__ void k_nn_f32_to_f16(long long n, const float *x, __half *y)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < n) y[t] = __float2half(x[t]);
}

// the prediction E = E_inc + mask * (D + b)[:, :6]
__global__ void k_nn_predict(long long M, const float *D, const float *b, const float *in, const float *mask,
                             float *E)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= M * NN_COUT) return;
    const long long r = t / NN_COUT;
    const int c = (int)(t % NN_COUT);
    E[t] = in[r * NN_CIN0 + 2 + c] + mask[r] * (D[r * 8 + c] + b[c]);
}

// per-sample relative squared error and dL/d(out) (layer-3 pre-activation, 8 columns)
//   L = (1/B) sum_b sum_{v, c} mask (E_pred - E)^2 / sum_{v, c} mask E^2
__global__ void k_nn_loss(long long M, long long V, int B, const float *D, const float *b, const float *in,
                          const float *mask, const float *tgt, const double *den, float *dOut, double *loss)
{
    __shared__ double red[256];
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double l = 0;
    if (r < M) {
        const long long bb = r / V;
        const double w = 1.0 / (den[bb] * B);
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            float g = 0.f;
            if (c < NN_COUT && mask[r] != 0.f) {
                const float e = in[r * NN_CIN0 + 2 + c] + (D[r * 8 + c] + b[c]);
                const float d = e - tgt[r * NN_COUT + c];
                l += (double)d * d * w;
                g = (float)(2.0 * d * w);
            }
            dOut[r * 8 + c] = g;
        }
    }
    red[threadIdx.x] = l;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0]);
}

// dZ = dX (from the next layer) * relu'(Z), in place on dX
__global__ void k_nn_relu_bwd(long long n, const float *Z, float *dX)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < n && !(Z[t] > 0.f)) dX[t] = 0.f;
}

__global__ void k_nn_absmax(long long n, const float *x, unsigned *amax)
{
    float m = 0.f;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(x[t]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(amax, __float_as_uint(m));
}

// scale s = 2^(10 - ceil(log2 max|dZ|)) (1 when dZ == 0); inv = 1 / s for the GEMM alpha
__global__ void k_nn_scale(const unsigned *amax, float *s, float *inv)
{
    const float m = __uint_as_float(*amax);
    int e = 0;
    if (m > 0.f) e = 10 - (int)ceilf(log2f(m));
    e = max(-100, min(100, e));
    *s = ldexpf(1.f, e);
    *inv = ldexpf(1.f, -e);
}

// out16[r][c] = fp16(dZ s), outT16[c][r] the same transposed
__global__ void k_nn_dz16(long long M, int C, const float *dZ, const float *s, __half *out16, __half *outT16)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= M * C) return;
    const long long r = t / C;
    const int c = (int)(t % C);
    const __half h = __float2half(dZ[t] * *s);
    out16[t] = h;
    outT16[(long long)c * M + r] = h;
}

// db[c] = sum_r dZ[r][c]: partials per block of rows, then a fixed-order sum
constexpr int NN_ROWS = 4096;
__global__ void k_nn_colsum_part(long long M, int C, const float *dZ, float *part)
{
    const int c = threadIdx.x % C, lane_rows = blockDim.x / C;
    const long long r0 = (long long)blockIdx.x * NN_ROWS;
    float s = 0.f;
    if (threadIdx.x < lane_rows * C)
        for (long long r = r0 + threadIdx.x / C; r < min(M, r0 + NN_ROWS); r += lane_rows) s += dZ[r * C + c];
    __shared__ float red[256];
    red[threadIdx.x] = threadIdx.x < lane_rows * C ? s : 0.f;
    __syncthreads();
    if (threadIdx.x < C) {
        float t = 0.f;
        for (int q = 0; q < lane_rows; ++q) t += red[q * C + threadIdx.x];
        part[(long long)blockIdx.x * C + threadIdx.x] = t;
    }
}
__global__ void k_nn_colsum_fin(int nblk, int C, const float *part, float *db)
{
    const int c = threadIdx.x;
    if (c >= C) return;
    float s = 0.f;
    for (int q = 0; q < nblk; ++q) s += part[(long long)q * C + c];
    db[c] = s;
}

// fp16 copies of W[co][o][ci] and of the flipped W'[ci][o][co] = W[co][26 - o][ci]
__global__ void k_nn_wcopy(int co_n, int ci_n, const float *W, __half *W16, __half *Wf16)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= co_n * 27 * ci_n) return;
    const int ci = t % ci_n, o = (t / ci_n) % 27, co = t / (27 * ci_n);
    const __half h = __float2half(W[t]);
    W16[t] = h;
    Wf16[((long long)ci * 27 + (26 - o)) * co_n + co] = h;
}

__global__ void k_nn_adam(int n, float *p, const float *g, float *m, float *v, float lr, float b1, float b2, float c1,
                          float c2, float eps, int rows_live, int row_len)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    if (t / row_len >= rows_live) return;   // padded output rows stay zero
    const float gg = g[t];
    const float mm = b1 * m[t] + (1.f - b1) * gg, vv = b2 * v[t] + (1.f - b2) * gg * gg;
    m[t] = mm;
    v[t] = vv;
    p[t] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct NnWork {
    __half *X16[NN_LAYERS];   // layer inputs (fp16, [M][C])
    float *Z[NN_LAYERS];      // pre-activations (fp32, [M][Cout])
    __half *A;                // im2col (shared by the layers)
    __half *AT;               // transposed im2col
    float *dX;                // dL/d(layer input), fp32 [M][32]
    float *dZ;                // dL/d(pre-activation) of the current layer
    __half *dZ16, *dZT16;
    float *sc;                // s, 1/s
    unsigned *amax;
    float *part;
    double *den, *loss;
    float *in32, *mask32, *tgt32;
};

static size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

static int nn_workspace(midas_gpu_ctx *c, long long M, NnWork &w)
{
    const size_t x16 = al256(sizeof(__half) * M * 32), z32 = al256(sizeof(float) * M * 32);
    const size_t a = al256(sizeof(__half) * M * 27 * 32);
    const size_t part = al256(sizeof(float) * (M / NN_ROWS + 2) * 32);
    const size_t tot = NN_LAYERS * (x16 + z32) + 2 * a + 2 * z32 + 2 * x16 + 3 * 256 + part + al256(sizeof(double) * 64) +
                       al256(sizeof(float) * M * NN_CIN0) + al256(sizeof(float) * M) + al256(sizeof(float) * M * 6) + 1024;
    void *p;
    MIDAS_TRY(ensure(c, S_NN, tot, &p));
    char *q = (char *)p;
    auto take = [&](size_t b) { char *r = q; q += al256(b); return (void *)r; };
    for (int l = 0; l < NN_LAYERS; ++l) {
        w.X16[l] = (__half *)take(x16);
        w.Z[l] = (float *)take(z32);
    }
    w.A = (__half *)take(a);
    w.AT = (__half *)take(a);
    w.dX = (float *)take(z32);
    w.dZ = (float *)take(z32);
    w.dZ16 = (__half *)take(x16);
    w.dZT16 = (__half *)take(x16);
    w.sc = (float *)take(64);
    w.amax = (unsigned *)take(64);
    w.loss = (double *)take(64);
    w.part = (float *)take(part);
    w.den = (double *)take(sizeof(double) * 64);
    w.in32 = (float *)take(sizeof(float) * M * NN_CIN0);
    w.mask32 = (float *)take(sizeof(float) * M);
    w.tgt32 = (float *)take(sizeof(float) * M * 6);
    return MIDAS_OK;
}

static unsigned nb(long long n, int t = 256) { return (unsigned)((n + t - 1) / t); }

static int nn_gemm(midas_gpu_ctx *c, int M, int N, int K, const __half *A, long long lda, const __half *Bt,
                   long long ldb, float *D, long long ldd, const float *alpha_dev)
{
    GemmArgs g{M, N, K, (const float *)A, lda, (const float *)Bt, ldb, D, ldd, 1.0f, 0.0f};
    g.h16 = 1;
    g.kclass = MIDAS_KC_NN;
    g.alpha_dev = alpha_dev;
    return gemm_tf32(c, g);
}

// forward through the layers; leaves Z[3] = the output pre-activation without bias
static int nn_forward(midas_gpu_ctx *c, midas_gpu_nn *net, int B, NnWork &w)
{
    const int G = net->grid;
    const long long M = (long long)B * G * G * G;
    ++c->launches;
    k_nn_f32_to_f16<<<nb(M * NN_CIN0), 256, 0, c->stream>>>(M * NN_CIN0, w.in32, w.X16[0]);
    for (int l = 0; l < NN_LAYERS; ++l) {
        const int ci = NN_CI[l], co = NN_CO[l];
        ++c->launches;
        k_nn_im2col<<<nb(M * 27 * (ci / 8)), 256, 0, c->stream>>>(w.X16[l], B, G, ci, w.A);
        MIDAS_TRY(nn_gemm(c, (int)M, co, 27 * ci, w.A, 27 * ci, net->W16[l], 27 * ci, w.Z[l], co, nullptr));
        if (l + 1 < NN_LAYERS) {
            ++c->launches;
            k_nn_bias_relu<<<nb(M * co), 256, 0, c->stream>>>(M, co, w.Z[l], net->b[l], w.X16[l + 1]);
        }
    }
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// loss and the gradients of every parameter (into net->gW / net->gb)
static int nn_backward(midas_gpu_ctx *c, midas_gpu_nn *net, int B, NnWork &w, double *loss)
{
    const int G = net->grid;
    const long long V = (long long)G * G * G, M = B * V;
    MIDAS_CUDA(c, cudaMemsetAsync(w.loss, 0, sizeof(double), c->stream));
    ++c->launches;
    k_nn_loss<<<nb(M), 256, 0, c->stream>>>(M, V, B, w.Z[3], net->b[3], w.in32, w.mask32, w.tgt32, w.den, w.dZ,
                                           w.loss);
    for (int l = NN_LAYERS - 1; l >= 0; --l) {
        const int ci = NN_CI[l], co = NN_CO[l];
        if (l < NN_LAYERS - 1) {   // dZ = dX(l+1) relu'(Z_l); dX was left in w.dX by the layer above
            ++c->launches;
            k_nn_relu_bwd<<<nb(M * co), 256, 0, c->stream>>>(M * co, w.Z[l], w.dX);
            MIDAS_CUDA(c, cudaMemcpyAsync(w.dZ, w.dX, sizeof(float) * M * co, cudaMemcpyDeviceToDevice, c->stream));
        }
        // bias gradient (unscaled)
        const int nblk = (int)((M + NN_ROWS - 1) / NN_ROWS);
        c->launches += 2;
        k_nn_colsum_part<<<nblk, 256, 0, c->stream>>>(M, co, w.dZ, w.part);
        k_nn_colsum_fin<<<1, 32, 0, c->stream>>>(nblk, co, w.part, net->gb[l]);
        // fp16 operands of the gradient GEMMs, scaled into range
        MIDAS_CUDA(c, cudaMemsetAsync(w.amax, 0, sizeof(unsigned), c->stream));
        c->launches += 3;
        k_nn_absmax<<<std::min<unsigned>(nb(M * co), 1024), 256, 0, c->stream>>>(M * co, w.dZ, w.amax);
        k_nn_scale<<<1, 1, 0, c->stream>>>(w.amax, w.sc, w.sc + 1);
        k_nn_dz16<<<nb(M * co), 256, 0, c->stream>>>(M, co, w.dZ, w.sc, w.dZ16, w.dZT16);
        // dW = dZ^T im2col(X) / s
        ++c->launches;
        k_nn_im2col_t<<<nb(M * 27 * ci), 256, 0, c->stream>>>(w.X16[l], B, G, ci, w.AT);
        MIDAS_TRY(nn_gemm(c, co, 27 * ci, (int)M, w.dZT16, M, w.AT, M, net->gW[l], 27 * ci, w.sc + 1));
        // dX = im2col(dZ) W'^T / s (not needed below the first layer)
        if (l > 0) {
            ++c->launches;
            k_nn_im2col<<<nb(M * 27 * (co / 8)), 256, 0, c->stream>>>(w.dZ16, B, G, co, w.A);
            MIDAS_TRY(nn_gemm(c, (int)M, ci, 27 * co, w.A, 27 * co, net->Wf16[l], 27 * co, w.dX, ci, w.sc + 1));
        }
    }
    MIDAS_CUDA(c, cudaGetLastError());
    if (loss) {
        MIDAS_CUDA(c, cudaMemcpyAsync(loss, w.loss, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return MIDAS_OK;
}

static int nn_refresh16(midas_gpu_ctx *c, midas_gpu_nn *net)
{
    for (int l = 0; l < NN_LAYERS; ++l) {
        ++c->launches;
        k_nn_wcopy<<<nb(nn_wcount(l)), 256, 0, c->stream>>>(NN_CO[l], NN_CI[l], net->W[l], net->W16[l], net->Wf16[l]);
    }
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// stage a batch: inputs [B][V][16], mask [B][V], target [B][V][6] (host or device);
// per-sample denominators sum(mask target^2) on the host
static int nn_stage(midas_gpu_ctx *c, midas_gpu_nn *net, int B, const float *in, const float *mask, const float *tgt,
                    NnWork &w)
{
    const long long V = (long long)net->grid * net->grid * net->grid, M = B * V;
    MIDAS_CUDA(c, cudaMemcpyAsync(w.in32, in, sizeof(float) * M * NN_CIN0, cudaMemcpyDefault, c->stream));
    MIDAS_CUDA(c, cudaMemcpyAsync(w.mask32, mask, sizeof(float) * M, cudaMemcpyDefault, c->stream));
    if (tgt) {
        MIDAS_CUDA(c, cudaMemcpyAsync(w.tgt32, tgt, sizeof(float) * M * 6, cudaMemcpyDefault, c->stream));
        std::vector<float> ht(M * 6), hm(M);
        MIDAS_CUDA(c, cudaMemcpyAsync(ht.data(), w.tgt32, sizeof(float) * M * 6, cudaMemcpyDeviceToHost, c->stream));
        MIDAS_CUDA(c, cudaMemcpyAsync(hm.data(), w.mask32, sizeof(float) * M, cudaMemcpyDeviceToHost, c->stream));
        MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
        std::vector<double> den(B, 0.0);
        for (long long r = 0; r < M; ++r)
            if (hm[r] != 0.f)
                for (int k = 0; k < 6; ++k) den[r / V] += (double)ht[r * 6 + k] * ht[r * 6 + k];
        for (auto &d : den)
            if (!(d > 0)) d = 1.0;
        MIDAS_CUDA(c, cudaMemcpyAsync(w.den, den.data(), sizeof(double) * B, cudaMemcpyHostToDevice, c->stream));
        MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// The network as a right preconditioner of flexible GMRES.  A Krylov vector v
// (cells, 3 complex rows per cell) is placed on the network's grid at its
// lattice position, as 16 channels per voxel:
//   0-1  Re, Im chi = eps - 1          2-7   s D^-1 v  (D = 1 - Znnpp, Jacobi)
//   8-13 s v                           14    mask (1)
//   15   Re 3 / (eps + 2)              (0 outside the cells)
// s scales v to O(1) entries.  The network's prediction -- channels 2-7 plus
// its output -- is the scaled approximation of Z^-1 v, gathered back to the
// cells and divided by s.  The lattice box is centred in the grid.
// ---------------------------------------------------------------------------
struct NnPlace {
    int ox, oy, oz, lo0, lo1, lo2;
};

static int nn_place(midas_gpu_ctx *c, const midas_gpu_nn *net, NnPlace *pl)
{
    if (!c->lattice || !c->lat_ijk) return c->err.set(MIDAS_ERR_UNSUPPORTED, "nn preconditioner: cells are not on a lattice");
    int o[3];
    for (int a = 0; a < 3; ++a) {
        const int ext = c->lat_hi[a] - c->lat_lo[a] + 1;
        if (ext > net->grid) return c->err.set(MIDAS_ERR_UNSUPPORTED, "nn preconditioner: lattice wider than the network grid");
        o[a] = (net->grid - ext) / 2;
    }
    *pl = NnPlace{o[0], o[1], o[2], c->lat_lo[0], c->lat_lo[1], c->lat_lo[2]};
    return MIDAS_OK;
}

__device__ __forceinline__ long long nn_voxel(const int *ijk, int i, int G, const NnPlace &pl)
{
    const int x = ijk[3 * i] - pl.lo0 + pl.ox, y = ijk[3 * i + 1] - pl.lo1 + pl.oy, z = ijk[3 * i + 2] - pl.lo2 + pl.oz;
    return ((long long)z * G + y) * G + x;
}

__device__ __forceinline__ double2 nn_cdiv(double2 a, double2 b)
{
    const double den = b.x * b.x + b.y * b.y;
    return make_double2((a.x * b.x + a.y * b.y) / den, (a.y * b.x - a.x * b.y) / den);
}

// one thread per (cell, column); V column k at V + k ldv; scale[k] (or s_all when scale is null)
__global__ void k_nn_prec_scatter(int ncell, int ncol, int G, NnPlace pl, const int *ijk, const double2 *eps,
                                  const double2 *znnpp, const double2 *V, long long ldv, const double *scale,
                                  double s_all, float *in, float *mask)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)ncell * ncol) return;
    const int i = (int)(t % ncell), k = (int)(t / ncell);
    const long long r = (long long)k * G * G * G + nn_voxel(ijk, i, G, pl);
    const double s = scale ? scale[k] : s_all;
    const double2 e = eps[i], d = make_double2(1.0 - znnpp[i].x, -znnpp[i].y);
    const double2 cm = nn_cdiv(make_double2(3.0, 0.0), make_double2(e.x + 2.0, e.y));
    float *row = in + r * NN_CIN0;
    row[0] = (float)(e.x - 1.0);
    row[1] = (float)e.y;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const double2 v = V[(long long)k * ldv + 3 * i + q], w = nn_cdiv(v, d);
        row[2 + 2 * q] = (float)(s * w.x);
        row[3 + 2 * q] = (float)(s * w.y);
        row[8 + 2 * q] = (float)(s * v.x);
        row[9 + 2 * q] = (float)(s * v.y);
    }
    row[14] = 1.f;
    row[15] = (float)cm.x;
    mask[r] = 1.f;
}

// Zout column k = (channels 2-7 + output + bias) / s at each cell
__global__ void k_nn_prec_gather(int ncell, int ncol, int G, NnPlace pl, const int *ijk, const float *in,
                                 const float *D, const float *b, double s_all, double2 *Zout, long long ldz)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)ncell * ncol) return;
    const int i = (int)(t % ncell), k = (int)(t / ncell);
    const long long r = (long long)k * G * G * G + nn_voxel(ijk, i, G, pl);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const double re = (double)in[r * NN_CIN0 + 2 + 2 * q] + (double)(D[r * 8 + 2 * q] + b[2 * q]);
        const double im = (double)in[r * NN_CIN0 + 3 + 2 * q] + (double)(D[r * 8 + 2 * q + 1] + b[2 * q + 1]);
        Zout[(long long)k * ldz + 3 * i + q] = make_double2(re / s_all, im / s_all);
    }
}

static int nn_check(midas_gpu_ctx *c, midas_gpu_nn *net, int B);

static int nn_prec_inputs(midas_gpu_ctx *c, midas_gpu_nn *net, int ncol, const double2 *V, long long ldv,
                          const double *scale, double s_all, float *in, float *mask, const NnPlace &pl)
{
    const long long M = (long long)ncol * net->grid * net->grid * net->grid;
    MIDAS_CUDA(c, cudaMemsetAsync(in, 0, sizeof(float) * M * NN_CIN0, c->stream));
    MIDAS_CUDA(c, cudaMemsetAsync(mask, 0, sizeof(float) * M, c->stream));
    ++c->launches;
    k_nn_prec_scatter<<<nb((long long)c->n * ncol), 256, 0, c->stream>>>(c->n, ncol, net->grid, pl, c->lat_ijk, c->eps,
                                                                        c->znnpp, V, ldv, scale, s_all, in, mask);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

// Zout = P(V) for unit-norm columns V (3n x ncol, ld ldv): the network preconditioner
int nn_prec_apply(midas_gpu_ctx *c, midas_gpu_nn *net, int ncol, const double2 *V, long long ldv, double2 *Zout,
                  long long ldz)
{
    MIDAS_TRY(nn_check(c, net, ncol));
    NnPlace pl;
    MIDAS_TRY(nn_place(c, net, &pl));
    const long long M = (long long)ncol * net->grid * net->grid * net->grid;
    NnWork w;
    MIDAS_TRY(nn_workspace(c, M, w));
    const double s = sqrt((double)c->n);   // |v| = 1: entries of s v are O(1)
    MIDAS_TRY(nn_prec_inputs(c, net, ncol, V, ldv, nullptr, s, w.in32, w.mask32, pl));
    MIDAS_TRY(nn_forward(c, net, ncol, w));
    ++c->launches;
    k_nn_prec_gather<<<nb((long long)c->n * ncol), 256, 0, c->stream>>>(c->n, ncol, net->grid, pl, c->lat_ijk, w.in32,
                                                                       w.Z[NN_LAYERS - 1], net->b[NN_LAYERS - 1], s,
                                                                       Zout, ldz);
    MIDAS_CUDA(c, cudaGetLastError());
    return MIDAS_OK;
}

static int nn_check(midas_gpu_ctx *c, midas_gpu_nn *net, int B)
{
    if (!c || !net) return MIDAS_ERR_ARG;
    if (B <= 0 || B > 64) return c->err.set(MIDAS_ERR_ARG, "nn: batch outside 1..64");
    if ((long long)B * net->grid * net->grid * net->grid > (1LL << 22))
        return c->err.set(MIDAS_ERR_ARG, "nn: batch x grid^3 above 2^22 voxels");
    return MIDAS_OK;
}

}  // namespace midas

using namespace midas;

extern "C" {

int midas_gpu_nn_free(midas_gpu_nn *net)
{
    if (!net) return MIDAS_OK;
    cudaSetDevice(net->device);
    for (int l = 0; l < NN_LAYERS; ++l) {
        float *f[] = {net->W[l], net->b[l], net->gW[l], net->gb[l], net->mW[l], net->vW[l], net->mb[l], net->vb[l]};
        for (float *p : f)
            if (p) cudaFree(p);
        if (net->W16[l]) cudaFree(net->W16[l]);
        if (net->Wf16[l]) cudaFree(net->Wf16[l]);
    }
    delete net;
    return MIDAS_OK;
}

int midas_gpu_nn_create(midas_gpu_ctx *c, int grid, unsigned long long seed, midas_gpu_nn **out)
{
    if (!c || !out || grid < 4 || grid > 128 || grid % 2) return MIDAS_ERR_ARG;   // even: 16-byte GEMM rows
    c->err = Err();
    cudaSetDevice(c->device);
    midas_gpu_nn *net = new midas_gpu_nn();
    net->device = c->device;
    net->grid = grid;
    std::mt19937_64 rng(seed);
    int st = MIDAS_OK;
    for (int l = 0; l < NN_LAYERS && st == MIDAS_OK; ++l) {
        const int n = nn_wcount(l), co = NN_CO[l];
        // He initialisation; the last layer starts small (the prediction starts near E_inc)
        std::normal_distribution<float> nd(0.f, sqrtf(2.f / (27.f * NN_CI[l])) * (l == NN_LAYERS - 1 ? 0.1f : 1.f));
        std::vector<float> w(n);
        for (int t = 0; t < n; ++t) w[t] = (l == NN_LAYERS - 1 && t / (27 * NN_CI[l]) >= NN_COUT) ? 0.f : nd(rng);
        float **wb[] = {&net->W[l], &net->gW[l], &net->mW[l], &net->vW[l]};
        for (float **b : wb)
            if (st == MIDAS_OK && cudaMalloc(b, sizeof(float) * n) != cudaSuccess) st = MIDAS_ERR_ALLOC;
        float **bb[] = {&net->b[l], &net->gb[l], &net->mb[l], &net->vb[l]};
        for (float **b : bb)
            if (st == MIDAS_OK && cudaMalloc(b, sizeof(float) * co) != cudaSuccess) st = MIDAS_ERR_ALLOC;
        if (st == MIDAS_OK && (cudaMalloc(&net->W16[l], sizeof(__half) * n) != cudaSuccess ||
                               cudaMalloc(&net->Wf16[l], sizeof(__half) * n) != cudaSuccess))
            st = MIDAS_ERR_ALLOC;
        if (st != MIDAS_OK) break;
        for (float **b : wb) cudaMemsetAsync(*b, 0, sizeof(float) * n, c->stream);
        for (float **b : bb) cudaMemsetAsync(*b, 0, sizeof(float) * co, c->stream);
        cudaMemcpyAsync(net->W[l], w.data(), sizeof(float) * n, cudaMemcpyHostToDevice, c->stream);
    }
    if (st == MIDAS_OK) st = nn_refresh16(c, net);
    if (st == MIDAS_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) st = MIDAS_ERR_CUDA;
    if (st != MIDAS_OK) {
        cudaGetLastError();
        midas_gpu_nn_free(net);
        return c->err.set(st, "nn_create: device allocation or set-up failed");
    }
    *out = net;
    return MIDAS_OK;
}

long long midas_gpu_nn_param_count(const midas_gpu_nn *net)
{
    (void)net;
    long long n = 0;
    for (int l = 0; l < NN_LAYERS; ++l) n += nn_wcount(l) + NN_CO[l];
    return n;
}

int midas_gpu_nn_params(midas_gpu_ctx *c, midas_gpu_nn *net, int set, float *buf, int grads)
{
    if (!c || !net || !buf) return MIDAS_ERR_ARG;
    c->err = Err();
    cudaSetDevice(c->device);
    if (set && grads) return c->err.set(MIDAS_ERR_ARG, "nn_params: gradients are read-only");
    long long off = 0;
    for (int l = 0; l < NN_LAYERS; ++l) {
        float *W = grads ? net->gW[l] : net->W[l], *b = grads ? net->gb[l] : net->b[l];
        const size_t nw = nn_wcount(l), nbias = NN_CO[l];
        if (set) {
            MIDAS_CUDA(c, cudaMemcpyAsync(W, buf + off, sizeof(float) * nw, cudaMemcpyDefault, c->stream));
            MIDAS_CUDA(c, cudaMemcpyAsync(b, buf + off + nw, sizeof(float) * nbias, cudaMemcpyDefault, c->stream));
        } else {
            MIDAS_CUDA(c, cudaMemcpyAsync(buf + off, W, sizeof(float) * nw, cudaMemcpyDefault, c->stream));
            MIDAS_CUDA(c, cudaMemcpyAsync(buf + off + nw, b, sizeof(float) * nbias, cudaMemcpyDefault, c->stream));
        }
        off += nw + nbias;
    }
    if (set) MIDAS_TRY(nn_refresh16(c, net));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    return MIDAS_OK;
}

int midas_gpu_nn_forward(midas_gpu_ctx *c, midas_gpu_nn *net, int batch, const float *inputs, const float *mask,
                         float *E)
{
    MIDAS_TRY(nn_check(c, net, batch));
    if (!inputs || !mask || !E) return MIDAS_ERR_ARG;
    c->err = Err();
    cudaSetDevice(c->device);
    const long long M = (long long)batch * net->grid * net->grid * net->grid;
    NnWork w;
    MIDAS_TRY(nn_workspace(c, M, w));
    MIDAS_TRY(nn_stage(c, net, batch, inputs, mask, nullptr, w));
    MIDAS_TRY(nn_forward(c, net, batch, w));
    float *out = E;
    if (!is_device_ptr(E)) {
        void *p;
        MIDAS_TRY(ensure(c, S_OUT0, sizeof(float) * M * 6, &p));
        out = (float *)p;
    }
    ++c->launches;
    k_nn_predict<<<nb(M * NN_COUT), 256, 0, c->stream>>>(M, w.Z[3], net->b[3], w.in32, w.mask32, out);
    MIDAS_CUDA(c, cudaGetLastError());
    if (out != E) MIDAS_CUDA(c, cudaMemcpyAsync(E, out, sizeof(float) * M * 6, cudaMemcpyDeviceToHost, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    return check_flag(c, "nn_forward");
}

int midas_gpu_nn_prec_grid(midas_gpu_ctx *c, midas_gpu_nn *net, int ncol, const double *V, const double *scale,
                           float *inputs, float *mask)
{
    MIDAS_TRY(nn_check(c, net, ncol));
    if (!V || !scale || !inputs || !mask) return MIDAS_ERR_ARG;
    c->err = Err();
    cudaSetDevice(c->device);
    if (c->n <= 0) return c->err.set(MIDAS_ERR_STATE, "nn_prec_grid: no cells");
    NnPlace pl;
    MIDAS_TRY(nn_place(c, net, &pl));
    const long long M = (long long)ncol * net->grid * net->grid * net->grid;
    const size_t vb = sizeof(double2) * 3 * (size_t)c->n * ncol;
    void *pv, *ps, *po;
    MIDAS_TRY(ensure(c, S_IN2, vb, &pv));
    MIDAS_TRY(ensure(c, S_IN3, sizeof(double) * ncol, &ps));
    MIDAS_TRY(ensure(c, S_OUT0, sizeof(float) * M * (NN_CIN0 + 1), &po));
    MIDAS_CUDA(c, cudaMemcpyAsync(pv, V, vb, cudaMemcpyDefault, c->stream));
    MIDAS_CUDA(c, cudaMemcpyAsync(ps, scale, sizeof(double) * ncol, cudaMemcpyDefault, c->stream));
    float *din = (float *)po, *dmask = din + M * NN_CIN0;
    MIDAS_TRY(nn_prec_inputs(c, net, ncol, (const double2 *)pv, 3LL * c->n, (const double *)ps, 0.0, din, dmask, pl));
    MIDAS_CUDA(c, cudaMemcpyAsync(inputs, din, sizeof(float) * M * NN_CIN0, cudaMemcpyDefault, c->stream));
    MIDAS_CUDA(c, cudaMemcpyAsync(mask, dmask, sizeof(float) * M, cudaMemcpyDefault, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    return check_flag(c, "nn_prec_grid");
}

int midas_gpu_nn_gradients(midas_gpu_ctx *c, midas_gpu_nn *net, int batch, const float *inputs, const float *mask,
                           const float *target, double *loss)
{
    MIDAS_TRY(nn_check(c, net, batch));
    if (!inputs || !mask || !target) return MIDAS_ERR_ARG;
    c->err = Err();
    cudaSetDevice(c->device);
    const long long M = (long long)batch * net->grid * net->grid * net->grid;
    NnWork w;
    MIDAS_TRY(nn_workspace(c, M, w));
    MIDAS_TRY(nn_stage(c, net, batch, inputs, mask, target, w));
    MIDAS_TRY(nn_forward(c, net, batch, w));
    double l = 0;
    MIDAS_TRY(nn_backward(c, net, batch, w, &l));
    if (loss) *loss = l;
    return check_flag(c, "nn_gradients");
}

int midas_gpu_nn_train_step(midas_gpu_ctx *c, midas_gpu_nn *net, int batch, const float *inputs, const float *mask,
                            const float *target, float lr, double *loss)
{
    MIDAS_TRY(midas_gpu_nn_gradients(c, net, batch, inputs, mask, target, loss));
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    net->step += 1;
    const float c1 = 1.f - powf(b1, (float)net->step), c2 = 1.f - powf(b2, (float)net->step);
    for (int l = 0; l < NN_LAYERS; ++l) {
        const int live = l == NN_LAYERS - 1 ? NN_COUT : NN_CO[l];
        c->launches += 2;
        k_nn_adam<<<nb(nn_wcount(l)), 256, 0, c->stream>>>(nn_wcount(l), net->W[l], net->gW[l], net->mW[l],
                                                           net->vW[l], lr, b1, b2, c1, c2, eps, live, 27 * NN_CI[l]);
        k_nn_adam<<<1, 32, 0, c->stream>>>(NN_CO[l], net->b[l], net->gb[l], net->mb[l], net->vb[l], lr, b1, b2, c1, c2,
                                          eps, live, 1);
    }
    MIDAS_TRY(nn_refresh16(c, net));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    return check_flag(c, "nn_train_step");
}

}  // extern "C"
