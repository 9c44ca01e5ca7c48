// prep.cu -- scene preparation on the device (sm_103a): voxelisation, block
// partition and block extension, the inputs of the CBFM solve.
//
// The reference prepares a scene on the host before the solve: the sphere
// voxeliser (src/Discretization.f90:246-310), the block division
// (src/Division_blocks.f90) and Extend_blocks (src/Extend_blocks.f90:46-151).
// For batches of many small scatterers (hundreds of aggregates) that host work
// is a serial step between GPU solves; here each piece is a flag pass over a
// candidate index space plus an order-preserving compaction, so the results
// come out in exactly the order the host loops produce them.
//
//   voxelise_sphere   the reference's seven-domain sphere voxeliser: the
//                     inscribed cube, then the six slabs around it, each swept
//                     z, y, x with the inside test sqrt(x^2 + y^2 + z^2) < ap;
//   voxelise_spheres  union of spheres on one lattice (aggregates), lattice
//                     order x slowest, z fastest;
//   box_partition     nx x ny x nz bounding-box blocks, a stable counting sort
//                     of the cells by block (empty blocks dropped);
//   extend_blocks     SetBlockCtrs contours, neighbours by bounding-sphere
//                     distance, and every neighbour cell inside the block box
//                     grown by ExtLength + Sc / 2, neighbours in block order.
// Every floating-point operation is an explicitly rounded intrinsic, in the
// host restatement's order, so the flags agree bit for bit.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace midas {

// exclusive scan of n flags / counts (one CTA of 1024 threads, int64 totals)
__global__ void __launch_bounds__(1024) k_prep_scan(long long n, const int *in, long long *out)
{
    __shared__ long long part[32];
    __shared__ long long carry;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) carry = 0;
    __syncthreads();
    for (long long base = 0; base < n; base += 1024) {
        const long long v = base + tid < n ? in[base + tid] : 0;
        long long x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) part[w] = x;
        __syncthreads();
        if (w == 0) {
            long long p = part[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const long long y = __shfl_up_sync(0xffffffffu, p, o);
                if (lane >= o) p += y;
            }
            part[lane] = p;
        }
        __syncthreads();
        const long long incl = x + (w > 0 ? part[w - 1] : 0);
        if (base + tid < n) out[base + tid] = carry + incl - v;
        __syncthreads();
        if (tid == 1023) carry += incl;
        __syncthreads();
    }
    if (tid == 0) out[n] = carry;
}

// ---------------------------------------------------------------------------
// sphere voxeliser (src/Discretization.f90:246-310)
// ---------------------------------------------------------------------------
struct SphDom {
    double sx[7], sy[7], sz[7];
    int nx[7], ny[7], nz[7];
    long long off[8];   // first candidate of each domain
    double ap, sc;
};

__device__ __forceinline__ void sph_candidate(const SphDom &D, long long t, int &d, double &px, double &py,
                                              double &pz)
{
    d = 0;
    while (d < 6 && t >= D.off[d + 1]) ++d;
    const long long u = t - D.off[d];
    const int ix = (int)(u % D.nx[d]) + 1;
    const int iy = (int)((u / D.nx[d]) % D.ny[d]) + 1;
    const int iz = (int)(u / ((long long)D.nx[d] * D.ny[d])) + 1;
    px = __dadd_rn(D.sx[d], __dmul_rn((double)ix - 0.5, D.sc));
    py = __dadd_rn(D.sy[d], __dmul_rn((double)iy - 0.5, D.sc));
    pz = __dadd_rn(D.sz[d], __dmul_rn((double)iz - 0.5, D.sc));
}

__global__ void k_sph_flags(SphDom D, int *flag)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= D.off[7]) return;
    int d;
    double px, py, pz;
    sph_candidate(D, t, d, px, py, pz);
    const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(px, px), __dmul_rn(py, py)), __dmul_rn(pz, pz)));
    flag[t] = (d == 0 || r < D.ap) ? 1 : 0;
}

__global__ void k_sph_emit(SphDom D, const int *flag, const long long *pos, long long cap, double *x, double *y,
                           double *z)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= D.off[7] || !flag[t] || pos[t] >= cap) return;
    int d;
    double px, py, pz;
    sph_candidate(D, t, d, px, py, pz);
    x[pos[t]] = px;
    y[pos[t]] = py;
    z[pos[t]] = pz;
}

int voxelise_sphere(midas_gpu_ctx *c, double dm, double sc, long long cap, double *x, double *y, double *z,
                    long long *ncell)
{
    if (!(dm > 0) || !(sc > 0) || dm / sc > 4096) return c->err.set(MIDAS_ERR_ARG, "voxelise_sphere: bad size");
    SphDom D;
    const double ap = dm / 2.;
    const int nd = (int)floor(dm / sc + 0.5);                       // nint(dm / Sc)
    const double q = (double)0.8f * ap / (double)sqrtf(3.0f);       // 0.8 and sqrt(3.) in single precision
    const int next = (int)ceil((ap - q) / sc);
    const int nin = nd - 2 * next;
    const double api = (nin * sc) / 2.;
    const double sx[7] = {-api, -ap, -ap, api, -api, -api, -ap}, sy[7] = {-api, -ap, -ap, -ap, -ap, api, -ap},
                 sz[7] = {-api, -ap, -api, -api, -api, -api, api};
    const int nx[7] = {nin, nd, next, next, nin, nin, nd}, ny[7] = {nin, nd, nd, nd, next, next, nd},
              nz[7] = {nin, next, nin, nin, nin, nin, next};
    D.off[0] = 0;
    for (int d = 0; d < 7; ++d) {
        D.sx[d] = sx[d]; D.sy[d] = sy[d]; D.sz[d] = sz[d];
        D.nx[d] = std::max(nx[d], 1); D.ny[d] = std::max(ny[d], 1); D.nz[d] = std::max(nz[d], 1);
        const long long cnt = (nx[d] > 0 && ny[d] > 0 && nz[d] > 0) ? (long long)nx[d] * ny[d] * nz[d] : 0;
        D.off[d + 1] = D.off[d] + cnt;
    }
    D.ap = ap;
    D.sc = sc;
    const long long tot = D.off[7];
    void *p;
    MIDAS_TRY(ensure(c, S_PREP, sizeof(int) * (size_t)tot + sizeof(long long) * (size_t)(tot + 1) + 512, &p));
    int *flag = (int *)p;
    long long *pos = (long long *)(((uintptr_t)(flag + tot) + 255) & ~(uintptr_t)255);
    c->launches += 2;
    k_sph_flags<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(D, flag);
    k_prep_scan<<<1, 1024, 0, c->stream>>>(tot, flag, pos);
    MIDAS_CUDA(c, cudaGetLastError());
    MIDAS_CUDA(c, cudaMemcpyAsync(ncell, pos + tot, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
    if (x && y && z && cap > 0) {
        ++c->launches;
        k_sph_emit<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(D, flag, pos, cap, x, y, z);
        MIDAS_CUDA(c, cudaGetLastError());
    }
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// union of spheres on one lattice (aggregates of monomers)
// ---------------------------------------------------------------------------
__global__ void k_spheres_flags(long long tot, int d0, int d1, int d2, double lo0, double lo1, double lo2, double d,
                                int nsph, const double *cen, double a2, int *flag)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= tot) return;
    const int k = (int)(t % d2), j = (int)((t / d2) % d1), i = (int)(t / ((long long)d1 * d2));
    const double px = __dadd_rn(lo0, __dmul_rn((double)i + 0.5, d));
    const double py = __dadd_rn(lo1, __dmul_rn((double)j + 0.5, d));
    const double pz = __dadd_rn(lo2, __dmul_rn((double)k + 0.5, d));
    int in = 0;
    for (int s = 0; s < nsph && !in; ++s) {
        const double dx = __dsub_rn(px, cen[3 * s]), dy = __dsub_rn(py, cen[3 * s + 1]),
                     dz = __dsub_rn(pz, cen[3 * s + 2]);
        in = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)) < a2;
    }
    flag[t] = in;
}

__global__ void k_spheres_emit(long long tot, int d0, int d1, int d2, double lo0, double lo1, double lo2, double d,
                               const int *flag, const long long *pos, long long cap, double *x, double *y, double *z)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= tot || !flag[t] || pos[t] >= cap) return;
    const int k = (int)(t % d2), j = (int)((t / d2) % d1), i = (int)(t / ((long long)d1 * d2));
    x[pos[t]] = __dadd_rn(lo0, __dmul_rn((double)i + 0.5, d));
    y[pos[t]] = __dadd_rn(lo1, __dmul_rn((double)j + 0.5, d));
    z[pos[t]] = __dadd_rn(lo2, __dmul_rn((double)k + 0.5, d));
}

int voxelise_spheres(midas_gpu_ctx *c, int nsph, const double *centres, double a, int cells_per_diameter,
                     long long cap, double *x, double *y, double *z, long long *ncell, double *edge)
{
    if (nsph <= 0 || !centres || !(a > 0) || cells_per_diameter <= 0)
        return c->err.set(MIDAS_ERR_ARG, "voxelise_spheres: bad arguments");
    std::vector<double> h(3 * (size_t)nsph);
    MIDAS_CUDA(c, cudaMemcpy(h.data(), centres, sizeof(double) * h.size(), cudaMemcpyDefault));
    const double d = 2.0 * a / cells_per_diameter;
    double lo[3], hi[3];
    int dims[3];
    for (int k = 0; k < 3; ++k) {
        lo[k] = hi[k] = h[k];
        for (int s = 1; s < nsph; ++s) { lo[k] = std::min(lo[k], h[3 * s + k]); hi[k] = std::max(hi[k], h[3 * s + k]); }
        lo[k] -= a;
        dims[k] = (int)ceil((hi[k] + a - lo[k]) / d) + 1;
    }
    const long long tot = (long long)dims[0] * dims[1] * dims[2];
    if (tot > (1LL << 31)) return c->err.set(MIDAS_ERR_ARG, "voxelise_spheres: lattice too large");
    void *p;
    MIDAS_TRY(ensure(c, S_PREP, sizeof(int) * (size_t)tot + sizeof(long long) * (size_t)(tot + 1) +
                                    sizeof(double) * h.size() + 1024, &p));
    int *flag = (int *)p;
    long long *pos = (long long *)(((uintptr_t)(flag + tot) + 255) & ~(uintptr_t)255);
    double *dcen = (double *)(((uintptr_t)(pos + tot + 1) + 255) & ~(uintptr_t)255);
    MIDAS_CUDA(c, cudaMemcpyAsync(dcen, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, c->stream));
    c->launches += 2;
    k_spheres_flags<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(tot, dims[0], dims[1], dims[2], lo[0], lo[1],
                                                                          lo[2], d, nsph, dcen, a * a, flag);
    k_prep_scan<<<1, 1024, 0, c->stream>>>(tot, flag, pos);
    MIDAS_CUDA(c, cudaGetLastError());
    MIDAS_CUDA(c, cudaMemcpyAsync(ncell, pos + tot, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
    if (x && y && z && cap > 0) {
        ++c->launches;
        k_spheres_emit<<<(unsigned)((tot + 255) / 256), 256, 0, c->stream>>>(tot, dims[0], dims[1], dims[2], lo[0],
                                                                             lo[1], lo[2], d, flag, pos, cap, x, y, z);
        MIDAS_CUDA(c, cudaGetLastError());
    }
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    if (edge) *edge = d;
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// bounding-box partition: block of each cell, stable counting sort
// ---------------------------------------------------------------------------
__global__ void k_minmax3(int n, const double *x, const double *y, const double *z, double *out)
{
    __shared__ double red[6][256];
    double v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        v[0] = fmin(v[0], x[i]); v[1] = fmin(v[1], y[i]); v[2] = fmin(v[2], z[i]);
        v[3] = fmax(v[3], x[i]); v[4] = fmax(v[4], y[i]); v[5] = fmax(v[5], z[i]);
    }
    for (int q = 0; q < 6; ++q) red[q][threadIdx.x] = v[q];
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int q = 0; q < 6; ++q)
                red[q][threadIdx.x] = q < 3 ? fmin(red[q][threadIdx.x], red[q][threadIdx.x + o])
                                            : fmax(red[q][threadIdx.x], red[q][threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x < 6) out[threadIdx.x] = red[threadIdx.x][0];
}

__global__ void k_block_id(int n, const double *x, const double *y, const double *z, const double *mm, int nx, int ny,
                           int nz, int *bid)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double p[3] = {x[i], y[i], z[i]};
    const int ns[3] = {nx, ny, nz};
    int ijk[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double span = mm[3 + a] > mm[a] ? __dsub_rn(mm[3 + a], mm[a]) : 1.0;
        const double f = __dmul_rn(__ddiv_rn(__dsub_rn(p[a], mm[a]), span), (double)ns[a]);
        ijk[a] = f >= 0.0 ? min((int)fmin(f, (double)ns[a]), ns[a] - 1) : 0;   // NaN or negative -> block 0
    }
    bid[i] = (ijk[2] * ny + ijk[1]) * nx + ijk[0];
}

// chunk histograms: hist[b * nchunk + ch] = cells of chunk ch in block b
constexpr int PREP_CHUNK = 256;
__global__ void k_chunk_hist(int n, int nb, const int *bid, int *hist)
{
    const int ch = blockIdx.x * blockDim.x + threadIdx.x, nchunk = (n + PREP_CHUNK - 1) / PREP_CHUNK;
    if (ch >= nchunk) return;
    for (int b = 0; b < nb; ++b) hist[(long long)b * nchunk + ch] = 0;
    const int i1 = min(n, (ch + 1) * PREP_CHUNK);
    for (int i = ch * PREP_CHUNK; i < i1; ++i) hist[(long long)bid[i] * nchunk + ch] += 1;
}

// stable scatter: each chunk's cells in index order to start[b * nchunk + ch]
__global__ void k_chunk_scatter(int n, int nb, const int *bid, long long *start, int *perm, int base)
{
    const int ch = blockIdx.x * blockDim.x + threadIdx.x, nchunk = (n + PREP_CHUNK - 1) / PREP_CHUNK;
    if (ch >= nchunk) return;
    const int i1 = min(n, (ch + 1) * PREP_CHUNK);
    for (int i = ch * PREP_CHUNK; i < i1; ++i) {
        const long long o = (long long)bid[i] * nchunk + ch;
        perm[start[o]] = i + base;
        start[o] += 1;   // the chunk owns its slot range of block bid[i]: advance its cursor
    }
}

int box_partition(midas_gpu_ctx *c, int n, const double *x, const double *y, const double *z, int nx, int ny, int nz,
                  int *perm, int *blk_offsets, int *nblocks)
{
    if (n <= 0 || nx <= 0 || ny <= 0 || nz <= 0 || (long long)nx * ny * nz > 4096)
        return c->err.set(MIDAS_ERR_ARG, "box_partition: bad sizes");
    const int nb = nx * ny * nz, nchunk = (n + PREP_CHUNK - 1) / PREP_CHUNK;
    const long long nh = (long long)nb * nchunk;
    void *p;
    MIDAS_TRY(ensure(c, S_PREP, sizeof(double) * 8 + sizeof(int) * ((size_t)n + nh) + sizeof(long long) * (nh + 1) +
                                    1024, &p));
    double *mm = (double *)p;
    int *bid = (int *)(mm + 8);
    int *hist = bid + n;
    long long *start = (long long *)(((uintptr_t)(hist + nh) + 255) & ~(uintptr_t)255);
    c->launches += 5;
    k_minmax3<<<1, 256, 0, c->stream>>>(n, x, y, z, mm);
    k_block_id<<<(n + 255) / 256, 256, 0, c->stream>>>(n, x, y, z, mm, nx, ny, nz, bid);
    k_chunk_hist<<<(nchunk + 127) / 128, 128, 0, c->stream>>>(n, nb, bid, hist);
    k_prep_scan<<<1, 1024, 0, c->stream>>>(nh, hist, start);   // block-major: blocks in order, chunks in order
    std::vector<long long> hstart(nb + 1);
    // block b starts at start[b * nchunk]
    for (int b = 0; b < nb; ++b)
        MIDAS_CUDA(c, cudaMemcpyAsync(&hstart[b], start + (long long)b * nchunk, sizeof(long long),
                                      cudaMemcpyDeviceToHost, c->stream));
    MIDAS_CUDA(c, cudaMemcpyAsync(&hstart[nb], start + nh, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
    k_chunk_scatter<<<(nchunk + 127) / 128, 128, 0, c->stream>>>(n, nb, bid, start, perm, c->opts.index_base);
    MIDAS_CUDA(c, cudaGetLastError());
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    // offsets of the non-empty blocks
    int k = 0;
    blk_offsets[0] = c->opts.index_base;
    for (int b = 0; b < nb; ++b)
        if (hstart[b + 1] > hstart[b]) blk_offsets[++k] = (int)hstart[b + 1] + c->opts.index_base;
    *nblocks = k;
    return MIDAS_OK;
}

// ---------------------------------------------------------------------------
// Extend_blocks (src/Extend_blocks.f90:46-151) with SetBlockCtrs
// (src/Division_blocks.f90:1616-1662): box and bounding sphere per block
// ---------------------------------------------------------------------------
// ctr[b * 10 + ...]: box lo (3), box hi (3), sphere centre (3), radius
__global__ void k_block_ctrs(const int *offs, const double *x, const double *y, const double *z, double *ctr)
{
    __shared__ double red[6][256];
    __shared__ double box[6];
    const int b = blockIdx.x, i0 = offs[b], i1 = offs[b + 1];
    double v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        v[0] = fmin(v[0], x[i]); v[1] = fmin(v[1], y[i]); v[2] = fmin(v[2], z[i]);
        v[3] = fmax(v[3], x[i]); v[4] = fmax(v[4], y[i]); v[5] = fmax(v[5], z[i]);
    }
    for (int q = 0; q < 6; ++q) red[q][threadIdx.x] = v[q];
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int q = 0; q < 6; ++q)
                red[q][threadIdx.x] = q < 3 ? fmin(red[q][threadIdx.x], red[q][threadIdx.x + o])
                                            : fmax(red[q][threadIdx.x], red[q][threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x < 6) box[threadIdx.x] = red[threadIdx.x][0];
    __syncthreads();
    // bounding sphere: centre of the box, radius = largest centroid distance
    const double c0 = __ddiv_rn(__dadd_rn(box[0], box[3]), 2.0), c1 = __ddiv_rn(__dadd_rn(box[1], box[4]), 2.0),
                 c2 = __ddiv_rn(__dadd_rn(box[2], box[5]), 2.0);
    double r2 = 0;
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const double dx = __dsub_rn(x[i], c0), dy = __dsub_rn(y[i], c1), dz = __dsub_rn(z[i], c2);
        r2 = fmax(r2, __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
    }
    red[0][threadIdx.x] = r2;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[0][threadIdx.x] = fmax(red[0][threadIdx.x], red[0][threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double *o = ctr + 10 * b;
        for (int q = 0; q < 6; ++q) o[q] = box[q];
        o[6] = c0;
        o[7] = c1;
        o[8] = c2;
        o[9] = __dsqrt_rn(red[0][0]);
    }
}

__global__ void k_cell_block(const int *offs, int nb, int *bid)
{
    const int b = blockIdx.y;
    const int i = offs[b] + blockIdx.x * blockDim.x + threadIdx.x;
    if (i < offs[b + 1]) bid[i] = b;
}

// flag[b * n + i] = cell i (of block bid[i]) extends block b
__global__ void k_ext_flags(int n, int nb, const int *bid, const unsigned char *adj, const double *lohi,
                            const double *x, const double *y, const double *z, int *flag)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (i >= n) return;
    const int bp = bid[i];
    int f = 0;
    if (bp != b && adj[(long long)b * nb + bp]) {
        const double *q = lohi + 6 * b;
        f = q[0] <= x[i] && x[i] <= q[3] && q[1] <= y[i] && y[i] <= q[4] && q[2] <= z[i] && z[i] <= q[5];
    }
    flag[(long long)b * n + i] = f;
}

__global__ void k_ext_emit(int n, int nb, const int *flag, const long long *pos, long long cap, int base, int *ext)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, b = blockIdx.y;
    if (i >= n) return;
    const long long t = (long long)b * n + i;
    if (flag[t] && pos[t] < cap) ext[pos[t]] = i + base;
}

int extend_blocks(midas_gpu_ctx *c, int n, const double *x, const double *y, const double *z, int nb,
                  const int *offs_host, double ext_length, double sc, int *ext_offsets, long long cap, int *ext_idx,
                  long long *ntotal)
{
    if (n <= 0 || nb <= 0 || (long long)nb * n > (1LL << 30) || !(ext_length >= 0) || !(sc > 0))
        return c->err.set(MIDAS_ERR_ARG, "extend_blocks: bad sizes");
    const long long nf = (long long)nb * n;
    void *p;
    MIDAS_TRY(ensure(c, S_PREP, sizeof(int) * ((size_t)nb + 1 + n + nf) + sizeof(double) * (16 * (size_t)nb) +
                                    (size_t)nb * nb + sizeof(long long) * (nf + 1) + 4096, &p));
    char *base = (char *)p;
    auto take = [&](size_t bytes) { char *q = base; base += (bytes + 255) & ~(size_t)255; return (void *)q; };
    int *doffs = (int *)take(sizeof(int) * (nb + 1));
    int *bid = (int *)take(sizeof(int) * n);
    int *flag = (int *)take(sizeof(int) * nf);
    double *ctr = (double *)take(sizeof(double) * 10 * nb);
    double *lohi = (double *)take(sizeof(double) * 6 * nb);
    unsigned char *adj = (unsigned char *)take((size_t)nb * nb);
    long long *pos = (long long *)take(sizeof(long long) * (nf + 1));
    MIDAS_CUDA(c, cudaMemcpyAsync(doffs, offs_host, sizeof(int) * (nb + 1), cudaMemcpyHostToDevice, c->stream));
    int maxb = 1;
    for (int b = 0; b < nb; ++b) maxb = std::max(maxb, offs_host[b + 1] - offs_host[b]);
    c->launches += 2;
    k_block_ctrs<<<nb, 256, 0, c->stream>>>(doffs, x, y, z, ctr);
    k_cell_block<<<dim3((maxb + 255) / 256, nb), 256, 0, c->stream>>>(doffs, nb, bid);
    std::vector<double> h(10 * (size_t)nb);
    MIDAS_CUDA(c, cudaMemcpyAsync(h.data(), ctr, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    // neighbours by bounding-sphere distance and the grown boxes (host, nb^2 tests)
    std::vector<unsigned char> hadj((size_t)nb * nb, 0);
    std::vector<double> hlh(6 * (size_t)nb);
    for (int b = 0; b < nb; ++b) {
        const double *sb = &h[10 * (size_t)b];
        for (int q = 0; q < 3; ++q) {
            hlh[6 * b + q] = (sb[q] - ext_length) - sc / 2.0;
            hlh[6 * b + 3 + q] = (sb[3 + q] + ext_length) + sc / 2.0;
        }
        for (int bp = 0; bp < nb; ++bp) {
            if (bp == b) continue;
            const double *sp = &h[10 * (size_t)bp];
            const double dx = sp[6] - sb[6], dy = sp[7] - sb[7], dz = sp[8] - sb[8];
            const double dis = sqrt((dx * dx + dy * dy) + dz * dz);
            hadj[(size_t)b * nb + bp] = !(dis > (sb[9] + sp[9]) + ext_length);
        }
    }
    MIDAS_CUDA(c, cudaMemcpyAsync(adj, hadj.data(), hadj.size(), cudaMemcpyHostToDevice, c->stream));
    MIDAS_CUDA(c, cudaMemcpyAsync(lohi, hlh.data(), sizeof(double) * hlh.size(), cudaMemcpyHostToDevice, c->stream));
    const dim3 grd((unsigned)((n + 255) / 256), (unsigned)nb);
    c->launches += 2;
    k_ext_flags<<<grd, 256, 0, c->stream>>>(n, nb, bid, adj, lohi, x, y, z, flag);
    k_prep_scan<<<1, 1024, 0, c->stream>>>(nf, flag, pos);
    std::vector<long long> hpos(nb + 1);
    for (int b = 0; b <= nb; ++b)
        MIDAS_CUDA(c, cudaMemcpyAsync(&hpos[b], pos + (long long)b * n, sizeof(long long), cudaMemcpyDeviceToHost,
                                      c->stream));
    if (ext_idx && cap > 0) {
        ++c->launches;
        k_ext_emit<<<grd, 256, 0, c->stream>>>(n, nb, flag, pos, cap, c->opts.index_base, ext_idx);
    }
    MIDAS_CUDA(c, cudaGetLastError());
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int b = 0; b <= nb; ++b) ext_offsets[b] = (int)hpos[b] + c->opts.index_base;
    *ntotal = hpos[nb];
    return MIDAS_OK;
}

}  // namespace midas

using namespace midas;

// device buffer for an output that may be host memory: the caller's pointer when
// it is device memory, else a pool slot (copied back by out_done)
static int out_buf(midas_gpu_ctx *c, void *user, size_t bytes, int slot, void **dev)
{
    if (is_device_ptr(user)) { *dev = user; return MIDAS_OK; }
    return ensure(c, slot, bytes, dev);
}
static int out_done(midas_gpu_ctx *c, void *user, const void *dev, size_t bytes)
{
    if (user == dev || bytes == 0) return MIDAS_OK;
    MIDAS_CUDA(c, cudaMemcpyAsync(user, dev, bytes, cudaMemcpyDeviceToHost, c->stream));
    MIDAS_CUDA(c, cudaStreamSynchronize(c->stream));
    return MIDAS_OK;
}

extern "C" {

int midas_gpu_voxelise_sphere(midas_gpu_ctx *c, double dm, double sc, long long cap, double *xc, double *yc,
                              double *zc, long long *ncell)
{
    if (!c || !ncell) return MIDAS_ERR_ARG;
    c->err = Err();
    cudaSetDevice(c->device);
    const bool want = xc && yc && zc && cap > 0;
    const size_t b = sizeof(double) * (want ? (size_t)cap : 0);
    void *dx = nullptr, *dy = nullptr, *dz = nullptr;
    if (want) {
        MIDAS_TRY(out_buf(c, xc, b, S_OUT0, &dx));
        MIDAS_TRY(out_buf(c, yc, b, S_OUT1, &dy));
        MIDAS_TRY(out_buf(c, zc, b, S_IN5, &dz));
    }
    long long cnt = 0;
    MIDAS_TRY(voxelise_sphere(c, dm, sc, want ? cap : 0, (double *)dx, (double *)dy, (double *)dz, &cnt));
    *ncell = cnt;
    if (want) {
        const size_t nb = sizeof(double) * (size_t)std::min(cnt, cap);
        MIDAS_TRY(out_done(c, xc, dx, nb));
        MIDAS_TRY(out_done(c, yc, dy, nb));
        MIDAS_TRY(out_done(c, zc, dz, nb));
    }
    return MIDAS_OK;
}

int midas_gpu_voxelise_spheres(midas_gpu_ctx *c, int nsph, const double *centres, double a, int cells_per_diameter,
                               long long cap, double *xc, double *yc, double *zc, long long *ncell, double *edge)
{
    if (!c || !ncell) return MIDAS_ERR_ARG;
    c->err = Err();
    cudaSetDevice(c->device);
    const bool want = xc && yc && zc && cap > 0;
    const size_t b = sizeof(double) * (want ? (size_t)cap : 0);
    void *dx = nullptr, *dy = nullptr, *dz = nullptr;
    if (want) {
        MIDAS_TRY(out_buf(c, xc, b, S_OUT0, &dx));
        MIDAS_TRY(out_buf(c, yc, b, S_OUT1, &dy));
        MIDAS_TRY(out_buf(c, zc, b, S_IN5, &dz));
    }
    long long cnt = 0;
    MIDAS_TRY(voxelise_spheres(c, nsph, centres, a, cells_per_diameter, want ? cap : 0, (double *)dx, (double *)dy,
                               (double *)dz, &cnt, edge));
    *ncell = cnt;
    if (want) {
        const size_t nb = sizeof(double) * (size_t)std::min(cnt, cap);
        MIDAS_TRY(out_done(c, xc, dx, nb));
        MIDAS_TRY(out_done(c, yc, dy, nb));
        MIDAS_TRY(out_done(c, zc, dz, nb));
    }
    return MIDAS_OK;
}

int midas_gpu_box_partition(midas_gpu_ctx *c, int n, const double *xc, const double *yc, const double *zc, int nx,
                            int ny, int nz, int *perm, int *blk_offsets, int *nblocks)
{
    if (!c || !xc || !yc || !zc || !perm || !blk_offsets || !nblocks) return MIDAS_ERR_ARG;
    c->err = Err();
    cudaSetDevice(c->device);
    const size_t b = sizeof(double) * (size_t)std::max(n, 0);
    const void *dx, *dy, *dz;
    MIDAS_TRY(to_device(c, xc, b, S_IN0, &dx));
    MIDAS_TRY(to_device(c, yc, b, S_IN1, &dy));
    MIDAS_TRY(to_device(c, zc, b, S_IN2, &dz));
    void *dp;
    MIDAS_TRY(out_buf(c, perm, sizeof(int) * (size_t)std::max(n, 1), S_OUT0, &dp));
    std::vector<int> offs((size_t)std::max(nx, 1) * std::max(ny, 1) * std::max(nz, 1) + 1);
    int nbk = 0;
    MIDAS_TRY(box_partition(c, n, (const double *)dx, (const double *)dy, (const double *)dz, nx, ny, nz, (int *)dp,
                            offs.data(), &nbk));
    MIDAS_TRY(out_done(c, perm, dp, sizeof(int) * (size_t)n));
    MIDAS_CUDA(c, cudaMemcpy(blk_offsets, offs.data(), sizeof(int) * (nbk + 1), cudaMemcpyDefault));
    *nblocks = nbk;
    return MIDAS_OK;
}

int midas_gpu_extend_blocks(midas_gpu_ctx *c, int n, const double *xc, const double *yc, const double *zc,
                            int nblocks, const int *blk_offsets, double ext_length, double sc, int *ext_offsets,
                            long long cap, int *ext_idx, long long *ntotal)
{
    if (!c || !xc || !yc || !zc || nblocks <= 0 || !blk_offsets || !ext_offsets || !ntotal) return MIDAS_ERR_ARG;
    c->err = Err();
    cudaSetDevice(c->device);
    std::vector<int> offs(nblocks + 1);
    MIDAS_CUDA(c, cudaMemcpy(offs.data(), blk_offsets, sizeof(int) * (nblocks + 1), cudaMemcpyDefault));
    for (auto &v : offs) v -= c->opts.index_base;
    if (offs[0] != 0 || offs[nblocks] != n) return c->err.set(MIDAS_ERR_ARG, "extend_blocks: offsets must cover n cells");
    for (int b = 0; b < nblocks; ++b)
        if (offs[b + 1] <= offs[b]) return c->err.set(MIDAS_ERR_ARG, "extend_blocks: empty or unordered block");
    const size_t b = sizeof(double) * (size_t)n;
    const void *dx, *dy, *dz;
    MIDAS_TRY(to_device(c, xc, b, S_IN0, &dx));
    MIDAS_TRY(to_device(c, yc, b, S_IN1, &dy));
    MIDAS_TRY(to_device(c, zc, b, S_IN2, &dz));
    const bool want = ext_idx && cap > 0;
    void *de = nullptr;
    if (want) MIDAS_TRY(out_buf(c, ext_idx, sizeof(int) * (size_t)cap, S_OUT0, &de));
    std::vector<int> eo(nblocks + 1);
    long long tot = 0;
    MIDAS_TRY(extend_blocks(c, n, (const double *)dx, (const double *)dy, (const double *)dz, nblocks, offs.data(),
                            ext_length, sc, eo.data(), want ? cap : 0, (int *)de, &tot));
    if (want) MIDAS_TRY(out_done(c, ext_idx, de, sizeof(int) * (size_t)std::min(tot, cap)));
    MIDAS_CUDA(c, cudaMemcpy(ext_offsets, eo.data(), sizeof(int) * (nblocks + 1), cudaMemcpyDefault));
    *ntotal = tot;
    return MIDAS_OK;
}

}  // extern "C"
