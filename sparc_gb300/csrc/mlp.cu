// Learned initial density: per-grid-point descriptors of the atomic environment and a small
// multilayer perceptron (BF16 weights, FP32 accumulation) with forward, backward and Adam
// kernels, so that the network is trained and evaluated on the device.
//
// No counterpart in the reference, which starts every SCF from the superposition of atomic
// densities (Init_electronDensity, src/orbitalElecDensInit.c:145, electronDens_at from
// Generate_PseudoChargeDensity, src/electrostatics.c:1005-1034). The network predicts the
// correction rho_SCF - rho_at; the caller adds it to rho_at, clips negative values and
// restores the electron count.
//
// Descriptors (24 per point): for 8 Gaussian radial bins g_b(r) = exp(-(r - mu_b)^2 / 2w^2)
// times a cosine cut-off at rcut, over all atom images within rcut of the point,
//   s_b  = sum_a g_b(r_a)                                   (l = 0)
//   p1_b = |sum_a g_b(r_a) r_a / r_a|^2                     (l = 1, rotation invariant)
//   p2_b = sum_m (sum_a g_b(r_a) Y_2m(r_a / r_a))^2         (l = 2, rotation invariant)
//
// Network: x (24, normalised by a per-feature shift and scale) -> 3 hidden layers of `width`
// with SiLU -> 1 output. Parameters are kept in FP32 (master copy, Adam moments) and used by
// the forward and backward GEMMs as BF16; activations and all sums are FP32.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "sgpu_internal.h"

struct sgpu_mlp {
    int device = 0;
    cudaStream_t stream = nullptr;
    int nin = 0, width = 0;
    long nparam = 0;
    long off_w[4] = {0, 0, 0, 0}, off_b[4] = {0, 0, 0, 0};  // layers 1..3 and the output
    float *master = nullptr, *grad = nullptr, *m1 = nullptr, *m2 = nullptr;
    __nv_bfloat16 *wbf = nullptr;
    float *shift = nullptr, *scale = nullptr;  // input normalisation (nin each)
    float *work = nullptr;                     // activations of the current batch
    size_t work_elems = 0;
    float *part = nullptr;                     // per-block partial weight gradients
    size_t part_elems = 0;
    double *lossbuf = nullptr;
    int step = 0;
};

namespace sgpu {
namespace {

constexpr int kBins = 8;
constexpr int kDesc = 3 * kBins;

struct DescImage {
    double x, y, z;
};

// one thread per grid point
__global__ void __launch_bounds__(256)
    k_descriptors(const DescImage *__restrict__ img, int nimg, int Nx, int Ny, int Nz, double hx,
                  double hy, double hz, double rcut, double width, float *__restrict__ out)
{
    const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long Nd = (long)Nx * Ny * Nz;
    if (p >= Nd) return;
    const int i = (int)(p % Nx), j = (int)((p / Nx) % Ny), k = (int)(p / ((long)Nx * Ny));
    const double px = i * hx, py = j * hy, pz = k * hz;
    float s[kBins], v1[kBins][3], v2[kBins][5];
#pragma unroll
    for (int b = 0; b < kBins; b++) {
        s[b] = 0.f;
        v1[b][0] = v1[b][1] = v1[b][2] = 0.f;
        v2[b][0] = v2[b][1] = v2[b][2] = v2[b][3] = v2[b][4] = 0.f;
    }
    const double rc2 = rcut * rcut;
    const double pi = 3.14159265358979323846;
    const float c2a = (float)(0.5 * sqrt(15.0 / pi)), c2b = (float)(0.25 * sqrt(5.0 / pi)),
                c2c = (float)(0.25 * sqrt(15.0 / pi));
    for (int a = 0; a < nimg; a++) {
        const double dx = img[a].x - px, dy = img[a].y - py, dz = img[a].z - pz;
        const double r2 = dx * dx + dy * dy + dz * dz;
        if (r2 >= rc2) continue;
        const double r = sqrt(r2);
        const float fc = (float)(0.5 * (cos(pi * r / rcut) + 1.0));
        const float ir = r > 1e-8 ? (float)(1.0 / r) : 0.f;
        const float ux = (float)dx * ir, uy = (float)dy * ir, uz = (float)dz * ir;
        const float y2[5] = {c2a * ux * uy, c2a * uy * uz, c2b * (2.f * uz * uz - ux * ux - uy * uy),
                             c2a * uz * ux, c2c * (ux * ux - uy * uy)};
#pragma unroll
        for (int b = 0; b < kBins; b++) {
            const double mu = rcut * b / (kBins - 1);
            const double t = (r - mu) / width;
            const float g = fc * (float)exp(-0.5 * t * t);
            s[b] += g;
            v1[b][0] += g * ux; v1[b][1] += g * uy; v1[b][2] += g * uz;
#pragma unroll
            for (int q = 0; q < 5; q++) v2[b][q] += g * y2[q];
        }
    }
    float *o = out + p * kDesc;
#pragma unroll
    for (int b = 0; b < kBins; b++) {
        o[b] = s[b];
        o[kBins + b] = v1[b][0] * v1[b][0] + v1[b][1] * v1[b][1] + v1[b][2] * v1[b][2];
        float t = 0.f;
#pragma unroll
        for (int q = 0; q < 5; q++) t += v2[b][q] * v2[b][q];
        o[2 * kBins + b] = t;
    }
}

// ---------------------------------------------------------------------------- GEMMs
// C[n x N] = op(A)[n x K] * op(B)[K x N] (+ bias), A FP32 row-major (lda), B BF16 weights.
// TB = false: B[k][j] = W[k * N + j] (forward: W is K x N). TB = true: B[k][j] = W[j * K + k]
// (backward data: the transpose of an N x K weight). 64 x 64 output tile per block, 256
// threads with 4 x 4 micro-tiles, K in chunks of 16 through shared memory.
constexpr int GT = 64, GK = 16;

template <bool TB>
__global__ void __launch_bounds__(256)
    k_gemm_aw(const float *__restrict__ A, long lda, const __nv_bfloat16 *__restrict__ W,
              const float *__restrict__ bias, float *__restrict__ C, long ldc, long n, int K,
              int N, const float *__restrict__ shift, const float *__restrict__ scale)
{
    __shared__ float As[GK][GT + 4];
    __shared__ float Bs[GK][GT + 4];
    const int tid = threadIdx.x;
    const int tr = tid / 16, tc = tid % 16;  // 16 x 16 threads, 4 x 4 each
    const long r0 = (long)blockIdx.x * GT;
    const int c0 = blockIdx.y * GT;
    float acc[4][4] = {{0}};
    for (int k0 = 0; k0 < K; k0 += GK) {
        // A tile: 64 rows x 16 k
        for (int e = tid; e < GT * GK; e += 256) {
            const int rr = e / GK, kk = e % GK;
            const long row = r0 + rr;
            const int kc = k0 + kk;
            float v = 0.f;
            if (row < n && kc < K) {
                v = A[row * lda + kc];
                if (shift) v = (v - shift[kc]) * scale[kc];
            }
            As[kk][rr] = v;
        }
        // B tile: 16 k x 64 cols
        for (int e = tid; e < GK * GT; e += 256) {
            const int kk = e / GT, cc = e % GT;
            const int kc = k0 + kk, col = c0 + cc;
            float v = 0.f;
            if (kc < K && col < N)
                v = __bfloat162float(TB ? W[(long)col * K + kc] : W[(long)kc * N + col]);
            Bs[kk][cc] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; kk++) {
            float a[4], b[4];
#pragma unroll
            for (int q = 0; q < 4; q++) { a[q] = As[kk][tr * 4 + q]; b[q] = Bs[kk][tc * 4 + q]; }
#pragma unroll
            for (int x = 0; x < 4; x++)
#pragma unroll
                for (int y = 0; y < 4; y++) acc[x][y] = fmaf(a[x], b[y], acc[x][y]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int x = 0; x < 4; x++) {
        const long row = r0 + tr * 4 + x;
        if (row >= n) continue;
#pragma unroll
        for (int y = 0; y < 4; y++) {
            const int col = c0 + tc * 4 + y;
            if (col < N) C[row * ldc + col] = acc[x][y] + (bias ? bias[col] : 0.f);
        }
    }
}

// weight gradient partials: P[blk][K x N] = sum over this block's rows of A[r][k] * D[r][j]
// (A FP32 n x K, D FP32 n x N); bias partials in the extra row P[blk][K][*] = sum D[r][j].
// 256 threads, each owns (K+1) * N / 256 outputs.
__global__ void __launch_bounds__(256)
    k_wgrad_partial(const float *__restrict__ A, long lda, const float *__restrict__ D, long ldd,
                    long n, int K, int N, long rows_per_block, float *__restrict__ P,
                    const float *__restrict__ shift, const float *__restrict__ scale)
{
    const long rs = (long)blockIdx.x * rows_per_block;
    const long re = min(n, rs + rows_per_block);
    const int tot = (K + 1) * N;
    float *out = P + (long)blockIdx.x * tot;
    for (int o = threadIdx.x; o < tot; o += blockDim.x) {
        const int k = o / N, j = o % N;
        float s = 0.f;
        if (k < K) {
            const float sh = shift ? shift[k] : 0.f, sc = shift ? scale[k] : 1.f;
            for (long r = rs; r < re; r++) {
                float a = A[r * lda + k];
                if (shift) a = (a - sh) * sc;
                s = fmaf(a, D[r * ldd + j], s);
            }
        } else {
            for (long r = rs; r < re; r++) s += D[r * ldd + j];
        }
        out[o] = s;
    }
}

// sum the partials of nblk blocks into the gradient (weights, then bias)
__global__ void k_wgrad_reduce(const float *__restrict__ P, int nblk, int K, int N,
                               float *__restrict__ gw, float *__restrict__ gb)
{
    const int tot = (K + 1) * N;
    for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < tot; o += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < nblk; b++) s += P[(long)b * tot + o];
        if (o < K * N) gw[o] += s; else gb[o - K * N] += s;
    }
}

__device__ __forceinline__ float sigm(float z) { return 1.f / (1.f + expf(-z)); }

// H = silu(Z) in place of a copy: Z kept for the backward pass
__global__ void k_silu(const float *__restrict__ Z, float *__restrict__ H, long n)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float z = Z[i];
        H[i] = z * sigm(z);
    }
}

// dZ = dH * silu'(Z)
__global__ void k_silu_back(const float *__restrict__ Z, float *__restrict__ dH, long n)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float z = Z[i], s = sigm(z);
        dH[i] *= s * (1.f + z * (1.f - s));
    }
}

// output layer: y = H . w + b (one warp per row); with a target, also loss sum and dY
__global__ void k_out_layer(const float *__restrict__ H, int width, long n,
                            const __nv_bfloat16 *__restrict__ w, const float *__restrict__ b,
                            float *__restrict__ y, const float *__restrict__ target,
                            float tscale, float *__restrict__ dy, double *__restrict__ loss)
{
    const long row = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    float s = 0.f;
    for (int j = lane; j < width; j += 32) s = fmaf(H[row * width + j], __bfloat162float(w[j]), s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) {
        s += b[0];
        if (y) y[row] = s;
        if (target) {
            const float r = s - target[row] * tscale;
            dy[row] = 2.f * r / (float)n;
            atomicAdd(loss, (double)r * r);
        }
    }
}

// dH[r][j] = dy[r] * w[j]
__global__ void k_out_back(const float *__restrict__ dy, const __nv_bfloat16 *__restrict__ w,
                           int width, long n, float *__restrict__ dH)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n * width; i += (long)gridDim.x * blockDim.x)
        dH[i] = dy[i / width] * __bfloat162float(w[i % width]);
}

// Adam with bias correction; refreshes the BF16 copy
__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m1,
                       float *__restrict__ m2, __nv_bfloat16 *__restrict__ pb, long n, float lr,
                       float b1, float b2, float eps, float c1, float c2)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float a = b1 * m1[i] + (1.f - b1) * gi;
        const float v = b2 * m2[i] + (1.f - b2) * gi * gi;
        m1[i] = a;
        m2[i] = v;
        const float upd = lr * (a / c1) / (sqrtf(v / c2) + eps);
        p[i] -= upd;
        pb[i] = __float2bfloat16(p[i]);
    }
}

__global__ void k_to_bf16(const float *__restrict__ p, __nv_bfloat16 *__restrict__ pb, long n)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        pb[i] = __float2bfloat16(p[i]);
}

int grid_for(long n) { return (int)std::max(1L, std::min((n + 255) / 256, 152L * 16)); }

}  // namespace

// activations of a batch of n rows: Z1 H1 Z2 H2 Z3 H3 (n x width each), y, dy (n)
static int mlp_work(sgpu_mlp *net, long n, float **Z, float **H, float **y, float **dy)
{
    const size_t need = (size_t)n * net->width * 6 + 2 * (size_t)n;
    if (need > net->work_elems) {
        if (net->work) cudaFree(net->work);
        net->work = nullptr;
        net->work_elems = 0;
        SGPU_CUDA_TRY(cudaMalloc(&net->work, sizeof(float) * need));
        net->work_elems = need;
    }
    const size_t L = (size_t)n * net->width;
    for (int l = 0; l < 3; l++) {
        Z[l] = net->work + (2 * l) * L;
        H[l] = net->work + (2 * l + 1) * L;
    }
    *y = net->work + 6 * L;
    *dy = *y + n;
    return SGPU_OK;
}

static int mlp_forward(sgpu_mlp *net, const float *x, long n, float **Z, float **H, float *y,
                       const float *target, float tscale, float *dy)
{
    cudaStream_t st = net->stream;
    const int W = net->width;
    const __nv_bfloat16 *wb = net->wbf;
    const float *b = net->master;
    for (int l = 0; l < 3; l++) {
        const float *in = l == 0 ? x : H[l - 1];
        const int K = l == 0 ? net->nin : W;
        dim3 g((unsigned)((n + GT - 1) / GT), (unsigned)((W + GT - 1) / GT));
        k_gemm_aw<false><<<g, 256, 0, st>>>(in, K, wb + net->off_w[l], b + net->off_b[l], Z[l], W,
                                            n, K, W, l == 0 ? net->shift : nullptr,
                                            l == 0 ? net->scale : nullptr);
        k_silu<<<grid_for(n * W), 256, 0, st>>>(Z[l], H[l], n * W);
    }
    k_out_layer<<<(unsigned)((n * 32 + 255) / 256), 256, 0, st>>>(
        H[2], W, n, wb + net->off_w[3], b + net->off_b[3], y, target, tscale, dy, net->lossbuf);
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

static int wgrad(sgpu_mlp *net, const float *A, int K, const float *D, int N, long n,
                 float *gw, float *gb, const float *shift, const float *scale)
{
    cudaStream_t st = net->stream;
    const int nblk = (int)std::min<long>(304, std::max<long>(1, (n + 255) / 256));
    const long rpb = (n + nblk - 1) / nblk;
    const size_t need = (size_t)nblk * (K + 1) * N;
    if (need > net->part_elems) {
        if (net->part) cudaFree(net->part);
        net->part = nullptr;
        net->part_elems = 0;
        SGPU_CUDA_TRY(cudaMalloc(&net->part, sizeof(float) * need));
        net->part_elems = need;
    }
    k_wgrad_partial<<<nblk, 256, 0, st>>>(A, K, D, N, n, K, N, rpb, net->part, shift, scale);
    k_wgrad_reduce<<<grid_for((long)(K + 1) * N), 256, 0, st>>>(net->part, nblk, K, N, gw, gb);
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

}  // namespace sgpu

using namespace sgpu;

extern "C" {

int sgpu_density_descriptors(sgpu_ctx *ctx, const double *cell, int n_atom,
                             const double *atom_pos, double rcut, double width, float *desc)
{
    if (!ctx || !cell || n_atom < 0 || (n_atom > 0 && !atom_pos) || !(rcut > 0) ||
        !(width > 0) || !desc || !is_device_ptr(desc)) {
        set_error("sgpu_density_descriptors: bad arguments (desc must be device memory)");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    // atom images within rcut of the cell
    std::vector<DescImage> im;
    for (int a = 0; a < n_atom; a++) {
        const double *p = atom_pos + 3 * a;
        int lo[3], hi[3];
        for (int d = 0; d < 3; d++) {
            lo[d] = (int)std::floor((-rcut - p[d]) / cell[d]);
            hi[d] = (int)std::ceil((cell[d] + rcut - p[d]) / cell[d]);
        }
        for (int r = lo[2]; r <= hi[2]; r++)
            for (int q = lo[1]; q <= hi[1]; q++)
                for (int s = lo[0]; s <= hi[0]; s++) {
                    const double x = p[0] + s * cell[0], y = p[1] + q * cell[1],
                                 z = p[2] + r * cell[2];
                    if (x < -rcut || x > cell[0] + rcut || y < -rcut || y > cell[1] + rcut ||
                        z < -rcut || z > cell[2] + rcut)
                        continue;
                    im.push_back(DescImage{x, y, z});
                }
    }
    DescImage *dimg = nullptr;
    cudaStream_t st = ctx->stream;
    if (!im.empty()) {
        SGPU_CUDA_TRY(cudaMallocAsync(&dimg, sizeof(DescImage) * im.size(), st));
        SGPU_CUDA_TRY(cudaMemcpyAsync(dimg, im.data(), sizeof(DescImage) * im.size(),
                                      cudaMemcpyHostToDevice, st));
    }
    k_descriptors<<<(unsigned)((ctx->Nd + 255) / 256), 256, 0, st>>>(
        dimg, (int)im.size(), ctx->Nx, ctx->Ny, ctx->Nz, cell[0] / ctx->Nx, cell[1] / ctx->Ny,
        cell[2] / ctx->Nz, rcut, width, desc);
    ctx->launches++;
    const cudaError_t e = cudaGetLastError();
    if (dimg) cudaFreeAsync(dimg, st);
    SGPU_CUDA_TRY(e);
    SGPU_CUDA_TRY(cudaStreamSynchronize(st));
    return SGPU_OK;
}

int sgpu_mlp_create(int device, int nin, int width, unsigned long long seed, sgpu_mlp **out)
{
    if (!out || nin < 1 || width < 1 || width > 1024) {
        set_error("sgpu_mlp_create: bad arguments");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(device));
    auto *net = new sgpu_mlp();
    net->device = device;
    net->nin = nin;
    net->width = width;
    long off = 0;
    const int fan_in[4] = {nin, width, width, width}, fan_out[4] = {width, width, width, 1};
    for (int l = 0; l < 4; l++) {
        net->off_w[l] = off;
        off += (long)fan_in[l] * fan_out[l];
        net->off_b[l] = off;
        off += fan_out[l];
    }
    net->nparam = off;
    // He-style uniform initialisation from a splitmix64 stream, biases zero
    std::vector<float> p(off, 0.f);
    unsigned long long z = seed;
    auto next = [&]() {
        z += 0x9E3779B97F4A7C15ull;
        unsigned long long t = z;
        t = (t ^ (t >> 30)) * 0xBF58476D1CE4E5B9ull;
        t = (t ^ (t >> 27)) * 0x94D049BB133111EBull;
        t ^= t >> 31;
        return (double)(t >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < 4; l++) {
        const double lim = std::sqrt(6.0 / fan_in[l]) * (l == 3 ? 0.1 : 1.0);
        for (long i = 0; i < (long)fan_in[l] * fan_out[l]; i++)
            p[net->off_w[l] + i] = (float)((2.0 * next() - 1.0) * lim);
    }
    bool ok = cudaStreamCreateWithFlags(&net->stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaMalloc(&net->master, sizeof(float) * off) == cudaSuccess &&
              cudaMalloc(&net->grad, sizeof(float) * off) == cudaSuccess &&
              cudaMalloc(&net->m1, sizeof(float) * off) == cudaSuccess &&
              cudaMalloc(&net->m2, sizeof(float) * off) == cudaSuccess &&
              cudaMalloc(&net->wbf, sizeof(__nv_bfloat16) * off) == cudaSuccess &&
              cudaMalloc(&net->shift, sizeof(float) * nin) == cudaSuccess &&
              cudaMalloc(&net->scale, sizeof(float) * nin) == cudaSuccess &&
              cudaMalloc(&net->lossbuf, sizeof(double)) == cudaSuccess;
    std::vector<float> zero(nin, 0.f), one(nin, 1.f);
    ok = ok && cudaMemcpy(net->master, p.data(), sizeof(float) * off, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemset(net->grad, 0, sizeof(float) * off) == cudaSuccess &&
         cudaMemset(net->m1, 0, sizeof(float) * off) == cudaSuccess &&
         cudaMemset(net->m2, 0, sizeof(float) * off) == cudaSuccess &&
         cudaMemcpy(net->shift, zero.data(), sizeof(float) * nin, cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(net->scale, one.data(), sizeof(float) * nin, cudaMemcpyHostToDevice) == cudaSuccess;
    if (ok) {
        k_to_bf16<<<grid_for(off), 256, 0, net->stream>>>(net->master, net->wbf, off);
        ok = cudaStreamSynchronize(net->stream) == cudaSuccess;
    }
    if (!ok) {
        sgpu_mlp_destroy(net);
        set_error("sgpu_mlp_create: device allocation failed");
        return SGPU_ERR_NOMEM;
    }
    *out = net;
    return SGPU_OK;
}

int sgpu_mlp_destroy(sgpu_mlp *net)
{
    if (!net) return SGPU_OK;
    cudaSetDevice(net->device);
    if (net->stream) cudaStreamSynchronize(net->stream);
    for (void *p : {(void *)net->master, (void *)net->grad, (void *)net->m1, (void *)net->m2,
                    (void *)net->wbf, (void *)net->shift, (void *)net->scale, (void *)net->work,
                    (void *)net->part, (void *)net->lossbuf})
        if (p) cudaFree(p);
    if (net->stream) cudaStreamDestroy(net->stream);
    delete net;
    return SGPU_OK;
}

int sgpu_mlp_nparam(sgpu_mlp *net, long *nparam)
{
    if (!net || !nparam) {
        set_error("sgpu_mlp_nparam: bad arguments");
        return SGPU_ERR_ARG;
    }
    *nparam = net->nparam;
    return SGPU_OK;
}

// which = 0 parameters (FP32 master), 1 gradient, 2 input shift, 3 input scale (host arrays)
int sgpu_mlp_get(sgpu_mlp *net, int which, float *out)
{
    if (!net || !out || which < 0 || which > 3) {
        set_error("sgpu_mlp_get: bad arguments");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(net->device));
    const float *src[4] = {net->master, net->grad, net->shift, net->scale};
    const long n = which < 2 ? net->nparam : net->nin;
    SGPU_CUDA_TRY(cudaMemcpyAsync(out, src[which], sizeof(float) * n, cudaMemcpyDeviceToHost,
                                  net->stream));
    SGPU_CUDA_TRY(cudaStreamSynchronize(net->stream));
    return SGPU_OK;
}

int sgpu_mlp_set(sgpu_mlp *net, int which, const float *in)
{
    if (!net || !in || which < 0 || which > 3 || which == 1) {
        set_error("sgpu_mlp_set: bad arguments (0 parameters, 2 shift, 3 scale)");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(net->device));
    float *dst[4] = {net->master, nullptr, net->shift, net->scale};
    const long n = which < 2 ? net->nparam : net->nin;
    SGPU_CUDA_TRY(cudaMemcpyAsync(dst[which], in, sizeof(float) * n, cudaMemcpyHostToDevice,
                                  net->stream));
    if (which == 0) k_to_bf16<<<grid_for(n), 256, 0, net->stream>>>(net->master, net->wbf, n);
    SGPU_CUDA_TRY(cudaStreamSynchronize(net->stream));
    return SGPU_OK;
}

int sgpu_mlp_forward(sgpu_mlp *net, const float *x, long n, float *y)
{
    if (!net || !x || !y || n < 0 || !is_device_ptr(x) || !is_device_ptr(y)) {
        set_error("sgpu_mlp_forward: bad arguments (x, y device memory)");
        return SGPU_ERR_ARG;
    }
    if (n == 0) return SGPU_OK;
    SGPU_CUDA_TRY(cudaSetDevice(net->device));
    float *Z[3], *H[3], *yy, *dy;
    SGPU_TRY(mlp_work(net, n, Z, H, &yy, &dy));
    SGPU_TRY(mlp_forward(net, x, n, Z, H, y, nullptr, 0.f, nullptr));
    SGPU_CUDA_TRY(cudaStreamSynchronize(net->stream));
    return SGPU_OK;
}

// Mean-squared-error loss of the batch against target * tscale, and its gradient added to the
// accumulated gradient (zeroed by sgpu_mlp_zero_grad).
int sgpu_mlp_loss_grad(sgpu_mlp *net, const float *x, const float *target, long n, float tscale,
                       double *loss)
{
    if (!net || !x || !target || n <= 0 || !is_device_ptr(x) || !is_device_ptr(target)) {
        set_error("sgpu_mlp_loss_grad: bad arguments (x, target device memory, n > 0)");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(net->device));
    cudaStream_t st = net->stream;
    float *Z[3], *H[3], *y, *dy;
    SGPU_TRY(mlp_work(net, n, Z, H, &y, &dy));
    SGPU_CUDA_TRY(cudaMemsetAsync(net->lossbuf, 0, sizeof(double), st));
    SGPU_TRY(mlp_forward(net, x, n, Z, H, y, target, tscale, dy));
    const int W = net->width;
    float *g = net->grad;
    // output layer: grad w4 = sum dy H3, grad b4 = sum dy; dH3 = dy w4 (into Z... use H slots)
    SGPU_TRY(wgrad(net, H[2], W, dy, 1, n, g + net->off_w[3], g + net->off_b[3], nullptr, nullptr));
    // dH3 overwrites H[2] after its last use
    k_out_back<<<grid_for(n * W), 256, 0, st>>>(dy, net->wbf + net->off_w[3], W, n, H[2]);
    for (int l = 2; l >= 0; l--) {
        // dZ_l = dH_l * silu'(Z_l), in H[l]
        k_silu_back<<<grid_for(n * W), 256, 0, st>>>(Z[l], H[l], n * W);
        const float *in = l == 0 ? x : H[l - 1];
        const int K = l == 0 ? net->nin : W;
        // weight gradient needs H[l-1] (activations): computed before H[l-1] becomes dH[l-1]
        if (l > 0) {
            // recompute H[l-1] = silu(Z[l-1]) is not needed: H[l-1] still holds activations
        }
        SGPU_TRY(wgrad(net, in, K, H[l], W, n, g + net->off_w[l], g + net->off_b[l],
                       l == 0 ? net->shift : nullptr, l == 0 ? net->scale : nullptr));
        if (l > 0) {
            // dH_{l-1} = dZ_l W_l^T, written over H[l-1] (its activations are no longer needed)
            dim3 gg((unsigned)((n + GT - 1) / GT), (unsigned)((W + GT - 1) / GT));
            k_gemm_aw<true><<<gg, 256, 0, st>>>(H[l], W, net->wbf + net->off_w[l], nullptr,
                                                H[l - 1], W, n, W, W, nullptr, nullptr);
        }
    }
    SGPU_CUDA_TRY(cudaGetLastError());
    double hl = 0.0;
    SGPU_CUDA_TRY(cudaMemcpyAsync(&hl, net->lossbuf, sizeof(double), cudaMemcpyDeviceToHost, st));
    SGPU_CUDA_TRY(cudaStreamSynchronize(st));
    if (loss) *loss = hl / (double)n;
    return SGPU_OK;
}

int sgpu_mlp_zero_grad(sgpu_mlp *net)
{
    if (!net) {
        set_error("sgpu_mlp_zero_grad: null network");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(net->device));
    SGPU_CUDA_TRY(cudaMemsetAsync(net->grad, 0, sizeof(float) * net->nparam, net->stream));
    return SGPU_OK;
}

int sgpu_mlp_adam_step(sgpu_mlp *net, float lr, float beta1, float beta2, float eps)
{
    if (!net || !(lr > 0)) {
        set_error("sgpu_mlp_adam_step: bad arguments");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(net->device));
    net->step++;
    const float c1 = 1.f - std::pow(beta1, (float)net->step);
    const float c2 = 1.f - std::pow(beta2, (float)net->step);
    k_adam<<<grid_for(net->nparam), 256, 0, net->stream>>>(net->master, net->grad, net->m1,
                                                           net->m2, net->wbf, net->nparam, lr,
                                                           beta1, beta2, eps, c1, c2);
    SGPU_CUDA_TRY(cudaGetLastError());
    SGPU_CUDA_TRY(cudaStreamSynchronize(net->stream));
    return SGPU_OK;
}

}  // extern "C"
