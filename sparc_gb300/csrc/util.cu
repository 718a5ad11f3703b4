// Elementwise helpers: precision conversion of column blocks and block exchange.
#include "sgpu_internal.h"

namespace sgpu {
namespace {

template <typename Tin, typename Tout>
__global__ void k_convert_cols(const Tin *__restrict__ src, long lds, Tout *__restrict__ dst,
                               long ldd, long rows, long total)
{
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total;
         t += (long)gridDim.x * blockDim.x) {
        const long n = t / rows, i = t - n * rows;
        dst[n * ldd + i] = (Tout)src[n * lds + i];
    }
}

template <typename T>
__global__ void k_swap_cols(T *__restrict__ a, long lda, T *__restrict__ b, long ldb, long rows,
                            long total)
{
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total;
         t += (long)gridDim.x * blockDim.x) {
        const long n = t / rows, i = t - n * rows;
        const T va = a[n * lda + i];
        a[n * lda + i] = b[n * ldb + i];
        b[n * ldb + i] = va;
    }
}

// FP64 FMA issue rate: 16 independent FMA chains per thread, iters steps each (unrolled by
// 4, so loop control is a small share of the issue slots). The result is stored only when it
// equals a value no chain reaches, so the stores never happen but the compiler must keep the
// arithmetic.
__global__ void __launch_bounds__(256) k_fp64_fma_rate(double seed, int iters, double *sink)
{
    constexpr int C = 16;
    double a[C];
#pragma unroll
    for (int c = 0; c < C; c++) a[c] = seed + threadIdx.x * 1e-7 + c * 1e-3;
    const double m = 0.999999, d = 1e-9;
#pragma unroll 4
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int c = 0; c < C; c++) a[c] = fma(a[c], m, d);
    }
    double t = 0.0;
#pragma unroll
    for (int c = 0; c < C; c++) t += a[c];
    if (t == -1.2345e300) sink[0] = t;
}

inline int grid_for(long total)
{
    long g = (total + 255) / 256;
    if (g > 152L * 32) g = 152L * 32;
    return (int)(g > 0 ? g : 1);
}

}  // namespace

template <typename Tin, typename Tout>
int convert_cols(const Tin *src, long lds, Tout *dst, long ldd, long rows, int ncol,
                 cudaStream_t st)
{
    const long total = rows * (long)ncol;
    if (total <= 0) return SGPU_OK;
    k_convert_cols<Tin, Tout><<<grid_for(total), 256, 0, st>>>(src, lds, dst, ldd, rows, total);
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

template <typename T>
int swap_blocks(T *a, long lda, T *b, long ldb, long rows, int ncol, cudaStream_t st)
{
    const long total = rows * (long)ncol;
    if (total <= 0) return SGPU_OK;
    k_swap_cols<T><<<grid_for(total), 256, 0, st>>>(a, lda, b, ldb, rows, total);
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

// Measured FP64 FMA rate of this GPU in TFLOP/s (2 flops per FMA), timed with CUDA events on
// the context stream: the ceiling of FP64 kernels that are bound by the FP64 pipe.
int fp64_fma_rate(sgpu_ctx *ctx, double *tflops)
{
    int nsm = 0;
    SGPU_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
    double *sink = nullptr;
    SGPU_TRY(ws_get(ctx, WS_MISC, sizeof(double), (void **)&sink));
    const int blocks = nsm * 8, threads = 256, iters = 1 << 13;
    cudaEvent_t e0, e1;
    SGPU_CUDA_TRY(cudaEventCreate(&e0));
    SGPU_CUDA_TRY(cudaEventCreate(&e1));
    k_fp64_fma_rate<<<blocks, threads, 0, ctx->stream>>>(1.0, 256, sink);  // warm-up
    SGPU_CUDA_TRY(cudaEventRecord(e0, ctx->stream));
    k_fp64_fma_rate<<<blocks, threads, 0, ctx->stream>>>(1.0, iters, sink);
    SGPU_CUDA_TRY(cudaEventRecord(e1, ctx->stream));
    SGPU_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    SGPU_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    SGPU_CUDA_TRY(cudaGetLastError());
    *tflops = 2.0 * 16.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
    return SGPU_OK;
}

template int convert_cols<double, float>(const double *, long, float *, long, long, int,
                                         cudaStream_t);
template int convert_cols<float, double>(const float *, long, double *, long, long, int,
                                         cudaStream_t);
template int convert_cols<double, double>(const double *, long, double *, long, long, int,
                                          cudaStream_t);
template int swap_blocks<double>(double *, long, double *, long, long, int, cudaStream_t);
template int swap_blocks<float>(float *, long, float *, long, long, int, cudaStream_t);

}  // namespace sgpu
