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

template int convert_cols<double, float>(const double *, long, float *, long, long, int,
                                         cudaStream_t);
template int convert_cols<float, double>(const float *, long, double *, long, long, int,
                                         cudaStream_t);
template int convert_cols<double, double>(const double *, long, double *, long, long, int,
                                          cudaStream_t);
template int swap_blocks<double>(double *, long, double *, long, long, int, cudaStream_t);
template int swap_blocks<float>(float *, long, float *, long, long, int, cudaStream_t);

}  // namespace sgpu
