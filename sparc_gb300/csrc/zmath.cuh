// Complex helpers for the k-point kernels (interleaved re, im: double2 for complex128, float2
// for complex64) and the index helpers of the periodic tile loaders.
#pragma once

#include <cuda_runtime.h>

namespace sgpu {
namespace zm {

template <typename CT> struct Real;
template <> struct Real<double2> { using type = double; };
template <> struct Real<float2> { using type = float; };

template <typename CT>
__device__ __forceinline__ CT cmul(CT a, CT b)
{
    return CT{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename CT>
__device__ __forceinline__ CT cadd(CT a, CT b) { return CT{a.x + b.x, a.y + b.y}; }
template <typename CT, typename R>
__device__ __forceinline__ CT cscale(CT a, R s) { return CT{a.x * s, a.y * s}; }

__device__ __forceinline__ int wrapz(int i, int n)
{
    i %= n;
    return i < 0 ? i + n : i;
}
__device__ __forceinline__ int floordiv(int i, int n)
{
    return i >= 0 ? i / n : -((-i + n - 1) / n);
}

// e^{i theta} in the block's precision (the angle is formed in FP64)
template <typename CT>
__device__ __forceinline__ CT phase(double theta)
{
    double s, c;
    sincos(theta, &s, &c);
    using R = typename Real<CT>::type;
    return CT{(R)c, (R)s};
}

}  // namespace zm
}  // namespace sgpu
