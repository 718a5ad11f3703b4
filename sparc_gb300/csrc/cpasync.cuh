// cp.async (global -> shared) copies addressed by shared-space byte address, and their
// group waits, for the kernels that stage planes in shared-memory rings.
#pragma once

namespace sgpu {
namespace {

__device__ __forceinline__ void cp_async4s(unsigned sa, const void *gmem)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8s(unsigned sa, const void *gmem)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16s(unsigned sa, const void *gmem)  // L2 only
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.wait_all;\n" ::: "memory");
}

template <int N>
__device__ __forceinline__ void cp_async_wait_group()
{
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

}  // namespace
}  // namespace sgpu
