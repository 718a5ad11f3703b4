// Shared-memory barrier (mbarrier) and bulk-copy helpers for kernels that stage data with
// asynchronous copies. Every wait is bounded: a wait that runs out returns false instead of
// spinning forever, and the caller records it in the context's status word and winds down.
#pragma once

namespace sgpu {
namespace {

constexpr long long kWaitCycles = 2000000000LL;  // bound of one barrier wait (SM cycles)

__device__ __forceinline__ void mbar_init(unsigned a, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned a)
{
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(a)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(unsigned a, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(a), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned a, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                 " selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok)
                 : "r"(a), "r"(parity)
                 : "memory");
    return ok != 0;
}
// the bounded spin after a failed first test, kept out of line so that the unrolled plane loop
// holds one try_wait per wait site
__device__ __noinline__ bool mbar_wait_slow(unsigned a, unsigned parity, long long limit)
{
    const long long t0 = clock64();
#pragma unroll 1
    for (;;) {
#pragma unroll 1
        for (int i = 0; i < 64; i++)
            if (mbar_test(a, parity)) return true;
        if (clock64() - t0 > limit) return false;
    }
}
// wait for the completion of the phase of parity `parity`; false once `limit` SM cycles
// have passed
__device__ __forceinline__ bool mbar_wait_bounded(unsigned a, unsigned parity,
                                                  long long limit = kWaitCycles)
{
    return mbar_test(a, parity) || mbar_wait_slow(a, parity, limit);
}

// the same wait with the waiting warp suspended inside try_wait (up to suspend_ns per try)
// instead of spinning: for waits on long asynchronous work (tensor-core MMAs), where spinning
// warps would take issue slots from the warps doing the other work of the SM
__device__ __forceinline__ bool mbar_test_suspend(unsigned a, unsigned parity, unsigned suspend_ns)
{
    unsigned ok;
    asm volatile("{\n .reg .pred p;\n"
                 " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
                 " selp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok)
                 : "r"(a), "r"(parity), "r"(suspend_ns)
                 : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool mbar_wait_suspend(unsigned a, unsigned parity,
                                                  long long limit = kWaitCycles)
{
    if (mbar_test_suspend(a, parity, 100000u)) return true;
    const long long t0 = clock64();
#pragma unroll 1
    while (!mbar_test_suspend(a, parity, 100000u))
        if (clock64() - t0 > limit) return false;
    return true;
}

__device__ __forceinline__ void bulk_g2s(unsigned dst, const void *src, unsigned bytes,
                                         unsigned mbar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes"
                 " [%0], [%1], %2, [%3];\n" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}

}  // namespace
}  // namespace sgpu
