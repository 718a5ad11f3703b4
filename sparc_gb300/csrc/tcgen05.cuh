// tcgen05 helpers (tensor memory, shared-memory matrix descriptors, MMA issue) for the
// library's tensor-core kernels. Layout facts these rely on, each checked on the GPU by the
// kernels' parity tests:
//  * a shared-memory operand without swizzle is a grid of core matrices of 8 rows x 16 bytes
//    (128 contiguous bytes); for a K-major operand the 8 rows are M (or N) indices and the
//    16 bytes hold 8 consecutive K values, for an MN-major operand the rows are K indices and
//    the 16 bytes hold 8 consecutive M (or N) values. In both cases the descriptor's leading
//    byte offset is the distance between core matrices adjacent in K and its stride byte
//    offset the distance between core matrices adjacent in M (or N);
//  * an M = 128 accumulator (cta_group::1) holds row i in TMEM lane i; an M = 64 accumulator
//    holds row i in lane (i mod 16) + 32 (i div 16), so a warp reading its 32-lane quarter q
//    finds rows 16 q .. 16 q + 15 in its lanes 0..15.
#pragma once

namespace sgpu {
namespace {

__device__ __forceinline__ unsigned tc_smem_u32(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor, no swizzle; lbo / sbo in bytes (multiples of 16); bit 46
// is the descriptor version of this architecture
__device__ __forceinline__ unsigned long long tc_desc(unsigned addr, unsigned lbo, unsigned sbo)
{
    return (unsigned long long)((addr & 0x3FFFFu) >> 4) |
           ((unsigned long long)(lbo >> 4) << 16) | ((unsigned long long)(sbo >> 4) << 32) |
           (1ull << 46);
}

// instruction descriptor of kind::f16 with FP32 accumulation and BF16 A and B; a_mn / b_mn
// select MN-major operands
__host__ __device__ constexpr unsigned tc_idesc_bf16(int M, int N, bool a_mn, bool b_mn)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) |
           ((b_mn ? 1u : 0u) << 16) | ((unsigned)(N >> 3) << 17) | ((unsigned)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma_bf16(unsigned tmem_d, unsigned long long adesc,
                                            unsigned long long bdesc, unsigned idesc,
                                            unsigned accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// arrive once on the barrier when every tcgen05.mma issued so far by this thread has completed
__device__ __forceinline__ void tc_commit(unsigned bar)
{
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
        : "memory");
}

__device__ __forceinline__ void tc_after_sync()
{
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void tc_before_sync()
{
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}
// generic-proxy shared-memory writes of this thread become visible to the tensor cores
__device__ __forceinline__ void tc_smem_to_async()
{
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// the whole warp allocates / frees `ncols` TMEM columns (a power of two >= 32)
__device__ __forceinline__ void tc_alloc(unsigned slot_smem, unsigned ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     slot_smem),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(unsigned taddr, unsigned ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr),
                 "r"(ncols)
                 : "memory");
}

// 32 consecutive 32-bit TMEM columns of this thread's lane (warp-collective)
__device__ __forceinline__ void tc_ld32(unsigned taddr, float *v)
{
    unsigned r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// 16 consecutive 32-bit TMEM columns of this thread's lane (warp-collective)
__device__ __forceinline__ void tc_ld16(unsigned taddr, float *v)
{
    unsigned r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace
}  // namespace sgpu
