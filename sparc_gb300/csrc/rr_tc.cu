// Rayleigh-Ritz products on the tensor cores (tcgen05): FP64- or FP32-accurate GEMMs from
// BF16 slices with exact fixed-point accumulation.
//
// The products of the Rayleigh-Ritz step, Mp = Yᵀ Y and Hp = Yᵀ (H Y) of DP_Project_Hamiltonian
// (src/eigenSolver.c:1022-1033) and X = Y Q of DP_Subspace_Rotation (src/eigenSolver.c:1415),
// are FP64 GEMMs in the reference. Here each operand row (the K-vector of one output row or
// column) is scaled by a power of two so that its entries lie in (-1, 1), and every entry is
// written as a sum of NS slices with 7 significant bits each,
//     u = sum_i S_i 2^(-7(i+1)),  S_0 in [-128, 128], S_i in [-64, 64] (i > 0),
// each slice stored as an exact BF16 number (its own power of two included). A product u v is
// the sum over slice pairs (i, j); pairs with i + j >= NS are dropped (below 2^(-7 NS)).
// The tensor cores multiply BF16 slices exactly and accumulate in FP32 in tensor memory
// (TMEM). Grouped by level l = i + j, all partial sums of a level are integer multiples of
// 2^(-7(l+2)); over a chunk of 512 K values the sums of levels 0, 1 and 2 stay below 2^24 of
// their unit, so their FP32 accumulation is exact. Levels >= 3 (2^-21 of the product and
// smaller) share a fourth accumulator whose FP32 rounding is below 1e-12 of the product. After
// each chunk the four accumulators are read out of TMEM and added, in compensated FP32
// arithmetic (error-free TwoSum, hi + lo carrying 48 bits), into per-thread running sums; the
// result is hi + lo in FP64 times the two row scales. With NS = 6 (21 slice products) the
// products are FP64-accurate (about 43 significant bits of |a||b|); with NS = 3 (6 products)
// they are FP32-accurate, which the FP32 filter's Rayleigh-Ritz step uses.
//
// Operands are split once per product by a streaming kernel into a tiled layout that is the
// tensor cores' own shared-memory layout (K-major, no swizzle: 8 x 16-byte core matrices), so
// the GEMM moves every (K step, 128-row block) group of NS slices with one bulk copy. For the
// rotation, Y's columns are first balanced by powers of two (and Q's rows by the inverse), so
// that a grid point's fixed-point row does not lose small columns to large ones.
//
// GEMM kernel (persistent, one CTA per SM looping over output tiles, 320 threads): warp 0
// issues the bulk copies into a ring of stages (four for 3 slices, two for 6), one thread of warp 1 issues tcgen05.mma (M = 128, N = 128, K = 16, BF16 inputs, FP32
// accumulators in four TMEM regions of 128 columns), warps 2-9 read the accumulators after
// each chunk (tcgen05.ld) and keep the compensated sums. Every barrier wait is bounded; a wait
// that runs out sets bit 4 of the status word and the kernel winds down (no copy left in
// flight, TMEM freed).
#include <algorithm>

#include <cuda_bf16.h>

#include "sgpu_internal.h"
#include "mbarrier.cuh"

namespace sgpu {
namespace {

constexpr int TM = 128;                         // output tile rows = TMEM lanes
constexpr int TN = 128;                         // output tile columns per accumulator
constexpr int TK = 32;                          // K per pipeline step
constexpr int TILE_ELEMS = TM * TK;             // one 128 x 32 BF16 slice tile
constexpr unsigned TILE_BYTES = TILE_ELEMS * 2; // 8 KB
constexpr int CHUNK_STEPS = 16;                 // K steps per exact chunk (512 K values)
constexpr int EPI_WARPS = 8;
constexpr int NTHREADS = 64 + 32 * EPI_WARPS;
constexpr int STATUS_TC_WAIT = 4;

template <int NS>
struct TcShape {
    static constexpr unsigned stage_bytes = 2u * NS * TILE_BYTES;  // A slices then B slices
    static constexpr int nstage = NS <= 3 ? 4 : 2;                 // ring depth
    static constexpr unsigned bar_off = nstage * stage_bytes;
    // full[nstage], empty[nstage], acc_full, acc_empty, done, TMEM address, abort flag; at
    // least 120 KB so that one CTA holds an SM (each CTA allocates all 512 TMEM columns)
    static constexpr unsigned need = bar_off + 16 * nstage + 32 + 1024;
    static constexpr unsigned smem_bytes = need > 120u * 1024 ? need : 120u * 1024;
};

struct TcParams {
    const __nv_bfloat16 *A;  // slices: [kstep][row block][slice][128 x 32 tile]
    const __nv_bfloat16 *B;
    int nrbA, nrbB;          // row blocks of A and B
    int ksteps;              // K steps of 32
    int mode;                // 0: Gram (upper tile pairs, split K), 1: rotation
    int ksplit;              // Gram: K ranges per tile pair
    int M, N;                // valid rows of A and of B (output rows / columns)
    const int *eA, *eB;      // power-of-two scale of each A row and B row
    double *C;               // Gram: partial sums [ksplit][N][M]; rotation: output (FP64)
    float *C32;              // rotation: FP32 output instead of C
    long ldc;
    int *status;
};

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor: K-major, no swizzle; core matrices 8 rows x 16 bytes,
// K-adjacent ones 128 bytes apart (leading byte offset), 8-row groups 512 bytes apart (stride
// byte offset); bit 46 is the descriptor version of this architecture
__device__ __forceinline__ unsigned long long smem_desc(unsigned addr)
{
    return (unsigned long long)((addr & 0x3FFFFu) >> 4) |
           ((unsigned long long)(128u >> 4) << 16) | ((unsigned long long)(512u >> 4) << 32) |
           (1ull << 46);
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major,
// N = 128 (bits 17-22 hold N/8), M = 128 (bits 24-28 hold M/16)
constexpr unsigned kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(TN >> 3) << 17) |
                            ((unsigned)(TM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(unsigned tmem_d, unsigned long long adesc,
                                         unsigned long long bdesc, unsigned accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
        : "memory");
}

// arrive once on the barrier when every tcgen05.mma issued so far by this thread has completed
__device__ __forceinline__ void mma_commit(unsigned bar)
{
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar)
        : "memory");
}

__device__ __forceinline__ void tc_fence_after()
{
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before()
{
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
}

// 16 consecutive 32-bit TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_ld16(unsigned taddr, float *v)
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

// error-free sum: s + e == a + b exactly (Knuth's TwoSum)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// exact float -> double through the bits (normal numbers; zero and the rest by conversion),
// so the epilogue spends no FP64-pipe instruction on it
__device__ __forceinline__ double f2d_exact(float f)
{
    const unsigned b = __float_as_uint(f);
    const unsigned be = (b >> 23) & 0xffu;
    if (be == 0u || be == 0xffu) return (double)f;
    return __longlong_as_double((long long)(((unsigned long long)(b >> 31) << 63) |
                                            ((unsigned long long)(be + 896u) << 52) |
                                            ((unsigned long long)(b & 0x7fffffu) << 29)));
}
// x 2^s by the exponent bits while the result stays a normal number (ldexp otherwise)
__device__ __forceinline__ double scale2(double x, int s)
{
    const long long b = __double_as_longlong(x);
    const int be = (int)((b >> 52) & 0x7ff);
    if (be == 0 || be + s <= 0 || be + s >= 0x7ff) return ldexp(x, s);
    return __longlong_as_double(b + ((long long)s << 52));
}
__device__ __forceinline__ float scale2f(float x, int s)
{
    const int b = __float_as_int(x);
    const int be = (b >> 23) & 0xff;
    if (be == 0 || be + s <= 0 || be + s >= 0xff) return ldexpf(x, s);
    return __int_as_float(b + (s << 23));
}

// Gram work item -> (row tile, column tile) with row tile <= column tile
__device__ __forceinline__ void upper_pair(int t, int nrb, int &mt, int &nt)
{
    mt = 0;
    int rem = t;
    while (rem >= nrb - mt) {
        rem -= nrb - mt;
        mt++;
    }
    nt = mt + rem;
}

template <int NS>
__global__ void __launch_bounds__(NTHREADS, 1) k_tc_gemm(const TcParams p)
{
    using S = TcShape<NS>;
    extern __shared__ __align__(1024) unsigned char smem[];
    const unsigned sbase = smem_u32(smem);
    constexpr int NST = S::nstage;
    const unsigned bar_full = sbase + S::bar_off;     // [NST]
    const unsigned bar_empty = bar_full + 8 * NST;    // [NST]
    const unsigned bar_accf = bar_empty + 8 * NST;
    const unsigned bar_acce = bar_accf + 8;
    const unsigned bar_done = bar_accf + 16;
    unsigned *tmem_slot = reinterpret_cast<unsigned *>(smem + S::bar_off + 16 * NST + 24);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + S::bar_off + 16 * NST + 28);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // ---- work items: tiles t = blockIdx.x, + gridDim.x, ...; the copy ring and the
    // accumulator barriers run on across tiles, so each CTA pays its set-up once
    const int ntiles = p.mode == 0 ? p.nrbA * (p.nrbA + 1) / 2 * p.ksplit : p.nrbA * p.nrbB;
    auto tile_of = [&](int t, int &mt, int &nt, int &ks0, int &ks1, int &split) {
        if (p.mode == 0) {
            const int npairs = p.nrbA * (p.nrbA + 1) / 2;
            split = t / npairs;
            upper_pair(t - split * npairs, p.nrbA, mt, nt);
            const int per = (p.ksteps + p.ksplit - 1) / p.ksplit;
            ks0 = split * per;
            ks1 = min(p.ksteps, ks0 + per);
        } else {
            mt = t / p.nrbB;
            nt = t - mt * p.nrbB;
            ks0 = 0;
            ks1 = p.ksteps;
            split = 0;
        }
        if (ks1 < ks0) ks1 = ks0;
    };

    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; s++) {
            mbar_init(bar_full + 8 * s, 1);
            mbar_init(bar_empty + 8 * s, 1);
        }
        mbar_init(bar_accf, 1);
        mbar_init(bar_acce, EPI_WARPS);
        mbar_init(bar_done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 1) {  // the whole warp allocates 512 TMEM columns (four accumulators)
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;\n" ::"r"(
                         smem_u32(tmem_slot))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tmem_slot;

    auto fail = [&]() {
        *abort_flag = 1;
        if (p.status) atomicOr(p.status, STATUS_TC_WAIT);
    };

    if (warp == 0) {
        // ---------------- producer: one bulk copy of the NS slices of A and of B per step
        if (lane == 0) {
            int it = 0;  // steps issued by this CTA (ring position)
            for (int t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x) {
                int mt, nt, ks0, ks1, split;
                tile_of(t, mt, nt, ks0, ks1, split);
                for (int s = ks0; s < ks1; s++, it++) {
                    const int st = it % NST;
                    if (it >= NST && !mbar_wait_bounded(bar_empty + 8 * st, (it / NST - 1) & 1)) {
                        fail();
                        break;
                    }
                    if (*abort_flag) break;
                    const __nv_bfloat16 *a = p.A + ((long)s * p.nrbA + mt) * (long)NS * TILE_ELEMS;
                    const __nv_bfloat16 *b = p.B + ((long)s * p.nrbB + nt) * (long)NS * TILE_ELEMS;
                    const unsigned dst = sbase + st * S::stage_bytes;
                    mbar_arrive_tx(bar_full + 8 * st, 2u * NS * TILE_BYTES);
                    bulk_g2s(dst, a, NS * TILE_BYTES, bar_full + 8 * st);
                    bulk_g2s(dst + NS * TILE_BYTES, b, NS * TILE_BYTES, bar_full + 8 * st);
                }
            }
            // no copy may land after the block exits: wait for the last fill of each stage
            const int issued = it;
            for (int st = 0; st < NST; st++) {
                const int last = issued - 1 - ((issued - 1 - st) % NST + NST) % NST;
                if (last >= 0 && !mbar_wait_bounded(bar_full + 8 * st, (last / NST) & 1)) fail();
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer
        if (lane == 0) {
            int it = 0, cg = 0;  // steps consumed, chunks completed (over all tiles)
            for (int t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x) {
                int mt, nt, ks0, ks1, split;
                tile_of(t, mt, nt, ks0, ks1, split);
                const int nsteps = ks1 - ks0;
                const int nchunks = (nsteps + CHUNK_STEPS - 1) / CHUNK_STEPS;
                for (int c = 0; c < nchunks && !*abort_flag; c++, cg++) {
                    if (cg > 0 && !mbar_wait_bounded(bar_acce, (cg - 1) & 1)) {
                        fail();
                        break;
                    }
                    tc_fence_after();
                    const int cend = min(nsteps, (c + 1) * CHUNK_STEPS);
                    for (int k = c * CHUNK_STEPS; k < cend; k++, it++) {
                        const int st = it % NST;
                        if (!mbar_wait_bounded(bar_full + 8 * st, (it / NST) & 1)) {
                            fail();
                            break;
                        }
                        if (*abort_flag) break;
                        tc_fence_after();
                        const unsigned a0 = sbase + st * S::stage_bytes;
                        const unsigned b0 = a0 + NS * TILE_BYTES;
                        const bool chunk_first = k == c * CHUNK_STEPS;
#pragma unroll
                        for (int i = 0; i < NS; i++) {
#pragma unroll
                            for (int j = 0; i + j < NS; j++) {
                                const int acc = min(i + j, 3);
                                const bool acc_first = i == 0 && j <= 3;
#pragma unroll
                                for (int kk = 0; kk < 2; kk++) {
                                    const unsigned accum =
                                        (chunk_first && acc_first && kk == 0) ? 0u : 1u;
                                    mma_bf16(tmem + acc * TN,
                                             smem_desc(a0 + i * TILE_BYTES + kk * 256),
                                             smem_desc(b0 + j * TILE_BYTES + kk * 256), accum);
                                }
                            }
                        }
                        mma_commit(bar_empty + 8 * st);  // the stage is free once these complete
                    }
                    mma_commit(bar_accf);  // the chunk's sums are complete
                }
            }
            mma_commit(bar_done);
            if (!mbar_wait_bounded(bar_done, 0)) fail();  // nothing in flight at dealloc
        }
    } else {
        // ---------------- epilogue: compensated sums of the chunk accumulators
        const int q = warp & 3;         // TMEM lane quarter this warp may access
        const int h = (warp - 2) >> 2;  // column half: 64 columns per warp
        const unsigned tl = tmem + ((unsigned)(32 * q) << 16) + (unsigned)(64 * h);
        int cg = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
            int mt, nt, ks0, ks1, split;
            tile_of(t, mt, nt, ks0, ks1, split);
            const int nchunks = (ks1 - ks0 + CHUNK_STEPS - 1) / CHUNK_STEPS;
            float hi[64], lo[64];
#pragma unroll
            for (int c = 0; c < 64; c++) hi[c] = lo[c] = 0.f;
            for (int c = 0; c < nchunks; c++, cg++) {
                if (*abort_flag) break;
                if (!mbar_wait_bounded(bar_accf, cg & 1)) {
                    fail();
                    break;
                }
                tc_fence_after();
                // levels 0, 1, 2, then the rest, into the running sums (cascaded TwoSum)
#pragma unroll
                for (int a = 0; a < (NS > 3 ? 4 : 3); a++) {
#pragma unroll
                    for (int g = 0; g < 4; g++) {
                        float l[16];
                        tmem_ld16(tl + a * TN + 16 * g, l);
#pragma unroll
                        for (int e = 0; e < 16; e++) {
                            float sum, err;
                            two_sum(hi[16 * g + e], l[e], sum, err);
                            hi[16 * g + e] = sum;
                            lo[16 * g + e] += err;
                        }
                    }
                }
                // the accumulators are free for the next chunk (of this tile or the next)
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(bar_acce);
            }
            if (*abort_flag) break;
            // ---- results: (hi + lo) times the two row scales
            const int m = mt * TM + 32 * q + lane;
            if (m < p.M) {
                const int em = p.eA[m];
                const int n0 = nt * TN + 64 * h;
                if (p.mode == 0) {
                    double *part = p.C + (long)split * p.N * p.M;  // [N][M], column-major
#pragma unroll
                    for (int c = 0; c < 64; c++) {
                        const int n = n0 + c;
                        // the upper triangle, mirrored: the result is exactly symmetric
                        if (n < p.N && (mt != nt || m <= n)) {
                            const double v =
                                scale2(f2d_exact(hi[c]) + f2d_exact(lo[c]), em + p.eB[n]);
                            part[(long)n * p.M + m] = v;
                            part[(long)m * p.M + n] = v;
                        }
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < 64; c++) {
                        const int n = n0 + c;
                        if (n < p.N) {
                            if (p.C32)  // FP32 output: no FP64 arithmetic
                                p.C32[(long)n * p.ldc + m] =
                                    scale2f(__fadd_rn(hi[c], lo[c]), em + p.eB[n]);
                            else
                                p.C[(long)n * p.ldc + m] =
                                    scale2(f2d_exact(hi[c]) + f2d_exact(lo[c]), em + p.eB[n]);
                        }
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;\n" ::"r"(tmem)
                     : "memory");
}

// ---------------- operand splitting

// The split runs in integer arithmetic (this part's FP64 pipe is slow): an entry x = m 2^p
// (m the signed integer significand) becomes the fixed-point integer U = round(x 2^(7 NS - e))
// of its row, |U| <= 2^(7 NS), cut into signed 7-bit digits S_i (each rounded to nearest, so
// |S_0| <= 128 and |S_i| <= 64 after it); slice i is S_i 2^(-7(i+1)), an exact BF16 number.
struct Bits {
    long long m;  // signed significand
    int p;        // power of two: x = m 2^p
    int fe;       // frexp exponent (|x| < 2^fe), or a large negative number for x = 0
};
__device__ __forceinline__ Bits bits_of(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int be = (int)((b >> 52) & 0x7ff);
    long long m = (long long)(b & ((1ull << 52) - 1));
    Bits r;
    if (be == 0) {
        r.p = -1074;
        r.fe = m ? -1022 : -(1 << 28);
    } else {
        m |= 1ll << 52;
        r.p = be - 1075;
        r.fe = be - 1022;
    }
    r.m = (b >> 63) ? -m : m;
    return r;
}
__device__ __forceinline__ Bits bits_of(float x)
{
    const unsigned b = __float_as_uint(x);
    const int be = (int)((b >> 23) & 0xff);
    long long m = (long long)(b & ((1u << 23) - 1));
    Bits r;
    if (be == 0) {
        r.p = -149;
        r.fe = m ? -126 : -(1 << 28);
    } else {
        m |= 1ll << 23;
        r.p = be - 150;
        r.fe = be - 126;
    }
    r.m = (b >> 31) ? -m : m;
    return r;
}

// slices of x 2^(-e) (|x 2^-e| < 1) as exact BF16 numbers S_i 2^(-7(i+1)), i < NS
template <int NS>
__device__ __forceinline__ void split7(Bits x, int e, __nv_bfloat16 *out)
{
    const int sh = x.p - e + 7 * NS;  // U = round(m 2^sh)
    long long V;
    if (sh >= 0) V = x.m << min(sh, 62);
    else if (sh > -62) V = (x.m + (1ll << (-sh - 1))) >> (-sh);
    else V = 0;
#pragma unroll
    for (int i = 0; i < NS; i++) {
        const int d = 7 * (NS - 1 - i);
        const long long S = d ? (V + (1ll << (d - 1))) >> d : V;
        V -= S << d;
        out[i] = __float2bfloat16_rn(__ll2float_rn(S) * __int_as_float((127 - 7 * (i + 1)) << 23));
    }
}

// element offset of (row r, k) inside a 128 x 32 tile: core matrix (r/8, k/8) at
// (r/8 * 4 + k/8) * 128 bytes, rows of 16 bytes
__device__ __forceinline__ int tile_off(int r, int k)
{
    return ((r >> 3) * 4 + (k >> 3)) * 64 + (r & 7) * 8 + (k & 7);
}

// power-of-two scale e of a row or column from the largest frexp exponent of its entries
// (max |x| < 2^e); 0 for a zero row
__device__ __forceinline__ int scale_of(int fe_max) { return fe_max < -(1 << 27) ? 0 : fe_max; }

// scale of each column of X (rows x cols, column-major), the entries of row r first scaled by
// 2^(ksign * ek[r]) when ek is given: one block per column
template <typename T>
__global__ void k_colmax_exp(const T *__restrict__ X, long ld, long rows, const int *ek,
                             int ksign, int *e)
{
    const T *x = X + (long)blockIdx.x * ld;
    int mx = -(1 << 28);
    for (long r = threadIdx.x; r < rows; r += blockDim.x)
        mx = max(mx, bits_of(x[r]).fe + (ek ? ksign * ek[r] : 0));
    __shared__ int red[32];
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x < 32) {
        mx = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : -(1 << 28);
        for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (threadIdx.x == 0) e[blockIdx.x] = scale_of(mx);
    }
}

// scale of each row of X (rows x cols, column-major), column c first scaled by 2^(-ec[c]):
// one thread per row
template <typename T>
__global__ void k_rowmax_exp(const T *__restrict__ X, long ld, long rows, int cols,
                             const int *__restrict__ ec, int *e)
{
    for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < rows;
         r += (long)gridDim.x * blockDim.x) {
        int mx = -(1 << 28);
        for (int c = 0; c < cols; c++) mx = max(mx, bits_of(X[(long)c * ld + r]).fe - ec[c]);
        e[r] = scale_of(mx);
    }
}

// Operand with K along each column of X (Gram operands: K = grid points; Q for the rotation:
// K = its row index, each row k first scaled by 2^(ksign * ek[k]) when ek is given): tile row
// = column n of X, tile K = rows of X. Block (step s, row block rb): 128 columns x 32 rows of
// X into NS slice tiles.
template <typename T, int NS>
__global__ void __launch_bounds__(256) k_split_cols(const T *__restrict__ X, long ld, long krows,
                                                    int ncols, const int *__restrict__ e,
                                                    const int *ek, int ksign, int nrb,
                                                    __nv_bfloat16 *__restrict__ out)
{
    const int s = blockIdx.x / nrb, rb = blockIdx.x - s * nrb;
    __nv_bfloat16 *tiles = out + ((long)s * nrb + rb) * (long)NS * TILE_ELEMS;
    for (int u = threadIdx.x; u < TM * 4; u += blockDim.x) {
        const int r = u >> 2, g = u & 3;
        const int n = rb * TM + r;
        const long k0 = (long)s * TK + g * 8;
        __nv_bfloat16 sl[8][NS];
        const int en = n < ncols ? e[n] : 0;
#pragma unroll
        for (int t = 0; t < 8; t++) {
            const long k = k0 + t;
            const bool in = n < ncols && k < krows;
            const Bits v = bits_of(in ? X[(long)n * ld + k] : T(0));
            split7<NS>(v, en - (ek && in ? ksign * ek[k] : 0), sl[t]);
        }
#pragma unroll
        for (int i = 0; i < NS; i++) {
            __align__(16) __nv_bfloat16 w[8];
#pragma unroll
            for (int t = 0; t < 8; t++) w[t] = sl[t][i];
            *reinterpret_cast<uint4 *>(tiles + i * TILE_ELEMS + tile_off(r, g * 8)) =
                *reinterpret_cast<const uint4 *>(w);
        }
    }
}

// Operand with K across the columns of X (the rotation's Y: tile row = grid point m, K =
// column index n of X, column n first scaled by 2^-ec[n]). Block (step s, row block rb): 128
// rows x 32 columns of X.
template <typename T, int NS>
__global__ void __launch_bounds__(256) k_split_rows(const T *__restrict__ X, long ld, long rows,
                                                    int kcols, const int *__restrict__ e,
                                                    const int *__restrict__ ec, int nrb,
                                                    __nv_bfloat16 *__restrict__ out)
{
    const int s = blockIdx.x / nrb, rb = blockIdx.x - s * nrb;
    __nv_bfloat16 *tiles = out + ((long)s * nrb + rb) * (long)NS * TILE_ELEMS;
    for (int u = threadIdx.x; u < TM * 4; u += blockDim.x) {
        const int g = u >> 7, r = u & 127;  // a warp: 32 consecutive rows, one K group
        const long m = (long)rb * TM + r;
        const int em = m < rows ? e[m] : 0;
        __nv_bfloat16 sl[8][NS];
#pragma unroll
        for (int t = 0; t < 8; t++) {
            const int k = s * TK + g * 8 + t;
            const bool in = m < rows && k < kcols;
            const Bits v = bits_of(in ? X[(long)k * ld + m] : T(0));
            split7<NS>(v, em + (in ? ec[k] : 0), sl[t]);
        }
#pragma unroll
        for (int i = 0; i < NS; i++) {
            __align__(16) __nv_bfloat16 w[8];
#pragma unroll
            for (int t = 0; t < 8; t++) w[t] = sl[t][i];
            *reinterpret_cast<uint4 *>(tiles + i * TILE_ELEMS + tile_off(r, g * 8)) =
                *reinterpret_cast<const uint4 *>(w);
        }
    }
}

// C = sum of the K-range partial sums (fixed order), ld ldc
__global__ void k_reduce_parts(const double *__restrict__ part, int ksplit, int n, double *C,
                               int ldc)
{
    const long total = (long)n * n;
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total;
         t += (long)gridDim.x * blockDim.x) {
        double v = 0.0;
        for (int s = 0; s < ksplit; s++) v += part[(long)s * total + t];
        const long j = t / n, i = t - j * n;
        C[j * ldc + i] = v;
    }
}

template <int NS>
int launch_gemm(sgpu_ctx *ctx, const TcParams &p, int ntiles, cudaStream_t st)
{
    constexpr unsigned smem = TcShape<NS>::smem_bytes;
    int nsm = 0;
    SGPU_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->device));
    const int nblocks = std::max(1, std::min(ntiles, nsm));  // persistent: one CTA per SM
    auto kern = k_tc_gemm<NS>;
    SGPU_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
    kern<<<nblocks, NTHREADS, smem, st>>>(p);
    SGPU_CUDA_TRY(cudaGetLastError());
    ctx->launches++;
    return SGPU_OK;
}

inline int blocks_for(long n, int per = 256)
{
    return (int)std::max<long>(1, std::min<long>((n + per - 1) / per, 152L * 64));
}

// split of a Gram operand (or Q) into the tiled slice layout, with per-column scales
template <typename T, int NS>
int split_cols(sgpu_ctx *ctx, const T *X, long ld, long krows, int ncols, int slot,
               __nv_bfloat16 **tiles, int **e, cudaStream_t st, const int *ek = nullptr,
               int ksign = 0)
{
    const int nrb = (ncols + TM - 1) / TM;
    const long ksteps = (krows + TK - 1) / TK;
    const size_t tbytes = sizeof(__nv_bfloat16) * (size_t)ksteps * nrb * NS * TILE_ELEMS;
    char *base = nullptr;
    SGPU_TRY(ws_get(ctx, slot, tbytes + sizeof(int) * ((size_t)ncols + 64), (void **)&base));
    *tiles = reinterpret_cast<__nv_bfloat16 *>(base);
    *e = reinterpret_cast<int *>(base + tbytes);
    {
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        k_colmax_exp<T><<<ncols, 256, 0, st>>>(X, ld, krows, ek, ksign, *e);
        SGPU_CUDA_TRY(cudaGetLastError());
    }
    {
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        k_split_cols<T, NS><<<(unsigned)(ksteps * nrb), 256, 0, st>>>(X, ld, krows, ncols, *e,
                                                                        ek, ksign, nrb, *tiles);
        SGPU_CUDA_TRY(cudaGetLastError());
    }
    ctx->launches += 2;
    return SGPU_OK;
}

// The rotation's Y: its columns are first balanced by powers of two (column c scaled by
// 2^-ec[c], ec from the column maxima; the caller scales row c of Q by 2^ec[c]), so that a
// grid point's fixed-point row does not lose the small columns to the large ones.
template <typename T, int NS>
int split_rows(sgpu_ctx *ctx, const T *X, long ld, long rows, int kcols, int slot,
               __nv_bfloat16 **tiles, int **e, int **ec, cudaStream_t st)
{
    const int nrb = (int)((rows + TM - 1) / TM);
    const int ksteps = (kcols + TK - 1) / TK;
    const size_t tbytes = sizeof(__nv_bfloat16) * (size_t)ksteps * nrb * NS * TILE_ELEMS;
    char *base = nullptr;
    SGPU_TRY(ws_get(ctx, slot, tbytes + sizeof(int) * ((size_t)rows + kcols + 128),
                    (void **)&base));
    *tiles = reinterpret_cast<__nv_bfloat16 *>(base);
    *e = reinterpret_cast<int *>(base + tbytes);
    *ec = *e + rows + 64;
    {
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        k_colmax_exp<T><<<kcols, 256, 0, st>>>(X, ld, rows, nullptr, 0, *ec);
        SGPU_CUDA_TRY(cudaGetLastError());
    }
    {
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        k_rowmax_exp<T><<<blocks_for(rows), 256, 0, st>>>(X, ld, rows, kcols, *ec, *e);
        SGPU_CUDA_TRY(cudaGetLastError());
    }
    {
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        k_split_rows<T, NS><<<(unsigned)((long)ksteps * nrb), 256, 0, st>>>(
            X, ld, rows, kcols, *e, *ec, nrb, *tiles);
        SGPU_CUDA_TRY(cudaGetLastError());
    }
    ctx->launches += 3;
    return SGPU_OK;
}

// one Gram-type product from split operands into C (ncol x ncol, ld ldc)
template <int NS>
int gram_tiles(sgpu_ctx *ctx, int ncol, const __nv_bfloat16 *ta, const int *ea,
               const __nv_bfloat16 *tb, const int *eb, double *C, int ldc, cudaStream_t st)
{
    const long Nd = ctx->Nd;
    const int nrb = (ncol + TM - 1) / TM;
    const int npairs = nrb * (nrb + 1) / 2;
    const int ksteps = (int)((Nd + TK - 1) / TK);
    int ksplit = std::max(1, 148 / npairs);
    ksplit = std::min(ksplit, std::max(1, ksteps / CHUNK_STEPS));
    double *part = nullptr;
    SGPU_TRY(ws_get(ctx, WS_TC_PART, sizeof(double) * (size_t)ksplit * ncol * ncol,
                    (void **)&part));
    TcParams p{};
    p.A = ta;
    p.B = tb;
    p.nrbA = p.nrbB = nrb;
    p.ksteps = ksteps;
    p.mode = 0;
    p.ksplit = ksplit;
    p.M = p.N = ncol;
    p.eA = ea;
    p.eB = eb;
    p.C = part;
    p.ldc = ncol;
    p.status = ctx->kstatus;
    SGPU_TRY(launch_gemm<NS>(ctx, p, npairs * ksplit, st));
    ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
    k_reduce_parts<<<blocks_for((long)ncol * ncol), 256, 0, st>>>(part, ksplit, ncol, C, ldc);
    SGPU_CUDA_TRY(cudaGetLastError());
    ctx->launches++;
    return SGPU_OK;
}

// Mp = Yᵀ Y and Hp = Yᵀ HY; Y is split once for both products
template <typename T, int NS>
int project_impl(sgpu_ctx *ctx, int ncol, const T *Y, long ldy, const T *HY, long ldh,
                 double *Hp, double *Mp, cudaStream_t st)
{
    const long Nd = ctx->Nd;
    __nv_bfloat16 *ty = nullptr, *th = nullptr;
    int *ey = nullptr, *eh = nullptr;
    SGPU_TRY((split_cols<T, NS>(ctx, Y, ldy, Nd, ncol, WS_SPLIT_A, &ty, &ey, st)));
    SGPU_TRY((split_cols<T, NS>(ctx, HY, ldh, Nd, ncol, WS_SPLIT_B, &th, &eh, st)));
    SGPU_TRY(gram_tiles<NS>(ctx, ncol, ty, ey, ty, ey, Mp, ncol, st));
    return gram_tiles<NS>(ctx, ncol, ty, ey, th, eh, Hp, ncol, st);
}

template <typename T, int NS>
int rotate_impl(sgpu_ctx *ctx, int ncol, const T *Y, long ldy, const double *Q, int ldq, T *X,
                long ldx, cudaStream_t st)
{
    const long Nd = ctx->Nd;
    __nv_bfloat16 *ta = nullptr, *tb = nullptr;
    int *ea = nullptr, *eb = nullptr;
    int *ecol = nullptr;  // column balance of Y; row c of Q gets the inverse power of two
    SGPU_TRY((split_rows<T, NS>(ctx, Y, ldy, Nd, ncol, WS_SPLIT_A, &ta, &ea, &ecol, st)));
    SGPU_TRY((split_cols<double, NS>(ctx, Q, ldq, ncol, ncol, WS_SPLIT_B, &tb, &eb, st, ecol,
                                     1)));
    TcParams p{};
    p.A = ta;
    p.B = tb;
    p.nrbA = (int)((Nd + TM - 1) / TM);
    p.nrbB = (ncol + TN - 1) / TN;
    p.ksteps = (ncol + TK - 1) / TK;
    p.mode = 1;
    p.ksplit = 1;
    p.M = (int)Nd;
    p.N = ncol;
    p.eA = ea;
    p.eB = eb;
    if constexpr (sizeof(T) == 4) p.C32 = X;
    else p.C = X;
    p.ldc = ldx;
    p.status = ctx->kstatus;
    return launch_gemm<NS>(ctx, p, p.nrbA * p.nrbB, st);
}

}  // namespace

// Hp = Yᵀ HY and Mp = Yᵀ Y (ncol x ncol, ld ncol, symmetric) for column-major Nd x ncol blocks,
// FP64-accurate (fp64_accurate) or FP32-accurate; the upper tile pairs are computed and
// mirrored (a symmetric eigensolver reads one triangle).
template <typename T>
int tc_project(sgpu_ctx *ctx, int ncol, const T *Y, long ldy, const T *HY, long ldh, double *Hp,
               double *Mp, bool fp64_accurate, cudaStream_t st)
{
    if (ncol <= 0) return SGPU_OK;
    if (fp64_accurate) return project_impl<T, 6>(ctx, ncol, Y, ldy, HY, ldh, Hp, Mp, st);
    return project_impl<T, 3>(ctx, ncol, Y, ldy, HY, ldh, Hp, Mp, st);
}

// X (Nd x ncol, ld ldx) = Y Q with Q ncol x ncol FP64 (ld ldq)
template <typename T>
int tc_rotate(sgpu_ctx *ctx, int ncol, const T *Y, long ldy, const double *Q, int ldq, T *X,
              long ldx, bool fp64_accurate, cudaStream_t st)
{
    if (ncol <= 0) return SGPU_OK;
    if (fp64_accurate) return rotate_impl<T, 6>(ctx, ncol, Y, ldy, Q, ldq, X, ldx, st);
    return rotate_impl<T, 3>(ctx, ncol, Y, ldy, Q, ldq, X, ldx, st);
}

template int tc_project<double>(sgpu_ctx *, int, const double *, long, const double *, long,
                                double *, double *, bool, cudaStream_t);
template int tc_project<float>(sgpu_ctx *, int, const float *, long, const float *, long,
                               double *, double *, bool, cudaStream_t);
template int tc_rotate<double>(sgpu_ctx *, int, const double *, long, const double *, int,
                               double *, long, bool, cudaStream_t);
template int tc_rotate<float>(sgpu_ctx *, int, const float *, long, const double *, int, float *,
                              long, bool, cudaStream_t);

}  // namespace sgpu
