// Fused nonlocal apply + next projection (FP32) on the tensor cores (tcgen05).
//
// The FP32 Chebyshev filter applies Vnl at every degree (src/nlocVecRoutines.c:798-886,
// called from src/eigenSolver.c:722-798) and projects the iterate it finishes for the next
// degree. Over a range of at most 128 covered grid points (consecutive in the order of compact
// blocks of the grid) whose atoms own at most 64 projector rows in all, both are small dense
// products with one shared matrix, the range's
// Chi tile C[point][row] (the Chi values of every atom image covering the point, images of one
// atom summed):
//     apply       T[point][col] += scale C[point][:] . alpha[:][col]       (M = 128 points)
//     projection  alpha_next[row][col] += dV Gamma_row sum_point C[point][row] T[point][col]
//                                                                           (M = 64 rows)
// with T the range's output tile (64 columns at a time). Each FP32 operand is written as the
// sum of three BF16 slices (hi, mid, lo: 24 significant bits), and the six slice products
// with i + j <= 2 are accumulated in FP32 in tensor memory, so the products are FP32-accurate
// (the split residuals and the dropped slice products are of order 2^-24 |C| |x|) and the
// accumulation is FP32 as on the CUDA cores.
//
// Per range (one CTA of 256 threads, two CTAs per SM): the Chi tile's three slices are built
// once in shared memory from the range's entries; then per group of 64 columns
//   1. the threads stage the group's alpha rows as BF16 slices (loaded one group ahead);
//   2. one thread issues the apply MMAs (A = Chi tile K-major, B = alpha MN-major; D in TMEM,
//      M = 128 lanes = points);
//   3. every thread reads 32 columns of one tile row out of TMEM, adds the tile values it
//      gathered from global memory one group ahead, writes the result back, and stages it as
//      BF16 slices (MN-major) in the buffer the alpha slices used;
//   4. one thread issues the projection MMAs (A = the same Chi tile read MN-major, so one copy
//      serves both products; B = the tile), and the threads add dV Gamma times the result to
//      alpha_next with vector atomics.
// Every covered output element is read and written once per launch and the Chi entries are
// read once per range. Barrier waits are bounded; a wait that runs out sets bit 8 of the
// status word and the block winds down.
#include <algorithm>
#include <unordered_map>
#include <vector>

#include <cuda_bf16.h>

#include "sgpu_internal.h"
#include "mbarrier.cuh"
#include "tcgen05.cuh"

namespace sgpu {
namespace {

constexpr int kTcPts = 128;      // covered points per range (apply M, projection K)
constexpr int kTcRows = 64;      // projector rows per range at most (apply K, projection M)
constexpr int kTcCols = 64;      // columns per group (N of both products)
constexpr int kTcCpt = 32;       // columns per thread: two threads per tile row
constexpr int kTcThreads = 256;
constexpr int STATUS_NL_TC_WAIT = 8;

// shared memory: the Chi tile's slices, then one buffer that holds the alpha slices of a column
// group (read by the apply) and then its tile slices (read by the projection), the range's row
// table and a barrier
constexpr unsigned kCdSlice = kTcPts * kTcRows * 2;  // 16 KB per BF16 slice
constexpr unsigned kAlSlice = kTcRows * kTcCols * 2; //  8 KB
constexpr unsigned kTlSlice = kTcPts * kTcCols * 2;  // 16 KB
constexpr unsigned kOffUB = 3 * kCdSlice;
constexpr unsigned kOffRows = kOffUB + 3 * kTlSlice;
constexpr unsigned kOffFac = kOffRows + 4 * kTcRows;
constexpr unsigned kOffBar = kOffFac + 4 * kTcRows;
constexpr unsigned kTcSmem = kOffBar + 64;  // 97 KB: two CTAs per SM
static_assert(3 * kAlSlice <= 3 * kTlSlice, "alpha slices fit the shared buffer");
static_assert(2 * (kTcSmem + 1024) <= 228 * 1024, "two CTAs per SM");

// Chi tile: core matrices of 8 points x 8 rows (16 bytes of rows per point), the 8 row blocks
// of a point block adjacent. K-major for the apply (M = points, K = rows: leading offset 128,
// stride 1024), MN-major for the projection (M = rows, K = points: leading 1024, stride 128).
__device__ __forceinline__ unsigned cd_off(int pt, int row)
{
    return (unsigned)((pt >> 3) * 1024 + (row >> 3) * 128 + (pt & 7) * 16 + (row & 7) * 2);
}
// alpha slices, MN-major (K = rows, N = columns): 8 rows x 8 columns per core matrix, the row
// blocks of one column block adjacent (leading offset 128, stride 1024)
__device__ __forceinline__ unsigned al_off(int row, int colblk)
{
    return (unsigned)(colblk * 1024 + (row >> 3) * 128 + (row & 7) * 16);
}
// tile slices, MN-major (K = points, N = columns): leading offset 128, stride 2048
__device__ __forceinline__ unsigned tl_off(int pt, int colblk)
{
    return (unsigned)(colblk * 2048 + (pt >> 3) * 128 + (pt & 7) * 16);
}

// x = hi + mid + lo + e, |e| <= 2^-24 |x| (round-to-nearest slices of 8 significant bits, each
// at most 2^-8 of the remainder it rounds; the differences are exact)
__device__ __forceinline__ void split3(float x, unsigned short &h, unsigned short &m,
                                       unsigned short &l)
{
    const __nv_bfloat16 bh = __float2bfloat16_rn(x);
    const float r1 = __fsub_rn(x, __bfloat162float(bh));
    const __nv_bfloat16 bm = __float2bfloat16_rn(r1);
    const float r2 = __fsub_rn(r1, __bfloat162float(bm));
    h = __bfloat16_as_ushort(bh);
    m = __bfloat16_as_ushort(bm);
    l = __bfloat16_as_ushort(__float2bfloat16_rn(r2));
}
// eight consecutive values -> one 16-byte piece of each slice (pairs converted together)
__device__ __forceinline__ void split8(const float *v, uint4 &s0, uint4 &s1, uint4 &s2)
{
    unsigned w[3][4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const __nv_bfloat162 h2 = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
        const float2 hf = __bfloat1622float2(h2);
        const float ra = __fsub_rn(v[2 * k], hf.x), rb = __fsub_rn(v[2 * k + 1], hf.y);
        const __nv_bfloat162 m2 = __floats2bfloat162_rn(ra, rb);
        const float2 mf = __bfloat1622float2(m2);
        const __nv_bfloat162 l2 = __floats2bfloat162_rn(__fsub_rn(ra, mf.x), __fsub_rn(rb, mf.y));
        w[0][k] = *reinterpret_cast<const unsigned *>(&h2);
        w[1][k] = *reinterpret_cast<const unsigned *>(&m2);
        w[2][k] = *reinterpret_cast<const unsigned *>(&l2);
    }
    s0 = make_uint4(w[0][0], w[0][1], w[0][2], w[0][3]);
    s1 = make_uint4(w[1][0], w[1][1], w[1][2], w[1][3]);
    s2 = make_uint4(w[2][0], w[2][1], w[2][2], w[2][3]);
}

struct TcTables {
    const int *pt0;     // nrange + 1: first point of each range in pts
    const int *row0;    // nrange + 1: first entry of each range's row list
    const int *rows;    // alpha row of every range row
    const int *ent0;    // nrange + 1: first merged entry of each range
    const int *ent;     // merged entry: point | row offset << 7 | projector count << 14
    const float *chi;   // merged entry: Chi values, jp per entry
    int jp;
    const int *pts;     // grid point of every range point (ranges back to back)
    const float *gamma;
};

__global__ void __launch_bounds__(kTcThreads, 2)
    k_nl_apply_project_tc(const TcTables T, int ncol, const float *__restrict__ alpha, long lda,
                          float scale, float *__restrict__ out, long ldo,
                          float *__restrict__ alpha_next, float dV, int *status)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const unsigned sb = tc_smem_u32(smem);
    int *rows = reinterpret_cast<int *>(smem + kOffRows);
    float *fac = reinterpret_cast<float *>(smem + kOffFac);
    const unsigned bar = sb + kOffBar;
    unsigned *tslot = reinterpret_cast<unsigned *>(smem + kOffBar + 8);
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int r = blockIdx.x;
    const int p0 = T.pt0[r], npt = T.pt0[r + 1] - p0;
    const int q0 = T.row0[r], nrow = T.row0[r + 1] - q0;
    const int e0 = T.ent0[r], e1 = T.ent0[r + 1];
    const int pt = t & 127, h = t >> 7;  // tile row (TMEM lane) and column half
    const int gp = pt < npt ? __ldg(T.pts + p0 + pt) : 0;
    const int ngroup = (ncol + kTcCols - 1) / kTcCols;
    const int g0 = r % ngroup;  // ranges start at different column groups
    // 16-byte alpha rows and atomics
    const bool vec_a = (lda & 3) == 0 && ((reinterpret_cast<uintptr_t>(alpha) |
                                           reinterpret_cast<uintptr_t>(alpha_next)) & 15) == 0;

    // tile values of this thread's 32 columns of a group (loaded one group ahead)
    float G[kTcCpt];
    auto gather = [&](int n0) {
        const int cb = n0 + kTcCpt * h;
        const float *src = out + (long)cb * ldo + gp;
        if (pt < npt && cb + kTcCpt <= ncol) {  // all 32 columns present
#pragma unroll
            for (int c = 0; c < kTcCpt; c++, src += ldo) G[c] = *src;
        } else {
#pragma unroll
            for (int c = 0; c < kTcCpt; c++, src += ldo)
                G[c] = (pt < npt && cb + c < ncol) ? *src : 0.f;
        }
    };
    // alpha pieces of a group: row t % 64, column blocks t / 64 and t / 64 + 4 (8 values each)
    float A[16];
    const int arow = t & 63;
    auto load_alpha = [&](int n0) {
#pragma unroll
        for (int u = 0; u < 2; u++) {
            float *a = A + 8 * u;
            const int c0 = n0 + 8 * ((t >> 6) + 4 * u);
            if (arow < nrow) {
                const float *ar = alpha + (long)rows[arow] * lda + c0;
                if (vec_a && c0 + 7 < ncol) {
                    const float4 x0 = __ldg(reinterpret_cast<const float4 *>(ar));
                    const float4 x1 = __ldg(reinterpret_cast<const float4 *>(ar) + 1);
                    a[0] = x0.x; a[1] = x0.y; a[2] = x0.z; a[3] = x0.w;
                    a[4] = x1.x; a[5] = x1.y; a[6] = x1.z; a[7] = x1.w;
                } else {
#pragma unroll
                    for (int k = 0; k < 8; k++) a[k] = c0 + k < ncol ? __ldg(ar + k) : 0.f;
                }
            } else {
#pragma unroll
                for (int k = 0; k < 8; k++) a[k] = 0.f;
            }
        }
    };

    gather(g0 * kTcCols);  // in flight while the Chi tile is built
    // this thread's first merged entry, loaded before the tile is zeroed (12 values per entry,
    // the layout of sets with at most 9 projectors per atom; others load in the loop below)
    const bool pre = T.jp == 12 && e0 + t < e1;
    int meta_pre = 0;
    float4 chi_pre[3];
    if (pre) {
        meta_pre = __ldg(T.ent + e0 + t);
        const float4 *c4 = reinterpret_cast<const float4 *>(T.chi + (long)(e0 + t) * 12);
#pragma unroll
        for (int q = 0; q < 3; q++) chi_pre[q] = __ldg(c4 + q);
    }
    if (t == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) tc_alloc(tc_smem_u32(tslot), 128);  // apply D: columns 0-63, projection: 64-127
    {
        const uint4 z = make_uint4(0u, 0u, 0u, 0u);
        uint4 *cz = reinterpret_cast<uint4 *>(smem);
        for (int i = t; i < (int)(3 * kCdSlice / 16); i += kTcThreads) cz[i] = z;
    }
    for (int i = t; i < kTcRows; i += kTcThreads) {
        const int row = i < nrow ? T.rows[q0 + i] : 0;
        rows[i] = row;
        fac[i] = i < nrow ? dV * T.gamma[row] : 0.f;
    }
    __syncthreads();
    load_alpha(g0 * kTcCols);
    // the Chi tile: merged entries (one per point and atom) into the three slices
    auto put_chi = [&](int lp, int row, float x) {
        unsigned short hs, ms, ls;
        split3(x, hs, ms, ls);
        const unsigned o = cd_off(lp, row);
        *reinterpret_cast<unsigned short *>(smem + o) = hs;
        *reinterpret_cast<unsigned short *>(smem + kCdSlice + o) = ms;
        *reinterpret_cast<unsigned short *>(smem + 2 * kCdSlice + o) = ls;
    };
    if (pre) {
        const int lp = meta_pre & 127, ro = (meta_pre >> 7) & 127, np = meta_pre >> 14;
        const float cv[12] = {chi_pre[0].x, chi_pre[0].y, chi_pre[0].z, chi_pre[0].w,
                              chi_pre[1].x, chi_pre[1].y, chi_pre[1].z, chi_pre[1].w,
                              chi_pre[2].x, chi_pre[2].y, chi_pre[2].z, chi_pre[2].w};
#pragma unroll
        for (int j = 0; j < 12; j++)
            if (j < np) put_chi(lp, ro + j, cv[j]);
    }
    for (int e = e0 + t + (pre ? kTcThreads : 0); e < e1; e += kTcThreads) {
        const int meta = T.ent[e];
        const int lp = meta & 127, ro = (meta >> 7) & 127, np = meta >> 14;
        const float *cv = T.chi + (long)e * T.jp;
        for (int j = 0; j < np; j++) put_chi(lp, ro + j, __ldg(cv + j));
    }
    tc_smem_to_async();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    const unsigned tmem = *tslot;
    const unsigned tA = tmem, tP = tmem + 64;
    const int ks_a = (nrow + 15) >> 4, ks_p = (npt + 15) >> 4;
    const unsigned tl = (unsigned)(32 * (warp & 3)) << 16;  // this warp's TMEM lane quarter
    constexpr unsigned idA = tc_idesc_bf16(128, kTcCols, false, true);
    constexpr unsigned idP = tc_idesc_bf16(64, kTcCols, true, true);
    unsigned phase = 0;
    bool ok = true;

    int gcur = g0;
    for (int gi = 0; gi < ngroup; gi++) {
        const int n0 = gcur * kTcCols;
        gcur = gcur + 1 == ngroup ? 0 : gcur + 1;  // the next group
        const int cb = n0 + kTcCpt * h;            // this thread's first column
        // 1. the alpha rows as slices (loaded one group ahead)
#pragma unroll
        for (int u = 0; u < 2; u++) {
            uint4 s0, s1, s2;
            split8(A + 8 * u, s0, s1, s2);
            const unsigned o = kOffUB + al_off(arow, (t >> 6) + 4 * u);
            *reinterpret_cast<uint4 *>(smem + o) = s0;
            *reinterpret_cast<uint4 *>(smem + kAlSlice + o) = s1;
            *reinterpret_cast<uint4 *>(smem + 2 * kAlSlice + o) = s2;
        }
        tc_smem_to_async();
        tc_before_sync();
        if (__syncthreads_or(!ok)) break;  // a wait of the previous group ran out
        // 2. apply: D = sum over slice pairs (i, j), i + j <= 2, of C_i alpha_j; descriptor
        //    address fields count 16 bytes, so offsets add to the base words
        if (t == 0) {
            tc_after_sync();
            const unsigned long long da = tc_desc(sb, 128, 1024);
            const unsigned long long db = tc_desc(sb + kOffUB, 128, 1024);
            unsigned acc = 0u;
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int j = 0; i + j < 3; j++)
                    for (int kk = 0; kk < ks_a; kk++) {
                        tc_mma_bf16(tA, da + ((i * kCdSlice + kk * 256) >> 4),
                                    db + ((j * kAlSlice + kk * 256) >> 4), idA, acc);
                        acc = 1u;
                    }
            tc_commit(bar);
        }
        if (mbar_wait_suspend(bar, phase)) phase ^= 1u;
        else ok = false;
        tc_after_sync();
        // 3. the finished tile T + scale D: to global memory, and as slices for the projection
        float v[kTcCpt];
        tc_ld32(tA + tl + kTcCpt * h, v);
#pragma unroll
        for (int c = 0; c < kTcCpt; c++) v[c] = __fmaf_rn(scale, v[c], G[c]);
        if (pt < npt) {
            float *dst = out + (long)cb * ldo + gp;
            if (cb + kTcCpt <= ncol) {
#pragma unroll
                for (int c = 0; c < kTcCpt; c++, dst += ldo) *dst = v[c];
            } else {
#pragma unroll
                for (int c = 0; c < kTcCpt; c++, dst += ldo)
                    if (cb + c < ncol) *dst = v[c];
            }
        }
        if (gi + 1 < ngroup) {  // in flight during the projection
            gather(gcur * kTcCols);
            load_alpha(gcur * kTcCols);
        }
        if (alpha_next) {
#pragma unroll
            for (int k = 0; k < kTcCpt / 8; k++) {
                uint4 s0, s1, s2;
                split8(v + 8 * k, s0, s1, s2);
                const unsigned o = kOffUB + tl_off(pt, 4 * h + k);
                *reinterpret_cast<uint4 *>(smem + o) = s0;
                *reinterpret_cast<uint4 *>(smem + kTlSlice + o) = s1;
                *reinterpret_cast<uint4 *>(smem + 2 * kTlSlice + o) = s2;
            }
            tc_smem_to_async();
            tc_before_sync();
            __syncthreads();
            // 4. projection: P = sum over (i, j), i + j <= 2, of C_i^T T_j
            if (t == 0) {
                tc_after_sync();
                const unsigned long long da = tc_desc(sb, 1024, 128);
                const unsigned long long db = tc_desc(sb + kOffUB, 128, 2048);
                unsigned acc = 0u;
#pragma unroll
                for (int i = 0; i < 3; i++)
#pragma unroll
                    for (int j = 0; i + j < 3; j++)
                        for (int kk = 0; kk < ks_p; kk++) {
                            tc_mma_bf16(tP, da + ((i * kCdSlice + kk * 2048) >> 4),
                                        db + ((j * kTlSlice + kk * 256) >> 4), idP, acc);
                            acc = 1u;
                        }
                tc_commit(bar);
            }
            if (mbar_wait_suspend(bar, phase)) phase ^= 1u;
            else ok = false;
            tc_after_sync();
            // alpha_next += dV Gamma P: rows 16 (warp & 3) + lane in lanes 0..15
            const int rho = 16 * (warp & 3) + lane;
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
                float pv[16];
                tc_ld16(tP + tl + kTcCpt * h + 16 * hh, pv);
                if (lane < 16 && rho < nrow) {
                    const float f = fac[rho];
                    const int c0 = cb + 16 * hh;
                    float *dst = alpha_next + (long)rows[rho] * lda + c0;
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        if (vec_a && c0 + 4 * k + 3 < ncol) {
                            atomicAdd(reinterpret_cast<float4 *>(dst + 4 * k),
                                      make_float4(f * pv[4 * k], f * pv[4 * k + 1],
                                                  f * pv[4 * k + 2], f * pv[4 * k + 3]));
                        } else {
#pragma unroll
                            for (int w = 0; w < 4; w++)
                                if (c0 + 4 * k + w < ncol)
                                    atomicAdd(dst + 4 * k + w, f * pv[4 * k + w]);
                        }
                    }
                }
            }
        }
        tc_before_sync();
    }
    if (__syncthreads_or(!ok)) {
        // a wait ran out: record it, and let every MMA issued finish before TMEM is freed (the
        // phase of a wait that ran out was not advanced, so this waits for the same commit)
        if (t == 0) atomicOr(status, STATUS_NL_TC_WAIT);
        mbar_wait_suspend(bar, phase);
    }
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (warp == 0) tc_dealloc(tmem, 128);
}

}  // namespace

bool nonlocal_tc_ready(const sgpu_ctx *ctx)
{
    return ctx->has_nl && ctx->nl.tc_nrange > 0;
}

int launch_nonlocal_apply_project_tc(sgpu_ctx *ctx, int ncol, const float *alpha, long lda,
                                     double scale, float *out, long ldo, float *alpha_next,
                                     cudaStream_t st)
{
    const Nonlocal &nl = ctx->nl;
    if (!ctx->has_nl || nl.ncov == 0 || ncol <= 0) return SGPU_OK;
    if (nl.tc_nrange == 0) {
        set_error("nonlocal: the tensor-core fused apply needs its range tables (none built)");
        return SGPU_ERR_STATE;
    }
    TcTables T{nl.tc_pt0, nl.tc_row0, nl.tc_rows, nl.tc_ent0, nl.tc_ent, nl.tc_chi,
               nl.range_jp, nl.tc_pts, nl.gamma32};
    ProfScope ps(ctx, SGPU_KERNEL_NL_APPLY, st);
    SGPU_CUDA_TRY(cudaFuncSetAttribute(k_nl_apply_project_tc,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem));
    k_nl_apply_project_tc<<<nl.tc_nrange, kTcThreads, kTcSmem, st>>>(
        T, ncol, alpha, lda, (float)scale, out, ldo, alpha_next, (float)ctx->dV, ctx->kstatus);
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

// Ranges of the tensor-core form. The covered points are taken in the order of compact blocks
// of kTcBx x kTcBy x kTcBz grid points (x fastest inside a block, blocks in grid order), so
// that a range of 128 consecutive points in that order is a compact piece of the grid that few
// atoms' spheres reach, while a warp's 32 points still form one 128-byte run of x (C2: 5.7 k
// ranges of 124 points and 42 rows on average, against 8.4 k ranges of 85 points and 58 rows
// in plain grid order; 1.21 against 1.63 ms per launch; 8-wide blocks cut the runs to 32 bytes
// and measured 1.46 ms); a range closes at kTcPts points or when the next point's atoms would
// take it past kTcRows projector rows. Per range: its points'
// grid indices, its atoms' rows (first use order) and one merged entry per (point, atom) whose
// Chi values are the sum over the atom's images at the point (FP64 sums, stored in FP32). When
// one covered point alone needs more than kTcRows rows no tables are built and the form is
// unavailable.
constexpr int kTcBx = 32, kTcBy = 4, kTcBz = 4;
int nonlocal_tc_build(Nonlocal &nl, int Nx, int Ny, const std::vector<int> &covpts,
                      const std::vector<int> &covptr, const std::vector<long> &ent_chi,
                      const std::vector<int4> &ent_meta, const double *chi)
{
    std::vector<int> pt0(1, 0), row0(1, 0), rows, ent0(1, 0), ent, pts;
    std::vector<float> chiv;
    const int jp = nl.range_jp;
    if (nl.max_np > jp || nl.max_np > kTcRows) {  // an atom's rows exceed an entry or a range
        nl.tc_nrange = 0;
        return SGPU_OK;
    }
    // covered points in block order
    std::vector<int> ord(nl.ncov);
    {
        const long nbx = (Nx + kTcBx - 1) / kTcBx, nby = (Ny + kTcBy - 1) / kTcBy;
        std::vector<long long> key(nl.ncov);
        for (int c = 0; c < nl.ncov; c++) {
            const long g = covpts[c];
            const long x = g % Nx, y = (g / Nx) % Ny, z = g / ((long)Nx * Ny);
            const long blk = ((z / kTcBz) * nby + y / kTcBy) * nbx + x / kTcBx;
            const long in = ((z % kTcBz) * kTcBy + y % kTcBy) * kTcBx + x % kTcBx;
            key[c] = (long long)blk * (kTcBx * kTcBy * kTcBz) + in;
            ord[c] = c;
        }
        std::sort(ord.begin(), ord.end(), [&](int a, int b) { return key[a] < key[b]; });
    }
    std::unordered_map<int, int> rowoff;  // atom (its first projector row) -> range row offset
    std::vector<double> acc(jp);
    int k = 0;
    while (k < nl.ncov) {
        const int q0 = k;
        rowoff.clear();
        int nrow = 0;
        while (k < nl.ncov && k - q0 < kTcPts) {
            const int p = ord[k];
            int add = 0;
            for (int e = covptr[p]; e < covptr[p + 1]; e++) {
                const int ip = ent_meta[e].x;
                bool seen = rowoff.count(ip) > 0;
                for (int e2 = covptr[p]; e2 < e && !seen; e2++) seen = ent_meta[e2].x == ip;
                if (!seen) add += ent_meta[e].y;
            }
            if (nrow + add > kTcRows) break;
            for (int e = covptr[p]; e < covptr[p + 1]; e++) {
                const int ip = ent_meta[e].x;
                if (!rowoff.count(ip)) {
                    rowoff[ip] = nrow;
                    for (int j = 0; j < ent_meta[e].y; j++) rows.push_back(ip + j);
                    nrow += ent_meta[e].y;
                }
            }
            k++;
        }
        if (k == q0) {  // one point needs more rows than a range holds: no tensor-core form
            nl.tc_nrange = 0;
            return SGPU_OK;
        }
        for (int kk = q0; kk < k; kk++) {
            const int c = ord[kk];
            pts.push_back(covpts[c]);
            // merged entries of point c, one per atom, in the order the atoms first appear
            for (int e = covptr[c]; e < covptr[c + 1]; e++) {
                const int ip = ent_meta[e].x, np = ent_meta[e].y;
                bool first = true;
                for (int e2 = covptr[c]; e2 < e && first; e2++) first = ent_meta[e2].x != ip;
                if (!first) continue;
                std::fill(acc.begin(), acc.end(), 0.0);
                for (int e2 = e; e2 < covptr[c + 1]; e2++) {
                    if (ent_meta[e2].x != ip) continue;
                    for (int j = 0; j < np; j++)
                        acc[j] += chi[ent_chi[e2] + (long)j * ent_meta[e2].z];
                }
                ent.push_back((kk - q0) | (rowoff[ip] << 7) | (np << 14));
                for (int j = 0; j < jp; j++) chiv.push_back(j < np ? (float)acc[j] : 0.f);
            }
        }
        pt0.push_back(k);
        row0.push_back((int)rows.size());
        ent0.push_back((int)ent.size());
    }
    nl.tc_nrange = (int)pt0.size() - 1;
    int rc = SGPU_OK;
    auto up = [&](auto **dst, const auto &v) {
        using T = std::remove_reference_t<decltype(v[0])>;
        if (rc != SGPU_OK) return;
        if (cudaMalloc((void **)dst, sizeof(T) * std::max<size_t>(v.size(), 1)) != cudaSuccess ||
            (!v.empty() && cudaMemcpy(*dst, v.data(), sizeof(T) * v.size(),
                                      cudaMemcpyHostToDevice) != cudaSuccess)) {
            set_error("set_nonlocal: device allocation of the tensor-core range tables failed");
            rc = SGPU_ERR_CUDA;
        }
    };
    up(&nl.tc_pt0, pt0);
    up(&nl.tc_pts, pts);
    up(&nl.tc_row0, row0);
    up(&nl.tc_rows, rows);
    up(&nl.tc_ent0, ent0);
    up(&nl.tc_ent, ent);
    up(&nl.tc_chi, chiv);
    if (rc != SGPU_OK) nl.tc_nrange = 0;
    return rc;
}

}  // namespace sgpu
