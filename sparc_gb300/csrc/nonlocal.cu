// Kleinman-Bylander nonlocal projector apply, split in two device passes.
//
// Reference: Vnl_vec_mult (src/nlocVecRoutines.c:798-886), per atom J:
//   alpha_J = dV * Chi_Jᵀ x[grid_pos_J]          (gather + dgemm, :806-833)
//   alpha_J[j, n] *= Gamma_J[j]                   (:843-866)
//   Hx[grid_pos_J] += Chi_J alpha_J               (dgemm + scatter, :869-884)
//
// GPU forms (the autotuner picks per context; see each kernel):
//   * project: a gathered GEMM with one atomic add per (projector, column) and block, dV *
//     Gamma folded in. Segment form: one block per segment of at most kSegPts points of one
//     atom image. Range form (FP32): one block per range of consecutive covered points, all
//     images over it, so each covered x element is read once and in grid order.
//   * apply: owner-computes over a CSR of covered grid points (per point over column blocks;
//     with alpha rows staged per chunk; with the Chi values hoisted; a dense product per
//     chunk), each output element written by one thread, or the range form (FP32), which
//     gathers a range's output tile into shared memory, adds every image's contribution there
//     and writes the tile back once.
#include <algorithm>
#include <numeric>

#include "sgpu_internal.h"

namespace sgpu {
namespace {

constexpr int kProjThreads = 256;
constexpr int kSegPts = 512;  // points of one image handled by one projection block
constexpr int kApplyChunk = kApplyChunkPts;   // covered points per block of the staged apply
constexpr size_t kApplyStageMax = 96 * 1024;  // staged alpha rows must fit this (bytes)
constexpr size_t kApplyDenseMax = 150 * 1024; // dense-chunk apply: staged rows and Chi (bytes)

template <typename T, int CB>
struct VecOf;
template <> struct VecOf<float, 4> { using type = float4; };
template <> struct VecOf<double, 2> { using type = double2; };

// alpha layout: alpha[row * lda + n], row = IP_displ[atom] + j (projector), n = column;
// lda is a multiple of the apply's column block so rows can be read as vectors.
//
// Projection kernel: block = one segment (at most kSegPts points) of one atom image. The
// segment's grid positions and its Chi rows (transposed to point-major, MAXJP values per point
// so a point's projectors load as 16-byte vectors) are staged in shared memory once. The block
// then walks column groups of NC: it gathers x[grid_pos, group] chunk by chunk into shared
// memory, and thread (column n, point half h) accumulates alpha[0..MAXJ-1, n] in registers
// over its half of each chunk; the two halves are summed through shared memory and added
// atomically into alpha, with dV * Gamma folded in.
template <typename T, int PCH, int NC, int MAXJ>
__global__ void __launch_bounds__(kProjThreads)
    k_nl_project(const int *__restrict__ seg_img, const int *__restrict__ seg_start,
                 const int *__restrict__ img_atom, const int *__restrict__ img_ndc,
                 const long *__restrict__ img_off, const long *__restrict__ img_chi_off,
                 const int *__restrict__ grid_pos, const T *__restrict__ chi,
                 const int *__restrict__ ip_displ, const T *__restrict__ gamma, int ncol,
                 const T *__restrict__ x, long ldx, T *__restrict__ alpha, long lda, T dV)
{
    constexpr int HALVES = kProjThreads / NC;
    static_assert(HALVES * NC == kProjThreads, "threads = columns x point groups");
    static_assert(kSegPts % PCH == 0 && PCH % HALVES == 0, "whole chunks");
    constexpr int VW = 16 / sizeof(T);                        // elements per 16-byte vector
    constexpr int MAXJP = (MAXJ + VW - 1) / VW * VW;          // padded projectors per point
    constexpr int GX = PCH * NC / kProjThreads;               // gathers per thread and chunk
    using V = typename VecOf<T, VW>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // x tile [NC][PCH + 1], reused after the chunk loop as the reduction buffer
    // [HALVES][MAXJ][NC]: the region holds the larger of the two
    constexpr size_t XS = (size_t)NC * (PCH + 1) > (size_t)HALVES * MAXJ * NC
                              ? (size_t)NC * (PCH + 1) : (size_t)HALVES * MAXJ * NC;
    T *cs = reinterpret_cast<T *>(smem_raw);                  // [kSegPts][MAXJP]
    T *xs = cs + (size_t)MAXJP * kSegPts;
    int *gps = reinterpret_cast<int *>(xs + XS);              // [kSegPts]

    const int g = seg_img[blockIdx.x];
    const int sbeg = seg_start[blockIdx.x];
    const int a = img_atom[g];
    const int np = ip_displ[a + 1] - ip_displ[a];
    const int ndc = img_ndc[g];
    const int cnt_seg = min(ndc - sbeg, kSegPts);
    const int *__restrict__ gp = grid_pos + img_off[g] + sbeg;
    const T *__restrict__ ch = chi + img_chi_off[g] + sbeg;
    const int t = threadIdx.x;
    const int n = t % NC, h = t / NC;

    for (int i = t; i < kSegPts; i += kProjThreads) gps[i] = i < cnt_seg ? gp[i] : 0;
    for (int e = t; e < MAXJP * kSegPts; e += kProjThreads) {
        const int i = e / MAXJP, j = e % MAXJP;
        cs[e] = (j < np && i < cnt_seg) ? __ldg(ch + (long)j * ndc + i) : T(0);
    }

    for (int n0 = 0; n0 < ncol; n0 += NC) {
        T acc[MAXJP];
#pragma unroll
        for (int j = 0; j < MAXJP; j++) acc[j] = T(0);
        for (int i0 = 0; i0 < cnt_seg; i0 += PCH) {
            const int cnt = min(PCH, cnt_seg - i0);
            __syncthreads();  // staging done / previous chunk consumed
            T v[GX];
#pragma unroll
            for (int u = 0; u < GX; u++) {
                const int e = t + u * kProjThreads;
                const int i = e % PCH, c = e / PCH;
                v[u] = (i < cnt && n0 + c < ncol)
                           ? __ldg(x + (long)(n0 + c) * ldx + gps[i0 + i]) : T(0);
            }
#pragma unroll
            for (int u = 0; u < GX; u++) {
                const int e = t + u * kProjThreads;
                xs[(e / PCH) * (PCH + 1) + e % PCH] = v[u];
            }
            __syncthreads();
            const T *xr = xs + n * (PCH + 1);
#pragma unroll 2
            for (int i = h; i < PCH; i += HALVES) {
                const T xv = xr[i];
                const V *cv = reinterpret_cast<const V *>(cs + (size_t)(i0 + i) * MAXJP);
#pragma unroll
                for (int q = 0; q < MAXJP / VW; q++) {
                    const V c4 = cv[q];
                    const T *ce = reinterpret_cast<const T *>(&c4);
#pragma unroll
                    for (int w = 0; w < VW; w++) acc[q * VW + w] += ce[w] * xv;
                }
            }
        }
        // sum the point groups, then one atomic add per (projector, column)
        __syncthreads();
        T *red = xs;  // reuse: [HALVES][MAXJ][NC]
#pragma unroll
        for (int j = 0; j < MAXJ; j++) red[((size_t)h * MAXJ + j) * NC + n] = acc[j];
        __syncthreads();
        for (int e = t; e < MAXJ * NC; e += kProjThreads) {
            const int j = e / NC, c = e % NC;
            if (j < np && n0 + c < ncol) {
                T s = T(0);
#pragma unroll
                for (int hh = 0; hh < HALVES; hh++) s += red[((size_t)hh * MAXJ + j) * NC + c];
                const int row = ip_displ[a] + j;
                atomicAdd(alpha + (long)row * lda + n0 + c, dV * gamma[row] * s);
            }
        }
    }
}

// Gathers the tile src[gps[lp], n0 + c] (lp < npt, c < NC, column n0 + c < ncol; zero
// elsewhere) into dst[lp * LD + c] with 4-byte cp.async copies, all of a thread's copies in
// flight together; returns once the tile is complete for this thread (the caller's barrier
// makes it complete for the block). 256 threads.
template <int LD, int NC>
__device__ __forceinline__ void gather_tile(const float *__restrict__ src, long lds, int n0,
                                            int ncol, const int *__restrict__ gps, int npt,
                                            float *__restrict__ dst)
{
    static_assert(kRangePts * NC % 256 == 0, "whole copies per thread");
#pragma unroll 8
    for (int u = 0; u < kRangePts * NC / 256; u++) {
        const int idx = threadIdx.x + u * 256;
        const int lp = idx % kRangePts, c = idx / kRangePts;
        float *d = dst + lp * LD + c;
        if (lp < npt && n0 + c < ncol) {
            const unsigned sa = (unsigned)__cvta_generic_to_shared(d);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa),
                         "l"(src + (long)(n0 + c) * lds + gps[lp])
                         : "memory");
        } else {
            *d = 0.f;
        }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Range projection (FP32): block = one range of at most kRangePts consecutive covered points
// (grid order). The range's entries, regrouped by image into work items, have their Chi rows
// (range_jp values each) and point indices staged in shared memory once. For each group of
// NC = 64 columns the block gathers x[range points, group] into shared memory (every covered
// x element is read once per launch, in grid order, whatever the number of spheres over it),
// then each warp takes work items in turn: lane l accumulates alpha[0..MAXJ-1] of columns
// 2l, 2l+1 over the item's entries and adds them atomically (one 8-byte atomic per pair),
// with dV * Gamma folded in. lda must be even.
template <int MAXJ>
__global__ void __launch_bounds__(256)
    k_nl_project_range(const int *__restrict__ rng_pt0, const int *__restrict__ rng_ent0,
                       const int *__restrict__ rng_item0, const int *__restrict__ item_e0,
                       const int2 *__restrict__ item_row, const int *__restrict__ pe_lp,
                       const float *__restrict__ pe_chi, const int *__restrict__ cov_pt,
                       const float *__restrict__ gamma, int ncol, const float *__restrict__ x,
                       long ldx, float *__restrict__ alpha, long lda, float dV)
{
    constexpr int NC = 64, XLD = NC + 2;             // columns per group, padded x row
    constexpr int MAXJP = (MAXJ + 3) / 4 * 4;        // staged Chi values per entry
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *xs = reinterpret_cast<float *>(smem_raw);  // [kRangePts][XLD]
    float *cs = xs + kRangePts * XLD;                 // [entries][MAXJP]
    const int r = blockIdx.x;
    const int p0 = rng_pt0[r], npt = rng_pt0[r + 1] - p0;
    const int eb = rng_ent0[r], ne = rng_ent0[r + 1] - eb;
    const int ib = rng_item0[r], ni = rng_item0[r + 1] - ib;
    int *lps = reinterpret_cast<int *>(cs + (size_t)ne * MAXJP);  // [entries]
    int *gps = lps + ne;                                          // [kRangePts]
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;

    for (int i = t; i < npt; i += 256) gps[i] = cov_pt[p0 + i];
    for (int i = t; i < ne; i += 256) lps[i] = pe_lp[eb + i];
    {
        const float4 *src = reinterpret_cast<const float4 *>(pe_chi + (long)eb * MAXJP);
        float4 *dst = reinterpret_cast<float4 *>(cs);
        for (int i = t; i < ne * (MAXJP / 4); i += 256) dst[i] = __ldg(src + i);
    }
    // column groups in an order rotated by the range index, so that neighbouring ranges (which
    // share atoms) add into different alpha columns at any one time
    const int ngroup = (ncol + NC - 1) / NC;
    for (int gi = 0; gi < ngroup; gi++) {
        const int n0 = ((gi + r) % ngroup) * NC;
        __syncthreads();  // staging done / previous group consumed
        gather_tile<XLD, NC>(x, ldx, n0, ncol, gps, npt, xs);
        __syncthreads();
        for (int it = warp; it < ni; it += 8) {
            const int2 row = item_row[ib + it];  // (first projector row, projector count)
            const int e0 = item_e0[ib + it] - eb, e1 = item_e0[ib + it + 1] - eb;
            float2 acc[MAXJ];  // (column 2l, column 2l+1) per projector, packed FMAs
#pragma unroll
            for (int j = 0; j < MAXJ; j++) acc[j] = make_float2(0.f, 0.f);
#pragma unroll 2
            for (int e = e0; e < e1; e++) {
                const float2 xv = *reinterpret_cast<const float2 *>(xs + lps[e] * XLD + 2 * lane);
                const float4 *cv = reinterpret_cast<const float4 *>(cs + (size_t)e * MAXJP);
#pragma unroll
                for (int q = 0; q < MAXJP / 4; q++) {
                    const float4 c4 = cv[q];
                    const float ce[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
                    for (int w = 0; w < 4; w++)
                        if (q * 4 + w < MAXJ)
                            acc[q * 4 + w] = __ffma2_rn(make_float2(ce[w], ce[w]), xv, acc[q * 4 + w]);
                }
            }
            const int c0 = n0 + 2 * lane;
#pragma unroll
            for (int j = 0; j < MAXJ; j++) {
                if (j < row.y) {
                    const float s = dV * gamma[row.x + j];
                    float *dst = alpha + (long)(row.x + j) * lda + c0;
                    if (c0 + 1 < ncol)  // lda and c0 are even: an 8-byte aligned pair
                        atomicAdd(reinterpret_cast<float2 *>(dst),
                                  make_float2(s * acc[j].x, s * acc[j].y));
                    else if (c0 < ncol)
                        atomicAdd(dst, s * acc[j].x);
                }
            }
        }
    }
}

// Range apply (FP32): the projection's ranges and work items run in reverse. Block = one range;
// for each group of 64 columns (rotated by the range index) it gathers the output tile of its
// points (os[point][64], one coalesced read of every covered output element), then each warp
// owns a run of consecutive points of the tile (runs with about equal entry counts, set at
// upload): it walks the work items in order and,
// for the item's entries on its points (item_wsplit gives their range per warp), lane l holds
// scale * alpha[row j, columns l and l+32] of the item's atom in registers and adds
// sum_j Chi_j alpha_j into its tile rows. The tile is then written back once: every covered
// output element is read and written once per launch, in grid order, and the additions per
// point run in a fixed order (item order).
template <int MAXJ>
__global__ void __launch_bounds__(256, 4)
    k_nl_apply_range(const int *__restrict__ rng_pt0, const int *__restrict__ rng_ent0,
                     const int *__restrict__ rng_item0, const int *__restrict__ item_wsplit,
                     const int2 *__restrict__ item_row, const int *__restrict__ pe_lp,
                     const float *__restrict__ pe_chi, const int *__restrict__ cov_pt, int ncol,
                     const float *__restrict__ alpha, long lda, float scale,
                     float *__restrict__ out, long ldo)
{
    constexpr int NC = 64, OLD = NC + 1;             // columns per group, padded tile row
    constexpr int MAXJP = (MAXJ + 3) / 4 * 4;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *cs = reinterpret_cast<float *>(smem_raw);  // [entries][MAXJP]
    const int r = blockIdx.x;
    const int p0 = rng_pt0[r], npt = rng_pt0[r + 1] - p0;
    const int eb = rng_ent0[r], ne = rng_ent0[r + 1] - eb;
    const int ib = rng_item0[r], ni = rng_item0[r + 1] - ib;
    float *os = cs + (size_t)ne * MAXJP;                          // [kRangePts][OLD]
    int *lps = reinterpret_cast<int *>(os + kRangePts * OLD);     // [entries]
    int *gps = lps + ne;                                          // [kRangePts]
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;

    for (int i = t; i < npt; i += 256) gps[i] = cov_pt[p0 + i];
    for (int i = t; i < ne; i += 256) lps[i] = pe_lp[eb + i];
    {
        const float4 *src = reinterpret_cast<const float4 *>(pe_chi + (long)eb * MAXJP);
        float4 *dst = reinterpret_cast<float4 *>(cs);
        for (int i = t; i < ne * (MAXJP / 4); i += 256) dst[i] = __ldg(src + i);
    }
    const int ngroup = (ncol + NC - 1) / NC;
    for (int gi = 0; gi < ngroup; gi++) {
        const int n0 = ((gi + r) % ngroup) * NC;
        __syncthreads();  // staging done / previous tile written back
        gather_tile<OLD, NC>(out, ldo, n0, ncol, gps, npt, os);
        __syncthreads();
        const int ca = n0 + lane, cb = n0 + lane + 32;
        // warp w owns the tile rows of its run of points (item_wsplit):
        // it walks every item but only the item's entries on its own points, so no two warps
        // write one tile row and the additions per point run in item order
        for (int it = 0; it < ni; it++) {
            const int *ws = item_wsplit + (long)(ib + it) * (kRangeWarps + 1);
            const int e0 = ws[warp] - eb, e1 = ws[warp + 1] - eb;
            if (e0 == e1) continue;
            const int2 row = item_row[ib + it];  // (first projector row, projector count)
            float2 a[MAXJ];  // scale * alpha of columns (lane, lane + 32)
#pragma unroll
            for (int j = 0; j < MAXJ; j++) {
                a[j] = make_float2(0.f, 0.f);
                if (j < row.y) {
                    const float *ar = alpha + (long)(row.x + j) * lda;
                    a[j] = make_float2(ca < ncol ? scale * __ldg(ar + ca) : 0.f,
                                       cb < ncol ? scale * __ldg(ar + cb) : 0.f);
                }
            }
#pragma unroll 4
            for (int e = e0; e < e1; e++) {  // entries are independent: four chains in flight
                const float4 *cv = reinterpret_cast<const float4 *>(cs + (size_t)e * MAXJP);
                float2 s = make_float2(0.f, 0.f);
#pragma unroll
                for (int q = 0; q < MAXJP / 4; q++) {
                    const float4 c4 = cv[q];
                    const float ce[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
                    for (int w = 0; w < 4; w++)
                        if (q * 4 + w < MAXJ) s = __ffma2_rn(make_float2(ce[w], ce[w]), a[q * 4 + w], s);
                }
                float *o = os + lps[e] * OLD;
                o[lane] += s.x;
                o[lane + 32] += s.y;
            }
        }
        __syncthreads();
#pragma unroll 8
        for (int u = 0; u < kRangePts * NC / 256; u++) {
            const int idx = t + u * 256;
            const int lp = idx % kRangePts, c = idx / kRangePts;
            if (lp < npt && n0 + c < ncol) out[(long)(n0 + c) * ldo + gps[lp]] = os[lp * OLD + c];
        }
    }
}

// Range apply with the next projection fused (FP32). The Chebyshev filter projects each new
// iterate right after the apply that finishes it, and that apply already holds the finished
// values of its range's covered points in shared memory, with the range's Chi rows staged. So
// per group of 64 columns this kernel gathers the output tile, adds scale * sum_j Chi_j
// alpha_j, writes the tile back, and then accumulates dV * Gamma * Chi^T tile per work item
// and adds it atomically into alpha_next (zeroed by the caller). Ranges partition the covered
// points, so a range's tile is final once its own apply is done; the separate projection of
// the next degree, and its read of every covered element, disappear.
//   apply: warp w owns the tile rows of its run of points (item_wsplit) as in
//     k_nl_apply_range; per element the same IEEE operations in the same item order, so the
//     output is bit-identical to k_nl_apply_range.
//   projection: per work item the entries are summed in order as in k_nl_project_range (the
//     same per-item partial sums), then added atomically.
// CPL = columns per lane. CPL 2: lane l owns columns 2l, 2l+1 and a warp takes one entry at a
// time (apply) or one work item (projection). CPL 4: lane l owns columns 4(l % 16) .. + 3, so
// each staged Chi value serves four columns and the tile moves in 16-byte pieces; the two
// half-warps take alternate entries of an item (distinct points of one image) in the apply and
// separate work items in the projection. The tuner times both.
// The range's work-item table (entry split by owning warp, projector rows, entry bounds) is
// staged in shared memory once, so an item costs the warps no dependent global loads.
constexpr int kItemFields = kRangeWarps + 5;  // wsplit[kRangeWarps + 1], row, count, e0, e1

template <int MAXJ, int CPL>
__global__ void __launch_bounds__(256, CPL == 2 ? (MAXJ <= 9 ? 4 : 2) : (MAXJ <= 9 ? 3 : 2))
    k_nl_apply_project_range(const int *__restrict__ rng_pt0, const int *__restrict__ rng_ent0,
                             const int *__restrict__ rng_item0, const int *__restrict__ item_e0,
                             const int *__restrict__ item_wsplit, const int2 *__restrict__ item_row,
                             const int *__restrict__ pe_lp, const float *__restrict__ pe_chi,
                             const int *__restrict__ cov_pt, const float *__restrict__ gamma,
                             int ncol, const float *__restrict__ alpha, long lda, float scale,
                             float *__restrict__ out, long ldo, float *__restrict__ alpha_next,
                             float dV)
{
    static_assert(CPL == 2 || CPL == 4, "two or four columns per lane");
    constexpr int NC = 64, OLD = NC + CPL;  // tile row: 64 columns + padding
    constexpr int MAXJP = (MAXJ + 3) / 4 * 4;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *cs = reinterpret_cast<float *>(smem_raw);  // [entries][MAXJP]
    const int r = blockIdx.x;
    const int p0 = rng_pt0[r], npt = rng_pt0[r + 1] - p0;
    const int eb = rng_ent0[r], ne = rng_ent0[r + 1] - eb;
    const int ib = rng_item0[r], ni = rng_item0[r + 1] - ib;
    float *os = cs + (size_t)ne * MAXJP;                          // [kRangePts][OLD]
    int *lps = reinterpret_cast<int *>(os + kRangePts * OLD);     // [entries]
    int *gps = lps + ne;                                          // [kRangePts]
    int *its = gps + kRangePts;                                   // [items][kItemFields]
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    // CPL 2: every lane on the entry, columns 2 lane, 2 lane + 1; CPL 4: half-warps
    const int half = CPL == 4 ? lane >> 4 : 0;
    const int q = CPL == 4 ? lane & 15 : lane;

    for (int i = t; i < npt; i += 256) gps[i] = cov_pt[p0 + i];
    for (int i = t; i < ne; i += 256) lps[i] = pe_lp[eb + i];
    for (int i = t; i < ni * kItemFields; i += 256) {
        const int it = i / kItemFields, f = i - it * kItemFields;
        int v;
        if (f <= kRangeWarps) v = item_wsplit[(long)(ib + it) * (kRangeWarps + 1) + f] - eb;
        else if (f == kRangeWarps + 1) v = item_row[ib + it].x;
        else if (f == kRangeWarps + 2) v = item_row[ib + it].y;
        else v = item_e0[ib + it + (f - kRangeWarps - 3)] - eb;
        its[i] = v;
    }
    {
        const float4 *src = reinterpret_cast<const float4 *>(pe_chi + (long)eb * MAXJP);
        float4 *dst = reinterpret_cast<float4 *>(cs);
        for (int i = t; i < ne * (MAXJP / 4); i += 256) dst[i] = __ldg(src + i);
    }
    const int ngroup = (ncol + NC - 1) / NC;
    for (int gi = 0; gi < ngroup; gi++) {
        const int n0 = ((gi + r) % ngroup) * NC;
        const int c0 = n0 + CPL * q;  // this lane's first column
        __syncthreads();  // staging done / previous tile written back and projected
        gather_tile<OLD, NC>(out, ldo, n0, ncol, gps, npt, os);
        __syncthreads();
        for (int it = 0; it < ni; it++) {
            const int *wi = its + it * kItemFields;
            const int e0 = wi[warp], e1 = wi[warp + 1];
            if (e0 == e1) continue;
            const int rx = wi[kRangeWarps + 1], ry = wi[kRangeWarps + 2];
            float2 alo[MAXJ], ahi[MAXJ];  // scale * alpha: columns (c0, c0+1), (c0+2, c0+3)
#pragma unroll
            for (int j = 0; j < MAXJ; j++) {
                alo[j] = ahi[j] = make_float2(0.f, 0.f);
                if (j < ry) {
                    const float *ar = alpha + (long)(rx + j) * lda + c0;
                    if (c0 + CPL - 1 < ncol) {  // lda and c0 are multiples of CPL: aligned
                        if constexpr (CPL == 4) {
                            const float4 v = __ldg(reinterpret_cast<const float4 *>(ar));
                            alo[j] = make_float2(scale * v.x, scale * v.y);
                            ahi[j] = make_float2(scale * v.z, scale * v.w);
                        } else {
                            const float2 v = __ldg(reinterpret_cast<const float2 *>(ar));
                            alo[j] = make_float2(scale * v.x, scale * v.y);
                        }
                    } else {
                        if (c0 < ncol) alo[j].x = scale * __ldg(ar);
                        if (c0 + 1 < ncol) alo[j].y = scale * __ldg(ar + 1);
                        if (CPL == 4 && c0 + 2 < ncol) ahi[j].x = scale * __ldg(ar + 2);
                    }
                }
            }
#pragma unroll 4
            for (int e = e0 + half; e < e1; e += CPL / 2) {
                const float4 *cv = reinterpret_cast<const float4 *>(cs + (size_t)e * MAXJP);
                float2 slo = make_float2(0.f, 0.f), shi = slo;
#pragma unroll
                for (int u = 0; u < MAXJP / 4; u++) {
                    const float4 c4 = cv[u];
                    const float ce[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
                    for (int w = 0; w < 4; w++)
                        if (u * 4 + w < MAXJ) {
                            slo = __ffma2_rn(make_float2(ce[w], ce[w]), alo[u * 4 + w], slo);
                            if constexpr (CPL == 4)
                                shi = __ffma2_rn(make_float2(ce[w], ce[w]), ahi[u * 4 + w], shi);
                        }
                }
                float *orow = os + lps[e] * OLD + CPL * q;
                if constexpr (CPL == 4) {
                    float4 ov = *reinterpret_cast<float4 *>(orow);
                    ov.x += slo.x;
                    ov.y += slo.y;
                    ov.z += shi.x;
                    ov.w += shi.y;
                    *reinterpret_cast<float4 *>(orow) = ov;
                } else {
                    float2 ov = *reinterpret_cast<float2 *>(orow);
                    ov.x += slo.x;
                    ov.y += slo.y;
                    *reinterpret_cast<float2 *>(orow) = ov;
                }
            }
        }
        __syncthreads();  // the tile holds the finished values of this range's points
#pragma unroll 8
        for (int u = 0; u < kRangePts * NC / 256; u++) {
            const int idx = t + u * 256;
            const int lp = idx % kRangePts, c = idx / kRangePts;
            if (lp < npt && n0 + c < ncol) out[(long)(n0 + c) * ldo + gps[lp]] = os[lp * OLD + c];
        }
        if (!alpha_next) continue;
        // work items in turn: one per warp (CPL 2) or one per half-warp (CPL 4)
        for (int it = warp * (CPL / 2) + half; it < ni; it += kRangeWarps * (CPL / 2)) {
            const int *wi = its + it * kItemFields;
            const int rx = wi[kRangeWarps + 1], ry = wi[kRangeWarps + 2];
            const int e0 = wi[kRangeWarps + 3], e1 = wi[kRangeWarps + 4];
            float2 plo[MAXJ], phi[MAXJ];
#pragma unroll
            for (int j = 0; j < MAXJ; j++) plo[j] = phi[j] = make_float2(0.f, 0.f);
#pragma unroll 2
            for (int e = e0; e < e1; e++) {
                const float *xrow = os + lps[e] * OLD + CPL * q;
                float2 xlo, xhi = make_float2(0.f, 0.f);
                if constexpr (CPL == 4) {
                    const float4 xv = *reinterpret_cast<const float4 *>(xrow);
                    xlo = make_float2(xv.x, xv.y);
                    xhi = make_float2(xv.z, xv.w);
                } else {
                    xlo = *reinterpret_cast<const float2 *>(xrow);
                }
                const float4 *cv = reinterpret_cast<const float4 *>(cs + (size_t)e * MAXJP);
#pragma unroll
                for (int u = 0; u < MAXJP / 4; u++) {
                    const float4 c4 = cv[u];
                    const float ce[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
                    for (int w = 0; w < 4; w++)
                        if (u * 4 + w < MAXJ) {
                            plo[u * 4 + w] = __ffma2_rn(make_float2(ce[w], ce[w]), xlo, plo[u * 4 + w]);
                            if constexpr (CPL == 4)
                                phi[u * 4 + w] = __ffma2_rn(make_float2(ce[w], ce[w]), xhi, phi[u * 4 + w]);
                        }
                }
            }
#pragma unroll
            for (int j = 0; j < MAXJ; j++) {
                if (j < ry) {
                    const float sj = dV * gamma[rx + j];
                    float *dst = alpha_next + (long)(rx + j) * lda + c0;
                    if (c0 + CPL - 1 < ncol) {
                        if constexpr (CPL == 4)
                            atomicAdd(reinterpret_cast<float4 *>(dst),
                                      make_float4(sj * plo[j].x, sj * plo[j].y, sj * phi[j].x,
                                                  sj * phi[j].y));
                        else
                            atomicAdd(reinterpret_cast<float2 *>(dst),
                                      make_float2(sj * plo[j].x, sj * plo[j].y));
                    } else {
                        if (c0 < ncol) atomicAdd(dst, sj * plo[j].x);
                        if (c0 + 1 < ncol) atomicAdd(dst + 1, sj * plo[j].y);
                        if (CPL == 4 && c0 + 2 < ncol) atomicAdd(dst + 2, sj * phi[j].x);
                    }
                }
            }
        }
    }
}

// Apply: one thread per covered grid point, looping over column blocks of CB; alpha rows are
// read as vectors (VW elements per load, broadcast across the warp when neighbouring points
// share an atom).
template <typename T, int CB, int VW, int NPMAX>
__global__ void __launch_bounds__(256)
    k_nl_apply(int ncov, const int *__restrict__ cov_pt, const int *__restrict__ cov_ptr,
               const long *__restrict__ ent_chi, const int4 *__restrict__ ent_meta,
               const T *__restrict__ chi, int ncol, const T *__restrict__ alpha, long lda,
               T scale, T *__restrict__ out, long ldo)
{
    using V = typename VecOf<T, VW>::type;
    const int cidx = blockIdx.x * blockDim.x + threadIdx.x;
    if (cidx >= ncov) return;
    const long p = cov_pt[cidx];
    const int e0 = cov_ptr[cidx], e1 = cov_ptr[cidx + 1];
    for (int n0 = 0; n0 < ncol; n0 += CB) {
        T acc[CB], ov[CB];
        // the output values are read first so their latency overlaps the projector sums
#pragma unroll
        for (int c = 0; c < CB; c++) {
            acc[c] = T(0);
            ov[c] = n0 + c < ncol ? out[(long)(n0 + c) * ldo + p] : T(0);
        }
        for (int e = e0; e < e1; e++) {
            const int4 meta = ent_meta[e];  // (first projector row, projector count, ndc, image)
            const int ip = meta.x, np = meta.y, ndc = meta.z;
            const T *__restrict__ ch = chi + ent_chi[e];
            T cvs[NPMAX];  // all Chi values of the entry, loads issued together
#pragma unroll
            for (int j = 0; j < NPMAX; j++) cvs[j] = j < np ? __ldg(ch + (long)j * ndc) : T(0);
#pragma unroll
            for (int j = 0; j < NPMAX; j++) {
                if (j >= np) break;
                const T cv = cvs[j];
                const V *__restrict__ al =
                    reinterpret_cast<const V *>(alpha + (long)(ip + j) * lda + n0);
#pragma unroll
                for (int c = 0; c < CB / VW; c++) {
                    const V av = __ldg(al + c);
                    const T *ae = reinterpret_cast<const T *>(&av);
#pragma unroll
                    for (int w = 0; w < VW; w++) acc[c * VW + w] += cv * ae[w];
                }
            }
        }
#pragma unroll
        for (int c = 0; c < CB; c++)
            if (n0 + c < ncol) out[(long)(n0 + c) * ldo + p] = ov[c] + scale * acc[c];
    }
}

// Apply with the Chi values hoisted: as k_nl_apply, but the Chi values and metadata of the
// point's first NE entries are loaded once into registers before the column loop, so each
// column block only reads the output block and alpha rows (L1); entries beyond the first NE
// (a few percent of points) are read per column block. Same summation order as k_nl_apply.
template <typename T, int CB, int VW, int NPMAX, int NE>
__global__ void __launch_bounds__(256)
    k_nl_apply_hoist(int ncov, const int *__restrict__ cov_pt, const int *__restrict__ cov_ptr,
                     const long *__restrict__ ent_chi, const int4 *__restrict__ ent_meta,
                     const T *__restrict__ chi, int ncol, const T *__restrict__ alpha, long lda,
                     T scale, T *__restrict__ out, long ldo)
{
    using V = typename VecOf<T, VW>::type;
    const int cidx = blockIdx.x * blockDim.x + threadIdx.x;
    if (cidx >= ncov) return;
    const long p = cov_pt[cidx];
    const int e0 = cov_ptr[cidx], e1 = cov_ptr[cidx + 1];
    T cr[NE][NPMAX];
    int ipr[NE], npr[NE];
#pragma unroll
    for (int ee = 0; ee < NE; ee++) {
        npr[ee] = 0;
        ipr[ee] = 0;
        if (e0 + ee < e1) {
            const int4 meta = ent_meta[e0 + ee];
            ipr[ee] = meta.x;
            npr[ee] = meta.y;
        }
    }
#pragma unroll
    for (int ee = 0; ee < NE; ee++) {
        const T *__restrict__ ch = chi + (e0 + ee < e1 ? ent_chi[e0 + ee] : 0);
        const int ndc = e0 + ee < e1 ? ent_meta[e0 + ee].z : 0;
#pragma unroll
        for (int j = 0; j < NPMAX; j++) cr[ee][j] = j < npr[ee] ? __ldg(ch + (long)j * ndc) : T(0);
    }
    for (int n0 = 0; n0 < ncol; n0 += CB) {
        T acc[CB], ov[CB];
#pragma unroll
        for (int c = 0; c < CB; c++) {
            acc[c] = T(0);
            ov[c] = n0 + c < ncol ? out[(long)(n0 + c) * ldo + p] : T(0);
        }
#pragma unroll
        for (int ee = 0; ee < NE; ee++) {
#pragma unroll
            for (int j = 0; j < NPMAX; j++) {
                if (j >= npr[ee]) break;
                const T cv = cr[ee][j];
                const V *__restrict__ al =
                    reinterpret_cast<const V *>(alpha + (long)(ipr[ee] + j) * lda + n0);
#pragma unroll
                for (int c = 0; c < CB / VW; c++) {
                    const V av = __ldg(al + c);
                    const T *ae = reinterpret_cast<const T *>(&av);
#pragma unroll
                    for (int w = 0; w < VW; w++) acc[c * VW + w] += cv * ae[w];
                }
            }
        }
        for (int e = e0 + NE; e < e1; e++) {
            const int4 meta = ent_meta[e];
            const int ip = meta.x, np = meta.y, ndc = meta.z;
            const T *__restrict__ ch = chi + ent_chi[e];
            T cvs[NPMAX];
#pragma unroll
            for (int j = 0; j < NPMAX; j++) cvs[j] = j < np ? __ldg(ch + (long)j * ndc) : T(0);
#pragma unroll
            for (int j = 0; j < NPMAX; j++) {
                if (j >= np) break;
                const T cv = cvs[j];
                const V *__restrict__ al =
                    reinterpret_cast<const V *>(alpha + (long)(ip + j) * lda + n0);
#pragma unroll
                for (int c = 0; c < CB / VW; c++) {
                    const V av = __ldg(al + c);
                    const T *ae = reinterpret_cast<const T *>(&av);
#pragma unroll
                    for (int w = 0; w < VW; w++) acc[c * VW + w] += cv * ae[w];
                }
            }
        }
#pragma unroll
        for (int c = 0; c < CB; c++)
            if (n0 + c < ncol) out[(long)(n0 + c) * ldo + p] = ov[c] + scale * acc[c];
    }
}

// Apply as a dense product per chunk (FP32): block = (chunk of kApplyChunk consecutive
// covered points, 64 columns), 256 threads = 128 points x 2 column halves. The alpha rows of
// the chunk's atoms (nr rows, listed in chunk_rows) and a dense Chi matrix C[nr][points]
// (zero where an atom's sphere misses a point; images of one atom over one point summed) are
// staged in shared memory, then thread (point, half) accumulates its 32 outputs over the nr
// rows: one C value and eight 16-byte alpha loads (the same for the whole warp) per 32 FMAs;
// then its 32 output values are read together and written back. Summation runs over staged
// rows, so results agree with the per-point forms to FP32 rounding.
__global__ void __launch_bounds__(256, 2)
    k_nl_apply_dense(int ncov, const int *__restrict__ cov_pt, const int *__restrict__ cov_ptr,
                     const long *__restrict__ ent_chi, const int4 *__restrict__ ent_meta,
                     const int *__restrict__ ent_slot, const int *__restrict__ chunk_row_ptr,
                     const int *__restrict__ chunk_rows, const float *__restrict__ chi, int ncol,
                     const float *__restrict__ alpha, long lda, float scale,
                     float *__restrict__ out, long ldo)
{
    constexpr int NC = 64, HC = 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int c = blockIdx.x;
    const int n0 = blockIdx.y * NC;
    const int r0 = chunk_row_ptr[c], nr = chunk_row_ptr[c + 1] - r0;
    float *As = reinterpret_cast<float *>(smem_raw);  // [nr][NC]
    float *Cs = As + (size_t)nr * NC;                 // [nr][kApplyChunk]
    const int t = threadIdx.x;
    const int pt = t % kApplyChunk, half = t / kApplyChunk;
    const int cidx = c * kApplyChunk + pt;
    const bool live = cidx < ncov;
    const long p = live ? cov_pt[cidx] : 0;
    const int cb = n0 + half * HC;
    for (int i = t; i < nr * kApplyChunk; i += 256) Cs[i] = 0.f;
    for (int i = t; i < nr * NC; i += 256) {
        const int r = i / NC, cc = i % NC;
        As[i] = n0 + cc < ncol ? alpha[(long)chunk_rows[r0 + r] * lda + n0 + cc] : 0.f;
    }
    __syncthreads();
    if (half == 0 && live) {  // one thread per point writes its column of C
        for (int e = cov_ptr[cidx]; e < cov_ptr[cidx + 1]; e++) {
            const int4 meta = ent_meta[e];
            const float *__restrict__ ch = chi + ent_chi[e];
            float *col = Cs + (size_t)ent_slot[e] * kApplyChunk + pt;
            for (int j = 0; j < meta.y; j++) col[(size_t)j * kApplyChunk] += __ldg(ch + (long)j * meta.z);
        }
    }
    __syncthreads();
    float2 acc[HC / 2];  // column pairs, packed FMAs
#pragma unroll
    for (int q = 0; q < HC / 2; q++) acc[q] = make_float2(0.f, 0.f);
    const float4 *Ah = reinterpret_cast<const float4 *>(As + half * HC);
#pragma unroll 2
    for (int k = 0; k < nr; k++) {
        const float cv = Cs[(size_t)k * kApplyChunk + pt];
        const float2 cv2 = make_float2(cv, cv);
        const float4 *a4 = Ah + (size_t)k * (NC / 4);
#pragma unroll
        for (int q = 0; q < HC / 4; q++) {
            const float4 a = a4[q];
            acc[2 * q] = __ffma2_rn(cv2, make_float2(a.x, a.y), acc[2 * q]);
            acc[2 * q + 1] = __ffma2_rn(cv2, make_float2(a.z, a.w), acc[2 * q + 1]);
        }
    }
    if (!live) return;
    float ov[HC];  // all loads of the output block in flight together
#pragma unroll
    for (int q = 0; q < HC; q++) ov[q] = cb + q < ncol ? out[(long)(cb + q) * ldo + p] : 0.f;
#pragma unroll
    for (int q = 0; q < HC; q++) {
        const float a = q % 2 ? acc[q / 2].y : acc[q / 2].x;
        if (cb + q < ncol) out[(long)(cb + q) * ldo + p] = ov[q] + scale * a;
    }
}

// Apply, staged: one block per (chunk of kApplyChunk consecutive covered points, block of CB
// columns). The alpha rows of every atom that touches the chunk are staged once in shared
// memory (rows listed in chunk_rows, each padded by 16 bytes so that rows start four banks
// apart: up to eight distinct rows per 16-byte warp read are served in one pass), and each
// thread accumulates its point's CB outputs from there with 16-byte reads; then the output
// block is read-modified-written once. Neighbouring covered points share atoms, so one staged row
// serves many threads.
template <typename T, int CB, int NPMAX>
__global__ void __launch_bounds__(kApplyChunk, 4)
    k_nl_apply_staged(int ncov, const int *__restrict__ cov_pt, const int *__restrict__ cov_ptr,
                      const long *__restrict__ ent_chi, const int4 *__restrict__ ent_meta,
                      const int *__restrict__ ent_slot, const int *__restrict__ chunk_row_ptr,
                      const int *__restrict__ chunk_rows, const T *__restrict__ chi, int ncol,
                      const T *__restrict__ alpha, long lda, T scale, T *__restrict__ out,
                      long ldo)
{
    constexpr int VW = 16 / sizeof(T);
    constexpr int LDS = CB + VW;  // padded row: consecutive rows start four banks apart
    using V = typename VecOf<T, VW>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *S = reinterpret_cast<T *>(smem_raw);  // [rows][LDS]
    const int c = blockIdx.x;
    const int n0 = blockIdx.y * CB;
    const int cidx = c * kApplyChunk + threadIdx.x;
    const bool live = cidx < ncov;
    const long p = live ? cov_pt[cidx] : 0;
    const int r0 = chunk_row_ptr[c], nr = chunk_row_ptr[c + 1] - r0;
    for (int e = threadIdx.x; e < nr * CB; e += blockDim.x) {
        const int r = e / CB, cc = e % CB;
        S[r * LDS + cc] = n0 + cc < ncol ? alpha[(long)chunk_rows[r0 + r] * lda + n0 + cc] : T(0);
    }
    __syncthreads();
    if (!live) return;
    const int e0 = cov_ptr[cidx], e1 = cov_ptr[cidx + 1];
    T acc[CB];
#pragma unroll
    for (int q = 0; q < CB; q++) acc[q] = T(0);
    for (int e = e0; e < e1; e++) {
        const int4 meta = ent_meta[e];  // (first projector row, projector count, ndc, image)
        const int np = meta.y, ndc = meta.z;
        const T *__restrict__ ch = chi + ent_chi[e];
        const T *__restrict__ srow = S + (long)ent_slot[e] * LDS;
        T cvs[NPMAX];
#pragma unroll
        for (int j = 0; j < NPMAX; j++) cvs[j] = j < np ? __ldg(ch + (long)j * ndc) : T(0);
#pragma unroll
        for (int j = 0; j < NPMAX; j++) {
            if (j >= np) break;
            const T cv = cvs[j];
            const V *sv = reinterpret_cast<const V *>(srow + j * LDS);
#pragma unroll
            for (int q = 0; q < CB / VW; q++) {
                const V a = sv[q];
                const T *ae = reinterpret_cast<const T *>(&a);
                if constexpr (sizeof(T) == 4) {  // packed pairs: same rounding per lane
#pragma unroll
                    for (int w = 0; w < VW; w += 2) {
                        const float2 r = __ffma2_rn(make_float2(cv, cv), make_float2(ae[w], ae[w + 1]),
                                                    make_float2(acc[q * VW + w], acc[q * VW + w + 1]));
                        acc[q * VW + w] = r.x;
                        acc[q * VW + w + 1] = r.y;
                    }
                } else {
#pragma unroll
                    for (int w = 0; w < VW; w++) acc[q * VW + w] += cv * ae[w];
                }
            }
        }
    }
    T ov[CB];  // the output block: all loads in flight together
#pragma unroll
    for (int q = 0; q < CB; q++) ov[q] = n0 + q < ncol ? out[(long)(n0 + q) * ldo + p] : T(0);
#pragma unroll
    for (int q = 0; q < CB; q++)
        if (n0 + q < ncol) out[(long)(n0 + q) * ldo + p] = ov[q] + scale * acc[q];
}

template <typename T>
const T *chi_of(const Nonlocal &nl);
template <>
const double *chi_of<double>(const Nonlocal &nl) { return nl.chi64; }
template <>
const float *chi_of<float>(const Nonlocal &nl) { return nl.chi32; }
template <typename T>
const T *gamma_of(const Nonlocal &nl);
template <>
const double *gamma_of<double>(const Nonlocal &nl) { return nl.gamma64; }
template <>
const float *gamma_of<float>(const Nonlocal &nl) { return nl.gamma32; }

}  // namespace

template <typename T>
static constexpr int apply_cb() { return sizeof(T) == 4 ? 16 : 8; }

long nonlocal_alpha_ld(int ncol, int elem_bytes)
{
    const int cb = elem_bytes == 4 ? 16 : 8;
    return ((long)ncol + cb - 1) / cb * cb;
}

template <typename T, int MAXJ>
static int project_launch(sgpu_ctx *ctx, int ncol, const T *x, long ldx, T *alpha, long lda,
                          const T *gamma, T dV, cudaStream_t st)
{
    constexpr int NC = sizeof(T) == 4 ? 128 : 64, PCH = 64;
    constexpr int VW = 16 / sizeof(T), MAXJP = (MAXJ + VW - 1) / VW * VW;
    constexpr int HALVES = kProjThreads / NC;
    const size_t xs_elems = std::max((size_t)NC * (PCH + 1), (size_t)HALVES * MAXJ * NC);
    const size_t smem = sizeof(T) * ((size_t)MAXJP * kSegPts + xs_elems) + sizeof(int) * kSegPts;
    auto kern = k_nl_project<T, PCH, NC, MAXJ>;
    SGPU_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    const Nonlocal &nl = ctx->nl;
    ProfScope ps(ctx, SGPU_KERNEL_NL_PROJECT, st);
    kern<<<nl.nseg, kProjThreads, smem, st>>>(
        nl.seg_img, nl.seg_start, nl.img_atom, nl.img_ndc, nl.img_off, nl.img_chi_off,
        nl.grid_pos, chi_of<T>(nl), nl.ip_displ, gamma, ncol, x, ldx, alpha, lda, dV);
    return SGPU_OK;
}

template <int MAXJ>
static int project_range_launch(sgpu_ctx *ctx, int ncol, const float *x, long ldx, float *alpha,
                                long lda, cudaStream_t st)
{
    const Nonlocal &nl = ctx->nl;
    const size_t smem = sizeof(float) * ((size_t)kRangePts * 66 + (size_t)nl.max_range_ent * nl.range_jp) +
                        sizeof(int) * ((size_t)nl.max_range_ent + kRangePts);
    auto kern = k_nl_project_range<MAXJ>;
    SGPU_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    ProfScope ps(ctx, SGPU_KERNEL_NL_PROJECT, st);
    kern<<<nl.nrange, 256, smem, st>>>(nl.rng_pt0, nl.rng_ent0, nl.rng_item0, nl.item_e0,
                                       nl.item_row, nl.pe_lp, nl.pe_chi32, nl.cov_pt, nl.gamma32,
                                       ncol, x, ldx, alpha, lda, (float)ctx->dV);
    return SGPU_OK;
}

// alpha += gamma * dV * Chi^T x with the segment kernel (the FP64 path and the plain
// projection of the force integrals)
template <typename T>
static int project_segments(sgpu_ctx *ctx, int ncol, const T *x, long ldx, T *alpha, long lda,
                            const T *gamma, T dV, cudaStream_t st)
{
    const Nonlocal &nl = ctx->nl;
    if (nl.max_np <= 9)
        SGPU_TRY(project_launch<T, 9>(ctx, ncol, x, ldx, alpha, lda, gamma, dV, st));
    else if (nl.max_np <= 18)
        SGPU_TRY(project_launch<T, 18>(ctx, ncol, x, ldx, alpha, lda, gamma, dV, st));
    else if (nl.max_np <= 32)
        SGPU_TRY(project_launch<T, 32>(ctx, ncol, x, ldx, alpha, lda, gamma, dV, st));
    else {
        set_error("nonlocal: more than 32 projectors per atom is not built");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

int launch_nonlocal_project_plain(sgpu_ctx *ctx, int ncol, const double *x, long ldx,
                                  double *alpha, long lda, const double *ones, cudaStream_t st)
{
    if (!ctx->has_nl || ctx->nl.nimg == 0 || ncol <= 0) return SGPU_OK;
    return project_segments<double>(ctx, ncol, x, ldx, alpha, lda, ones, 1.0, st);
}

template <typename T>
int launch_nonlocal_project(sgpu_ctx *ctx, int ncol, const T *x, long ldx, T *alpha, long lda,
                            cudaStream_t st)
{
    const Nonlocal &nl = ctx->nl;
    if (!ctx->has_nl || nl.nimg == 0 || ncol <= 0) return SGPU_OK;
    if constexpr (sizeof(T) == 4) {
        if (ctx->nl_project_variant == 1 && nl.nrange > 0) {
            if (nl.range_jp == 12)
                SGPU_TRY(project_range_launch<9>(ctx, ncol, x, ldx, alpha, lda, st));
            else if (nl.range_jp == 20)
                SGPU_TRY(project_range_launch<18>(ctx, ncol, x, ldx, alpha, lda, st));
            else
                SGPU_TRY(project_range_launch<32>(ctx, ncol, x, ldx, alpha, lda, st));
            SGPU_CUDA_TRY(cudaGetLastError());
            return SGPU_OK;
        }
    }
    return project_segments<T>(ctx, ncol, x, ldx, alpha, lda, gamma_of<T>(nl), (T)ctx->dV, st);
}

template <typename T>
int launch_nonlocal_apply(sgpu_ctx *ctx, int ncol, const T *alpha, long lda, double scale,
                          T *out, long ldo, cudaStream_t st)
{
    const Nonlocal &nl = ctx->nl;
    if (!ctx->has_nl || nl.ncov == 0 || ncol <= 0) return SGPU_OK;
    constexpr int CB = apply_cb<T>();
    constexpr int VW = sizeof(T) == 4 ? 4 : 2;
    constexpr int SCB = sizeof(T) == 4 ? 32 : 16;  // columns per block of the staged form
    const size_t stage = sizeof(T) * (size_t)nl.max_chunk_rows * (SCB + 16 / sizeof(T));
    if (ctx->nl_apply_variant == 1 && nl.nchunk > 0 && stage <= kApplyStageMax) {
        const dim3 sg(nl.nchunk, (ncol + SCB - 1) / SCB);
        ProfScope ps(ctx, SGPU_KERNEL_NL_APPLY, st);
#define SGPU_STAGED(NPM)                                                                     \
    {                                                                                        \
        auto kern = k_nl_apply_staged<T, SCB, NPM>;                                          \
        SGPU_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                           (int)std::max<size_t>(stage, 16)));               \
        kern<<<sg, kApplyChunk, std::max<size_t>(stage, 16), st>>>(                          \
            nl.ncov, nl.cov_pt, nl.cov_ptr, nl.ent_chi, nl.ent_meta, nl.ent_slot,            \
            nl.chunk_row_ptr, nl.chunk_rows, chi_of<T>(nl), ncol, alpha, lda, (T)scale, out, \
            ldo);                                                                            \
    }
        if (nl.max_np <= 9)
            SGPU_STAGED(9)
        else if (nl.max_np <= 18)
            SGPU_STAGED(18)
        else
            SGPU_STAGED(32)
#undef SGPU_STAGED
        SGPU_CUDA_TRY(cudaGetLastError());
        return SGPU_OK;
    }
    if constexpr (sizeof(T) == 4) {
        if (ctx->nl_apply_variant == 4 && nl.nrange > 0) {
            const size_t rsm = sizeof(float) * ((size_t)nl.max_range_ent * nl.range_jp +
                                                (size_t)kRangePts * 65) +
                               sizeof(int) * ((size_t)nl.max_range_ent + kRangePts);
            ProfScope ps(ctx, SGPU_KERNEL_NL_APPLY, st);
#define SGPU_RAPPLY(MJ)                                                                      \
    {                                                                                        \
        auto kern = k_nl_apply_range<MJ>;                                                    \
        SGPU_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                           (int)rsm));                                       \
        kern<<<nl.nrange, 256, rsm, st>>>(nl.rng_pt0, nl.rng_ent0, nl.rng_item0, nl.item_wsplit, \
                                          nl.item_row, nl.pe_lp, nl.pe_chi32, nl.cov_pt,     \
                                          ncol, alpha, lda, (float)scale, out, ldo);         \
    }
            if (nl.range_jp == 12)
                SGPU_RAPPLY(9)
            else if (nl.range_jp == 20)
                SGPU_RAPPLY(18)
            else
                SGPU_RAPPLY(32)
#undef SGPU_RAPPLY
            SGPU_CUDA_TRY(cudaGetLastError());
            return SGPU_OK;
        }
        const size_t dsm = sizeof(float) * (size_t)nl.max_chunk_rows * (64 + kApplyChunk);
        if (ctx->nl_apply_variant == 3 && nl.nchunk > 0 && dsm <= kApplyDenseMax) {
            SGPU_CUDA_TRY(cudaFuncSetAttribute(k_nl_apply_dense,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)std::max<size_t>(dsm, 16)));
            const dim3 dg(nl.nchunk, (ncol + 63) / 64);
            ProfScope ps(ctx, SGPU_KERNEL_NL_APPLY, st);
            k_nl_apply_dense<<<dg, 256, std::max<size_t>(dsm, 16), st>>>(
                nl.ncov, nl.cov_pt, nl.cov_ptr, nl.ent_chi, nl.ent_meta, nl.ent_slot,
                nl.chunk_row_ptr, nl.chunk_rows, nl.chi32, ncol, alpha, lda, (float)scale, out,
                ldo);
            SGPU_CUDA_TRY(cudaGetLastError());
            return SGPU_OK;
        }
    }
    const dim3 grid((nl.ncov + 255) / 256);
    ProfScope ps(ctx, SGPU_KERNEL_NL_APPLY, st);
    if (ctx->nl_apply_variant == 2) {
#define SGPU_HOIST(NPM, NE)                                                                  \
    k_nl_apply_hoist<T, CB, VW, NPM, NE><<<grid, 256, 0, st>>>(                              \
        nl.ncov, nl.cov_pt, nl.cov_ptr, nl.ent_chi, nl.ent_meta, chi_of<T>(nl), ncol, alpha, \
        lda, (T)scale, out, ldo)
        if (nl.max_np <= 9)
            SGPU_HOIST(9, 2);
        else if (nl.max_np <= 18)
            SGPU_HOIST(18, 1);
        else
            SGPU_HOIST(32, 1);
#undef SGPU_HOIST
        SGPU_CUDA_TRY(cudaGetLastError());
        return SGPU_OK;
    }
#define SGPU_APPLY(NPM)                                                                      \
    k_nl_apply<T, CB, VW, NPM><<<grid, 256, 0, st>>>(nl.ncov, nl.cov_pt, nl.cov_ptr,         \
                                                     nl.ent_chi, nl.ent_meta, chi_of<T>(nl), \
                                                     ncol, alpha, lda, (T)scale, out, ldo)
    if (nl.max_np <= 9)
        SGPU_APPLY(9);
    else if (nl.max_np <= 18)
        SGPU_APPLY(18);
    else
        SGPU_APPLY(32);
#undef SGPU_APPLY
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

template int launch_nonlocal_project<double>(sgpu_ctx *, int, const double *, long, double *,
                                             long, cudaStream_t);
template int launch_nonlocal_project<float>(sgpu_ctx *, int, const float *, long, float *, long,
                                            cudaStream_t);
int launch_nonlocal_apply_project(sgpu_ctx *ctx, int ncol, const float *alpha, long lda,
                                  double scale, float *out, long ldo, float *alpha_next,
                                  cudaStream_t st)
{
    const Nonlocal &nl = ctx->nl;
    if (!ctx->has_nl || nl.ncov == 0 || ncol <= 0) return SGPU_OK;
    if (nl.nrange == 0) {
        set_error("nonlocal: the fused apply needs the range tables (none built)");
        return SGPU_ERR_STATE;
    }
    if (ctx->nl_fuse_cpl == 3)
        return launch_nonlocal_apply_project_tc(ctx, ncol, alpha, lda, scale, out, ldo,
                                                alpha_next, st);
    const int cpl = ctx->nl_fuse_cpl == 4 ? 4 : 2;
    const size_t rsm = sizeof(float) * ((size_t)nl.max_range_ent * nl.range_jp +
                                        (size_t)kRangePts * (64 + cpl)) +
                       sizeof(int) * ((size_t)nl.max_range_ent + kRangePts +
                                      (size_t)nl.max_range_items * kItemFields);
    ProfScope ps(ctx, SGPU_KERNEL_NL_APPLY, st);
#define SGPU_FAPPLY(MJ, CPL)                                                                 \
    {                                                                                        \
        auto kern = k_nl_apply_project_range<MJ, CPL>;                                       \
        SGPU_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                           (int)rsm));                                       \
        kern<<<nl.nrange, 256, rsm, st>>>(nl.rng_pt0, nl.rng_ent0, nl.rng_item0, nl.item_e0, \
                                          nl.item_wsplit, nl.item_row, nl.pe_lp, nl.pe_chi32, \
                                          nl.cov_pt, nl.gamma32, ncol, alpha, lda,           \
                                          (float)scale, out, ldo, alpha_next,                \
                                          (float)ctx->dV);                                   \
    }
    if (cpl == 4) {
        if (nl.range_jp == 12)
            SGPU_FAPPLY(9, 4)
        else if (nl.range_jp == 20)
            SGPU_FAPPLY(18, 4)
        else
            SGPU_FAPPLY(32, 4)
    } else {
        if (nl.range_jp == 12)
            SGPU_FAPPLY(9, 2)
        else if (nl.range_jp == 20)
            SGPU_FAPPLY(18, 2)
        else
            SGPU_FAPPLY(32, 2)
    }
#undef SGPU_FAPPLY
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

template int launch_nonlocal_apply<double>(sgpu_ctx *, int, const double *, long, double,
                                           double *, long, cudaStream_t);
template int launch_nonlocal_apply<float>(sgpu_ctx *, int, const float *, long, double, float *,
                                          long, cudaStream_t);

void nonlocal_free(Nonlocal &nl)
{
    void *ptrs[] = {nl.ip_displ, nl.img_atom, nl.img_ndc, nl.img_off, nl.img_chi_off,
                    nl.grid_pos, nl.chi64,    nl.chi32,   nl.gamma64, nl.gamma32,
                    nl.cov_pt,   nl.cov_ptr,  nl.ent_chi, nl.ent_meta, nl.seg_img,
                    nl.seg_start, nl.ent_slot, nl.chunk_row_ptr, nl.chunk_rows,
                    nl.rng_pt0,  nl.rng_ent0, nl.rng_item0, nl.item_e0, nl.item_row,
                    nl.item_wsplit,
                    nl.pe_lp,    nl.pe_chi32, nl.tc_pt0, nl.tc_pts, nl.tc_row0, nl.tc_rows,
                    nl.tc_ent0,  nl.tc_ent,   nl.tc_chi};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    nl = Nonlocal();
}

namespace {
template <typename T>
int upload(T **dst, const T *src, size_t n)
{
    SGPU_CUDA_TRY(cudaMalloc((void **)dst, sizeof(T) * (n > 0 ? n : 1)));
    if (n > 0) SGPU_CUDA_TRY(cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice));
    return SGPU_OK;
}
}  // namespace

int nonlocal_upload(sgpu_ctx *ctx, int natom, const int *ip_displ, const double *gamma,
                    int nimg, const int *img_atom, const int *img_ndc, const int *grid_pos,
                    const double *chi)
{
    Nonlocal nl;
    nl.natom = natom;
    nl.nimg = nimg;
    nl.ntot = ip_displ[natom];
    for (int a = 0; a < natom; a++) {
        const int np = ip_displ[a + 1] - ip_displ[a];
        if (np < 0) {
            set_error("set_nonlocal: ip_displ must be non-decreasing");
            return SGPU_ERR_ARG;
        }
        nl.max_np = std::max(nl.max_np, np);
    }
    std::vector<long> off(nimg), chioff(nimg);
    long npos = 0, nchi = 0;
    for (int g = 0; g < nimg; g++) {
        if (img_atom[g] < 0 || img_atom[g] >= natom || img_ndc[g] < 0) {
            set_error("set_nonlocal: image " + std::to_string(g) + " has a bad atom or size");
            return SGPU_ERR_ARG;
        }
        off[g] = npos;
        chioff[g] = nchi;
        npos += img_ndc[g];
        nchi += (long)img_ndc[g] * (ip_displ[img_atom[g] + 1] - ip_displ[img_atom[g]]);
    }
    for (long i = 0; i < npos; i++) {
        if (grid_pos[i] < 0 || grid_pos[i] >= ctx->Nd) {
            set_error("set_nonlocal: grid position out of range");
            return SGPU_ERR_ARG;
        }
    }
    nl.npos = npos;
    nl.nchi = nchi;

    // point CSR: entries (image, local index) bucketed by grid point
    std::vector<int> count(ctx->Nd + 1, 0);
    for (long i = 0; i < npos; i++) count[grid_pos[i] + 1]++;
    std::vector<int> covpts;
    std::vector<int> covptr(1, 0);
    for (long p = 0; p < ctx->Nd; p++) {
        if (count[p + 1] > 0) {
            covpts.push_back((int)p);
            covptr.push_back(covptr.back() + count[p + 1]);
        }
    }
    std::vector<int> slot(ctx->Nd, -1);
    for (size_t c = 0; c < covpts.size(); c++) slot[covpts[c]] = covptr[c];
    std::vector<long> ent_chi(npos);
    std::vector<int4> ent_meta(npos);
    for (int g = 0; g < nimg; g++) {
        const int a = img_atom[g];
        const int ip = ip_displ[a], np = ip_displ[a + 1] - ip_displ[a];
        for (int ii = 0; ii < img_ndc[g]; ii++) {
            const int p = grid_pos[off[g] + ii];
            const int e = slot[p]++;
            ent_chi[e] = chioff[g] + ii;
            ent_meta[e] = make_int4(ip, np, img_ndc[g], g);
        }
    }
    nl.ncov = (int)covpts.size();
    nl.nent = npos;
    // staged apply: per chunk of kApplyChunk covered points, the alpha rows of the atoms its
    // entries use (each atom once) and, per entry, the staged row of its atom's first projector
    std::vector<int> chunk_row_ptr(1, 0), chunk_rows, ent_slot(npos, 0);
    nl.nchunk = (nl.ncov + kApplyChunk - 1) / kApplyChunk;
    {
        std::vector<int> atom_slot(natom, -1), touched;
        for (int c = 0; c < nl.nchunk; c++) {
            const int p0 = c * kApplyChunk, p1 = std::min(nl.ncov, p0 + kApplyChunk);
            int rows = 0;
            for (int e = covptr[p0]; e < covptr[p1]; e++) {
                const int ip = ent_meta[e].x, np = ent_meta[e].y;
                const int a = (int)(std::upper_bound(ip_displ, ip_displ + natom + 1, ip) -
                                    ip_displ) - 1;
                if (atom_slot[a] < 0) {
                    atom_slot[a] = rows;
                    touched.push_back(a);
                    for (int j = 0; j < np; j++) chunk_rows.push_back(ip + j);
                    rows += np;
                }
                ent_slot[e] = atom_slot[a];
            }
            for (int a : touched) atom_slot[a] = -1;
            touched.clear();
            chunk_row_ptr.push_back((int)chunk_rows.size());
            nl.max_chunk_rows = std::max(nl.max_chunk_rows, rows);
        }
    }
    // range projection: ranges of at most kRangePts consecutive covered points and
    // kRangeMaxEnt entries; within a range the entries are regrouped by image (then by point)
    // into work items of at most kRangeItemEnt entries, with their Chi rows in FP32
    std::vector<int> rng_pt0(1, 0), rng_ent0(1, 0), rng_item0(1, 0), item_e0(1, 0), pe_lp,
        item_wsplit;
    std::vector<int2> item_row;
    std::vector<float> pe_chi;
    {
        const int mj = nl.max_np <= 9 ? 9 : nl.max_np <= 18 ? 18 : 32;
        nl.range_jp = (mj + 3) / 4 * 4;
        pe_chi.reserve((size_t)npos * nl.range_jp);
        pe_lp.reserve(npos);
        std::vector<std::pair<long, int>> order;  // (image * Nd-span key, entry)
        int p = 0;
        while (p < nl.ncov) {
            const int q0 = p;
            int ents = 0;
            while (p < nl.ncov && p - q0 < kRangePts &&
                   ents + (covptr[p + 1] - covptr[p]) <= kRangeMaxEnt) {
                ents += covptr[p + 1] - covptr[p];
                p++;
            }
            if (p == q0) {
                set_error("set_nonlocal: more than " + std::to_string(kRangeMaxEnt) +
                          " projector spheres overlap at one grid point");
                return SGPU_ERR_ARG;
            }
            // the apply's owner warps: contiguous runs of the range's points with about equal
            // entry counts (a range cut by the entry cap holds fewer than kRangePts points)
            int wb[kRangeWarps + 1];
            {
                const long tot = covptr[p] - covptr[q0];
                int c = q0;
                wb[0] = 0;
                for (int w = 1; w < kRangeWarps; w++) {
                    const long target = tot * w / kRangeWarps;
                    while (c < p && covptr[c] - covptr[q0] < target) c++;
                    wb[w] = c - q0;
                }
                wb[kRangeWarps] = p - q0;
            }
            order.clear();
            for (int e = covptr[q0]; e < covptr[p]; e++) order.push_back({(long)ent_meta[e].w, e});
            // entries are already in point order; a stable sort by image keeps it per image
            std::stable_sort(order.begin(), order.end(),
                             [](const std::pair<long, int> &a, const std::pair<long, int> &b) {
                                 return a.first < b.first;
                             });
            size_t k = 0;
            while (k < order.size()) {
                const int g = (int)order[k].first;
                size_t k1 = k;
                while (k1 < order.size() && order[k1].first == g &&
                       (int)(k1 - k) < kRangeItemEnt)
                    k1++;
                const int4 meta = ent_meta[order[k].second];
                item_row.push_back(make_int2(meta.x, meta.y));
                const int first = (int)pe_lp.size();
                for (size_t u = k; u < k1; u++) {
                    const int e = order[u].second;
                    // the local point: entries of point c lie in [covptr[c], covptr[c+1])
                    const int c = (int)(std::upper_bound(covptr.begin() + q0, covptr.begin() + p + 1,
                                                         e) - covptr.begin()) - 1;
                    pe_lp.push_back(c - q0);
                    const int4 m = ent_meta[e];
                    for (int j = 0; j < nl.range_jp; j++)
                        pe_chi.push_back(j < m.y ? (float)chi[ent_chi[e] + (long)j * m.z] : 0.f);
                }
                item_e0.push_back((int)pe_lp.size());
                // the item's entries by owning warp: points ascend within the item
                for (int w = 0, e = first; w <= kRangeWarps; w++) {
                    while (e < (int)pe_lp.size() && (w == kRangeWarps || pe_lp[e] < wb[w])) e++;
                    item_wsplit.push_back(e);
                }
                k = k1;
            }
            rng_pt0.push_back(p);
            rng_ent0.push_back((int)pe_lp.size());
            nl.max_range_items = std::max(nl.max_range_items,
                                          (int)item_row.size() - rng_item0.back());
            rng_item0.push_back((int)item_row.size());
            nl.max_range_ent = std::max(nl.max_range_ent, ents);
        }
        nl.nrange = (int)rng_pt0.size() - 1;
        nl.nitem = (int)item_row.size();
    }
    // projection work split: segments of at most kSegPts points per image
    std::vector<int> seg_img, seg_start;
    for (int g = 0; g < nimg; g++)
        for (int s0 = 0; s0 < img_ndc[g]; s0 += kSegPts) {
            seg_img.push_back(g);
            seg_start.push_back(s0);
        }
    nl.nseg = (int)seg_img.size();

    std::vector<float> chi32(nchi), gamma32(nl.ntot);
    for (long i = 0; i < nchi; i++) chi32[i] = (float)chi[i];
    for (int i = 0; i < nl.ntot; i++) gamma32[i] = (float)gamma[i];

    int rc = SGPU_OK;
#define UP(dst, src, n)                                                                      \
    if (rc == SGPU_OK) rc = upload(&nl.dst, src, n)
    UP(ip_displ, ip_displ, (size_t)natom + 1);
    UP(img_atom, img_atom, (size_t)nimg);
    UP(img_ndc, img_ndc, (size_t)nimg);
    UP(img_off, off.data(), (size_t)nimg);
    UP(img_chi_off, chioff.data(), (size_t)nimg);
    UP(grid_pos, grid_pos, (size_t)npos);
    UP(chi64, chi, (size_t)nchi);
    UP(chi32, chi32.data(), (size_t)nchi);
    UP(gamma64, gamma, (size_t)nl.ntot);
    UP(gamma32, gamma32.data(), (size_t)nl.ntot);
    UP(cov_pt, covpts.data(), covpts.size());
    UP(cov_ptr, covptr.data(), covptr.size());
    UP(ent_chi, ent_chi.data(), ent_chi.size());
    UP(ent_meta, ent_meta.data(), ent_meta.size());
    UP(seg_img, seg_img.data(), seg_img.size());
    UP(seg_start, seg_start.data(), seg_start.size());
    UP(ent_slot, ent_slot.data(), ent_slot.size());
    UP(chunk_row_ptr, chunk_row_ptr.data(), chunk_row_ptr.size());
    UP(chunk_rows, chunk_rows.data(), chunk_rows.size());
    UP(rng_pt0, rng_pt0.data(), rng_pt0.size());
    UP(rng_ent0, rng_ent0.data(), rng_ent0.size());
    UP(rng_item0, rng_item0.data(), rng_item0.size());
    UP(item_e0, item_e0.data(), item_e0.size());
    UP(item_wsplit, item_wsplit.data(), item_wsplit.size());
    UP(item_row, item_row.data(), item_row.size());
    UP(pe_lp, pe_lp.data(), pe_lp.size());
    UP(pe_chi32, pe_chi.data(), pe_chi.size());
#undef UP
    if (rc == SGPU_OK)
        rc = nonlocal_tc_build(nl, ctx->Nx, ctx->Ny, covpts, covptr, ent_chi, ent_meta, chi);
    if (rc != SGPU_OK) {
        nonlocal_free(nl);
        return rc;
    }
    nonlocal_free(ctx->nl);
    ctx->nl = nl;
    ctx->has_nl = true;
    // a tensor-core fused form chosen for an earlier projector set needs tables this set may
    // not have: the CUDA-core form then takes over until the next tuning
    if (ctx->nl_fuse_cpl == 3 && nl.tc_nrange == 0) ctx->nl_fuse_cpl = 2;
    return SGPU_OK;
}

}  // namespace sgpu
