// k-point (Bloch) twins of the hot path: complex stencil with Bloch phases at the periodic
// faces, complex nonlocal apply with a Bloch factor per atom image, complex Chebyshev filter.
//
// Reference:
//   Lap_plus_diag_vec_mult_orth_kpt  src/lapVecRoutinesKpt.c:179-518 (ghost copies multiplied
//                                    by e^{-ikL} left of the cell, e^{+ikL} right of it, :370-460)
//   Vnl_vec_mult_kpt                 src/nlocVecRoutines.c:889-999 (alpha += e^{i theta} dV
//                                    Chiᵀ x, Hx += e^{-i theta} Chi alpha, theta = -k.(image shift))
//   Hamiltonian_vectors_mult_kpt     src/hamiltonianVecRoutines.c:132
//   ChebyshevFiltering_kpt           src/eigenSolverKpt.c:458-550
//
// Orbital blocks are complex (interleaved re, im; double2 for complex128, float2 for
// complex64) with the reference's column-major layout. The stencil loads every value at its
// unwrapped position: a value fetched across a periodic face is the wrapped grid value times
// e^{i k.(face shift)}, so the tile loader needs no ghost copy.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "sgpu_internal.h"
#include "zmath.cuh"
#include "zstencil_c64.cuh"

namespace sgpu {
namespace {

using zm::Real;
using zm::cmul;
using zm::cadd;
using zm::cscale;
using zm::wrapz;
using zm::floordiv;
using zm::phase;

struct KParams {
    double kLx, kLy, kLz;  // k_d * L_d
};

template <typename CT>
struct StencilZParams {
    const CT *__restrict__ x;
    CT *__restrict__ out;
    const CT *__restrict__ z;
    const double *__restrict__ v;  // real potential in FP64 (complex128) ...
    const float *__restrict__ v32; // ... or FP32 (complex64)
    long ldx, ldo, ldz;
    int Nx, Ny, Nz, nslab, zlen;
    double wx[kMaxFDn + 1], wy[kMaxFDn + 1], wz[kMaxFDn + 1];
    double c0, bv, s1, s2;
    KParams k;
};

// One point per thread, z-register queue with the plane k+R+1 in flight, the current plane
// plus its x/y halo in shared memory (two buffers, one barrier per plane), halo / potential /
// recurrence-term values for the next plane prefetched into registers one plane ahead (the
// scheme of the real FP64 kernel). Every fetched value is multiplied by the Bloch factor of its
// unwrapped position. The tile is blockDim.x x blockDim.y (chosen per grid by zstencil_tile so
// that small grids waste few threads), both at least R; the shared planes are dynamic.
template <typename CT>
struct ZW {  // FP32 copies of the FD weights and scalars, converted once per thread
    float wx[kMaxFDn + 1], wy[kMaxFDn + 1], wz[kMaxFDn + 1], c0, s1, s2, bv;
};

template <typename CT, int R>
__device__ __forceinline__ void stencil_z_body(const StencilZParams<CT> &p, int col, int slab)
{
    using RT = typename Real<CT>::type;
    extern __shared__ __align__(16) unsigned char zst_raw[];
    const int BX = blockDim.x, BY = blockDim.y;
    const int SW = BX + 2 * R, SP = (BY + 2 * R) * SW;  // shared row length, plane size
    CT *sp = reinterpret_cast<CT *>(zst_raw);             // [2][BY + 2R][BX + 2R]
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    const int zs = slab * p.zlen;
    const int ze = min(zs + p.zlen, p.Nz);
    if (zs >= ze) return;
    // complex64 works with FP32 copies of the weights (no FP64 conversion per use); complex128
    // reads them from the kernel parameters directly
    constexpr bool F32 = sizeof(RT) == 4;
    ZW<CT> w{};  // filled for complex64 blocks only
    if constexpr (F32) {
#pragma unroll
        for (int r = 0; r <= R; r++) {
            w.wx[r] = (float)p.wx[r]; w.wy[r] = (float)p.wy[r]; w.wz[r] = (float)p.wz[r];
        }
        w.c0 = (float)p.c0; w.s1 = (float)p.s1; w.s2 = (float)p.s2; w.bv = (float)p.bv;
    }
    auto WX = [&](int r) -> RT { if constexpr (F32) return w.wx[r]; else return p.wx[r]; };
    auto WY = [&](int r) -> RT { if constexpr (F32) return w.wy[r]; else return p.wy[r]; };
    auto WZ = [&](int r) -> RT { if constexpr (F32) return w.wz[r]; else return p.wz[r]; };
    const RT c0 = F32 ? (RT)w.c0 : (RT)p.c0, s1 = F32 ? (RT)w.s1 : (RT)p.s1;
    const RT s2 = F32 ? (RT)w.s2 : (RT)p.s2, bvr = F32 ? (RT)w.bv : (RT)p.bv;
    const int i = x0 + tx, j = y0 + ty;
    const bool active = (i < p.Nx) && (j < p.Ny);
    const int gi = wrapz(i, p.Nx), gj = wrapz(j, p.Ny);
    const long NxNy = (long)p.Nx * p.Ny;
    const CT *__restrict__ xc = p.x + (long)col * p.ldx;
    const CT *__restrict__ zc = p.z ? p.z + (long)col * p.ldz : nullptr;
    CT *__restrict__ oc = p.out + (long)col * p.ldo;
    const long own = gi + (long)gj * p.Nx;
    // Bloch factors of the thread's own column and of its halo sources (x/y shifts)
    const CT f_own = phase<CT>(floordiv(i, p.Nx) * p.k.kLx + floordiv(j, p.Ny) * p.k.kLy);
    const bool hx = tx < R, hy = ty < R;
    long hxl = 0, hxr = 0, hyl = 0, hyr = 0;
    CT f_xl{1, 0}, f_xr{1, 0}, f_yl{1, 0}, f_yr{1, 0};
    if (hx) {
        const int il = x0 - R + tx, ir = x0 + BX + tx;
        hxl = wrapz(il, p.Nx) + (long)gj * p.Nx;
        hxr = wrapz(ir, p.Nx) + (long)gj * p.Nx;
        f_xl = phase<CT>(floordiv(il, p.Nx) * p.k.kLx + floordiv(j, p.Ny) * p.k.kLy);
        f_xr = phase<CT>(floordiv(ir, p.Nx) * p.k.kLx + floordiv(j, p.Ny) * p.k.kLy);
    }
    if (hy) {
        const int jl = y0 - R + ty, jr = y0 + BY + ty;
        hyl = gi + (long)wrapz(jl, p.Ny) * p.Nx;
        hyr = gi + (long)wrapz(jr, p.Ny) * p.Nx;
        f_yl = phase<CT>(floordiv(i, p.Nx) * p.k.kLx + floordiv(jl, p.Ny) * p.k.kLy);
        f_yr = phase<CT>(floordiv(i, p.Nx) * p.k.kLx + floordiv(jr, p.Ny) * p.k.kLy);
    }
    // the z-shift factor of a plane is one of e^{-ikLz}, 1, e^{+ikLz} (the queue reaches at
    // most one period beyond the cell), so the three products with f_own are formed once
    const CT fz_m = cmul(f_own, phase<CT>(-p.k.kLz)), fz_p = cmul(f_own, phase<CT>(p.k.kLz));
    auto zload = [&](int kr) {  // own column at unwrapped plane kr
        const CT val = __ldg(xc + own + (long)wrapz(kr, p.Nz) * NxNy);
        const int d = floordiv(kr, p.Nz);
        const CT f = d == 0 ? f_own
                   : d == -1 ? fz_m
                   : d == 1 ? fz_p : cmul(f_own, phase<CT>(d * p.k.kLz));
        return cmul(val, f);
    };
    CT q[2 * R + 2];  // q[m] = plane k - R + m; q[2R+1] (plane k+R+1) is in flight
#pragma unroll
    for (int m = 0; m <= 2 * R; m++) q[m] = zload(zs - R + m);
    CT h0{0, 0}, h1{0, 0}, h2{0, 0}, h3{0, 0}, vv{0, 0}, zz{0, 0};
    auto prefetch = [&](int k) {  // halo, potential and recurrence term of plane k
        const long pk = (long)k * NxNy;
        if (hx) { h0 = cmul(__ldg(xc + pk + hxl), f_xl); h1 = cmul(__ldg(xc + pk + hxr), f_xr); }
        if (hy) { h2 = cmul(__ldg(xc + pk + hyl), f_yl); h3 = cmul(__ldg(xc + pk + hyr), f_yr); }
        if (p.v) vv.x = (RT)(p.bv * p.v[own + pk]);
        if (p.v32) vv.x = bvr * p.v32[own + pk];
        if (zc) zz = zc[own + pk];
    };
    prefetch(zs);
    for (int k = zs; k < ze; k++) {
        CT *s = sp + (k & 1) * SP;
        q[2 * R + 1] = zload(k + R + 1);
        s[(ty + R) * SW + tx + R] = q[R];
        if (hx) { s[(ty + R) * SW + tx] = h0; s[(ty + R) * SW + tx + BX + R] = h1; }
        if (hy) { s[ty * SW + tx + R] = h2; s[(ty + BY + R) * SW + tx + R] = h3; }
        const RT vcur = vv.x;
        const CT zcur = zz;
        if (k + 1 < ze) prefetch(k + 1);
        __syncthreads();
        if (active) {
            // three independent chains (x, y, z) of fused multiply-adds per component
            CT rx = cscale(q[R], c0), ry{0, 0}, rz{0, 0};
            const CT *srow = s + (ty + R) * SW + tx + R;
#pragma unroll
            for (int r = 1; r <= R; r++) {
                const CT sx = cadd(srow[-r], srow[r]);
                const CT sy = cadd(srow[-r * SW], srow[r * SW]);
                const CT sz = cadd(q[R - r], q[R + r]);
                const RT a = WX(r), b = WY(r), c = WZ(r);
                rx.x = fma(sx.x, a, rx.x); rx.y = fma(sx.y, a, rx.y);
                ry.x = fma(sy.x, b, ry.x); ry.y = fma(sy.y, b, ry.y);
                rz.x = fma(sz.x, c, rz.x); rz.y = fma(sz.y, c, rz.y);
            }
            CT res = cadd(rx, cadd(ry, rz));
            if (p.v || p.v32) res = cadd(res, cscale(q[R], vcur));
            CT o = cscale(res, s1);
            if (zc) o = cadd(o, cscale(zcur, s2));
            oc[own + (long)k * NxNy] = o;
        }
#pragma unroll
        for (int m = 0; m <= 2 * R; m++) q[m] = q[m + 1];
    }
}

constexpr int kPairMaxThreads = 320;

template <int R>
__global__ void __launch_bounds__(kPairMaxThreads)
    k_stencil_z_c64(const __grid_constant__ ZPairConst g, const ZPairParams p)
{
    stencil_c64_pairs<R>(g, p, blockIdx.z / g.nslab, blockIdx.z % g.nslab);
}

// Tile of the pair kernel: BX (even, points) with the least padding of Nx, then BY with
// the least padding of Ny among the heights that keep the block within kPairMaxThreads.
static void zpair_tile(int Nx, int Ny, int R, int *bx2, int *by)
{
    int best = 1 << 30;
    *bx2 = 16;
    for (int t = std::min(32, std::max(4, (Nx + 1) / 2)); t >= 4; t--) {
        const int waste = (Nx + 2 * t - 1) / (2 * t) * (2 * t) - Nx;
        if (waste < best) { best = waste; *bx2 = t; }
    }
    best = 1 << 30;
    *by = R;
    for (int t = std::max(R, kPairMaxThreads / *bx2); t >= R; t--) {
        if (*bx2 * t > kPairMaxThreads) continue;
        const int waste = (Ny + t - 1) / t * t - Ny;
        if (waste < best) { best = waste; *by = t; }
    }
}

// The pair kernel applies when every fetch is within one period of the cell and the pairs are
// 16-byte aligned.
static bool zpair_ok(int Nx, int Ny, int Nz, int R, int bx2, int by)
{
    const int BX = 2 * bx2;
    const int tx = (Nx + BX - 1) / BX, ty = (Ny + by - 1) / by;
    const ZRing z = zring_shape(bx2, by, R, kPairAhead);
    return Nx % 2 == 0 && R % 2 == 0 && R < Nx && R < Ny && R < Nz &&
           tx * BX + R <= 2 * Nx && ty * by + R <= 2 * Ny &&
           z.ncopy <= kPairCopies * bx2 * by && z.bytes <= 200 * 1024;
}

static size_t zpair_smem(int bx2, int by, int R)
{
    return zring_shape(bx2, by, R, kPairAhead).bytes;
}

// Threads per block of the complex stencil: complex128 (FP64-pipe bound, more registers per
// point) at most 256, complex64 at most 512.
template <typename CT>
__host__ __device__ constexpr int zstencil_threads() { return sizeof(CT) == 16 ? 256 : 512; }

// Tile of the complex stencil for an Nx x Ny plane: the widest x extent in [16, 64] with the
// least padding, then the tallest y extent in [R, maxt / bx] with the least padding.
static void zstencil_tile(int Nx, int Ny, int R, int maxt, int *bx, int *by)
{
    int best = 1 << 30;
    *bx = 32;
    for (int t = std::min(64, std::max(16, Nx)); t >= 16; t--) {
        const int waste = (Nx + t - 1) / t * t - Nx;
        if (waste < best) { best = waste; *bx = t; }
    }
    best = 1 << 30;
    *by = R;
    for (int t = std::max(R, maxt / *bx); t >= R; t--) {
        if (*bx * t > maxt) continue;
        const int waste = (Ny + t - 1) / t * t - Ny;
        if (waste < best) { best = waste; *by = t; }
    }
}

template <typename CT>
static size_t zstencil_smem(int bx, int by, int R)
{
    return sizeof(CT) * 2 * (size_t)(bx + 2 * R) * (by + 2 * R);
}

template <typename CT, int R>
__global__ void __launch_bounds__(zstencil_threads<CT>()) k_stencil_z(const StencilZParams<CT> p)
{
    stencil_z_body<CT, R>(p, blockIdx.z / p.nslab, blockIdx.z % p.nslab);
}

// projection: block = (atom image g, group of 32 columns), threads stride over the image's
// points; alpha[row * lda + n] += e^{i theta_g} dV Gamma_row sum_i Chi[i, j] x[gp_i, n]
constexpr int kProjCols = 32;
template <typename CT, int MAXJ>
__device__ __forceinline__ void nl_project_z_body(
    const int *__restrict__ img_atom, const int *__restrict__ img_ndc,
    const long *__restrict__ img_off, const long *__restrict__ img_chi_off,
    const int *__restrict__ grid_pos, const double *__restrict__ chi,
    const int *__restrict__ ip_displ, const double *__restrict__ gamma,
    const double2 *__restrict__ img_phase, int ncol, const CT *__restrict__ x, long ldx,
    CT *__restrict__ alpha, long lda, double dV, int g, int n0)
{
    using RT = typename Real<CT>::type;
    constexpr int NC = kProjCols, PG = 8;  // 32 columns x 8 point groups
    const int a = img_atom[g];
    const int np = ip_displ[a + 1] - ip_displ[a];
    const int ndc = img_ndc[g];
    const int *__restrict__ gp = grid_pos + img_off[g];
    const double *__restrict__ ch = chi + img_chi_off[g];
    const int c = threadIdx.x % NC, pgi = threadIdx.x / NC;
    const int n = n0 + c;
    CT acc[MAXJ];
#pragma unroll
    for (int j = 0; j < MAXJ; j++) acc[j] = CT{0, 0};
    if (n < ncol) {
        for (int ii = pgi; ii < ndc; ii += PG) {
            const CT xv = __ldg(x + (long)n * ldx + gp[ii]);
#pragma unroll
            for (int j = 0; j < MAXJ; j++)
                if (j < np) {
                    const RT cv = (RT)__ldg(ch + (long)j * ndc + ii);
                    acc[j] = CT{acc[j].x + cv * xv.x, acc[j].y + cv * xv.y};
                }
        }
    }
    __shared__ CT red[PG][NC];
    const double2 ph = img_phase[g];  // (cos theta, sin theta)
    for (int j = 0; j < np && j < MAXJ; j++) {
        __syncthreads();
        red[pgi][c] = acc[j];
        __syncthreads();
        if (pgi == 0 && n < ncol) {
            double sr = 0.0, si = 0.0;
#pragma unroll
            for (int q = 0; q < PG; q++) { sr += red[q][c].x; si += red[q][c].y; }
            const int row = ip_displ[a] + j;
            const double f = dV * gamma[row];
            const double ar = f * (ph.x * sr - ph.y * si), ai = f * (ph.x * si + ph.y * sr);
            RT *dst = reinterpret_cast<RT *>(alpha + (long)row * lda + n);
            atomicAdd(dst, (RT)ar);
            atomicAdd(dst + 1, (RT)ai);
        }
    }
}

template <typename CT, int MAXJ>
__global__ void __launch_bounds__(256)
    k_nl_project_z(const int *__restrict__ img_atom, const int *__restrict__ img_ndc,
                   const long *__restrict__ img_off, const long *__restrict__ img_chi_off,
                   const int *__restrict__ grid_pos, const double *__restrict__ chi,
                   const int *__restrict__ ip_displ, const double *__restrict__ gamma,
                   const double2 *__restrict__ img_phase, int ncol, const CT *__restrict__ x,
                   long ldx, CT *__restrict__ alpha, long lda, double dV)
{
    nl_project_z_body<CT, MAXJ>(img_atom, img_ndc, img_off, img_chi_off, grid_pos, chi,
                                ip_displ, gamma, img_phase, ncol, x, ldx, alpha, lda, dV,
                                blockIdx.x, blockIdx.y * kProjCols);
}

// apply: one thread per covered point, all columns; Hx[p] += s1 e^{-i theta_g} Chi alpha
template <typename CT, int NPMAX>
__device__ __forceinline__ void nl_apply_z_body(
    int ncov, const int *__restrict__ cov_pt, const int *__restrict__ cov_ptr,
    const long *__restrict__ ent_chi, const int4 *__restrict__ ent_meta,
    const double *__restrict__ chi, const double2 *__restrict__ img_phase, int ncol,
    const CT *__restrict__ alpha, long lda, double scale, CT *__restrict__ out, long ldo,
    int cidx)
{
    using RT = typename Real<CT>::type;
    if (cidx >= ncov) return;
    const long p = cov_pt[cidx];
    const int e0 = cov_ptr[cidx], e1 = cov_ptr[cidx + 1];
    for (int n = 0; n < ncol; n++) {
        CT acc{0, 0};
        for (int e = e0; e < e1; e++) {
            const int4 meta = ent_meta[e];
            const int ip = meta.x, np = meta.y, ndc = meta.z;
            const double *__restrict__ ch = chi + ent_chi[e];
            CT s{0, 0};
#pragma unroll
            for (int j = 0; j < NPMAX; j++) {
                if (j >= np) break;
                const RT cv = (RT)__ldg(ch + (long)j * ndc);
                const CT av = alpha[(long)(ip + j) * lda + n];
                s = CT{s.x + cv * av.x, s.y + cv * av.y};
            }
            const double2 ph = img_phase[meta.w];  // e^{-i theta} = (cos, -sin)
            acc = CT{acc.x + (RT)(ph.x * s.x + ph.y * s.y), acc.y + (RT)(ph.x * s.y - ph.y * s.x)};
        }
        CT *o = out + (long)n * ldo + p;
        *o = CT{o->x + (RT)scale * acc.x, o->y + (RT)scale * acc.y};
    }
}

// Staged apply (as k_nl_apply_staged for real blocks): block = (chunk of kApplyChunkZ covered
// points, CB columns); the alpha rows of the chunk's atoms are staged in shared memory (each
// row padded by 16 bytes, so distinct rows read by one warp start four banks apart), and
// each entry's contribution is (e^{-i theta_g} Chi_j) alpha_j, with the phase-scaled Chi value
// formed once per projector in the block's own precision (complex64 blocks read the FP32 Chi
// values and round the phase once per entry, so no FP64 arithmetic runs per projector).
constexpr int kApplyChunkZ = kApplyChunkPts;    // the chunking of the nonlocal upload
constexpr size_t kZStageMax = 96 * 1024;         // staged rows must fit this (bytes)
template <typename CT, int CB>
__host__ __device__ constexpr int zstage_ld() { return CB + (int)(16 / sizeof(CT)); }
template <typename CT, int CB, int NPMAX>
__device__ __forceinline__ void nl_apply_z_staged_body(
    int ncov, const int *__restrict__ cov_pt, const int *__restrict__ cov_ptr,
    const long *__restrict__ ent_chi, const int4 *__restrict__ ent_meta,
    const int *__restrict__ ent_slot, const int *__restrict__ chunk_row_ptr,
    const int *__restrict__ chunk_rows, const typename Real<CT>::type *__restrict__ chi,
    const double2 *__restrict__ img_phase, int ncol, const CT *__restrict__ alpha, long lda,
    double scale, CT *__restrict__ out, long ldo, int c, int n0, CT *S)
{
    using RT = typename Real<CT>::type;
    const int cidx = c * kApplyChunkZ + threadIdx.x;
    const bool live = cidx < ncov;
    const long p = live ? cov_pt[cidx] : 0;
    CT ov[CB];
#pragma unroll
    for (int q = 0; q < CB; q++)
        ov[q] = (live && n0 + q < ncol) ? out[(long)(n0 + q) * ldo + p] : CT{0, 0};
    const int r0 = chunk_row_ptr[c], nr = chunk_row_ptr[c + 1] - r0;
    constexpr int LDS = zstage_ld<CT, CB>();
    for (int e = threadIdx.x; e < nr * CB; e += blockDim.x) {
        const int r = e / CB, cc = e % CB;
        S[r * LDS + cc] = n0 + cc < ncol ? alpha[(long)chunk_rows[r0 + r] * lda + n0 + cc] : CT{0, 0};
    }
    __syncthreads();
    if (!live) return;
    const int e0 = cov_ptr[cidx], e1 = cov_ptr[cidx + 1];
    CT acc[CB];
#pragma unroll
    for (int q = 0; q < CB; q++) acc[q] = CT{0, 0};
    for (int e = e0; e < e1; e++) {
        const int4 meta = ent_meta[e];
        const int np = meta.y, ndc = meta.z;
        const RT *__restrict__ ch = chi + ent_chi[e];
        const CT *srow = S + (long)ent_slot[e] * LDS;
        const double2 ph = img_phase[meta.w];  // e^{-i theta} = (cos, -sin)
        const RT phx = (RT)ph.x, phy = (RT)ph.y;
#pragma unroll
        for (int j = 0; j < NPMAX; j++) {
            if (j >= np) break;
            const RT cv = __ldg(ch + (long)j * ndc);
            const CT t{cv * phx, -cv * phy};
#pragma unroll
            for (int q = 0; q < CB; q++) acc[q] = cadd(acc[q], cmul(t, srow[j * LDS + q]));
        }
    }
#pragma unroll
    for (int q = 0; q < CB; q++)
        if (n0 + q < ncol)
            out[(long)(n0 + q) * ldo + p] = cadd(ov[q], cscale(acc[q], (RT)scale));
}

template <typename CT>
__host__ __device__ constexpr int zapply_cb() { return sizeof(CT) == 16 ? 4 : 8; }

template <typename CT, int NPMAX>
__global__ void __launch_bounds__(kApplyChunkZ)
    k_nl_apply_z_staged(int ncov, const int *__restrict__ cov_pt, const int *__restrict__ cov_ptr,
                        const long *__restrict__ ent_chi, const int4 *__restrict__ ent_meta,
                        const int *__restrict__ ent_slot, const int *__restrict__ chunk_row_ptr,
                        const int *__restrict__ chunk_rows,
                        const typename Real<CT>::type *__restrict__ chi,
                        const double2 *__restrict__ img_phase, int ncol,
                        const CT *__restrict__ alpha, long lda, double scale,
                        CT *__restrict__ out, long ldo)
{
    extern __shared__ __align__(16) unsigned char zsmem[];
    constexpr int CB = zapply_cb<CT>();
    nl_apply_z_staged_body<CT, CB, NPMAX>(ncov, cov_pt, cov_ptr, ent_chi, ent_meta, ent_slot,
                                          chunk_row_ptr, chunk_rows, chi, img_phase, ncol,
                                          alpha, lda, scale, out, ldo, blockIdx.x,
                                          blockIdx.y * CB, reinterpret_cast<CT *>(zsmem));
}

template <typename CT, int NPMAX>
__global__ void __launch_bounds__(256)
    k_nl_apply_z(int ncov, const int *__restrict__ cov_pt, const int *__restrict__ cov_ptr,
                 const long *__restrict__ ent_chi, const int4 *__restrict__ ent_meta,
                 const double *__restrict__ chi, const double2 *__restrict__ img_phase,
                 int ncol, const CT *__restrict__ alpha, long lda, double scale,
                 CT *__restrict__ out, long ldo)
{
    nl_apply_z_body<CT, NPMAX>(ncov, cov_pt, cov_ptr, ent_chi, ent_meta, chi, img_phase, ncol,
                               alpha, lda, scale, out, ldo, blockIdx.x * blockDim.x + threadIdx.x);
}

// ------------------------------------------------------------ batched (k-point, spin) blocks
//
// All blocks of one filter call advance one degree per group of three launches (projection,
// stencil + recurrence, apply), each launch covering every block: the work tables map a
// launch's grid to (block, column) pairs, so blocks of uneven column counts share one launch.
// Per-block data (buffers, Bloch vector, image phases, projection coefficients) and the
// per-(block, degree) recurrence scalars live in device tables written before each call, so
// the degree loop is captured once as a CUDA graph and replayed while the shapes repeat.

template <typename CT>
struct BBlock {
    CT *buf[3];             // X, Y and the routing scratch block
    long ld[3];
    CT *alpha;              // ntot x ncol projection coefficients (lda = ncol)
    const double2 *phase;   // e^{i theta_g} per image for this block's k
    double kL[3];           // k_d * L_d
    double2 bf[9];          // e^{i d k_a L_a}, index 3 a + d + 1 (a = x, y, z; d = -1, 0, 1)
    int ncol, spin;
};

struct BCoef {
    double c0, s1, s2;      // centre weight (with the shift), output and recurrence scales
};

struct BConst {
    double wx[kMaxFDn + 1], wy[kMaxFDn + 1], wz[kMaxFDn + 1];
    int Nx, Ny, Nz, nslab, zlen, m;
    long Nd;
    const double *veff64;
    const float *veff32;
};

template <typename CT, int R>
__global__ void __launch_bounds__(zstencil_threads<CT>())
    k_stencil_zb(const BBlock<CT> *__restrict__ blocks, const BCoef *__restrict__ coef,
                 const int2 *__restrict__ work, const BConst cs, int deg, int in_sel,
                 int out_sel, int z_sel)
{
    const int w = blockIdx.z / cs.nslab, slab = blockIdx.z % cs.nslab;
    const int2 bc = work[w];
    const BBlock<CT> &B = blocks[bc.x];
    const BCoef cf = coef[(long)bc.x * cs.m + deg];
    StencilZParams<CT> p;
    p.x = B.buf[in_sel]; p.ldx = B.ld[in_sel];
    p.out = B.buf[out_sel]; p.ldo = B.ld[out_sel];
    p.z = z_sel >= 0 ? B.buf[z_sel] : nullptr; p.ldz = z_sel >= 0 ? B.ld[z_sel] : 0;
    const bool f64 = sizeof(CT) == 16;
    p.v = f64 ? cs.veff64 + (long)B.spin * cs.Nd : nullptr;
    p.v32 = f64 ? nullptr : cs.veff32 + (long)B.spin * cs.Nd;
    p.Nx = cs.Nx; p.Ny = cs.Ny; p.Nz = cs.Nz; p.nslab = cs.nslab; p.zlen = cs.zlen;
#pragma unroll
    for (int r = 0; r <= kMaxFDn; r++) { p.wx[r] = cs.wx[r]; p.wy[r] = cs.wy[r]; p.wz[r] = cs.wz[r]; }
    p.c0 = cf.c0; p.bv = 1.0; p.s1 = cf.s1; p.s2 = cf.s2;
    p.k.kLx = B.kL[0]; p.k.kLy = B.kL[1]; p.k.kLz = B.kL[2];
    stencil_z_body<CT, R>(p, bc.y, slab);
}

template <int R>
__global__ void __launch_bounds__(kPairMaxThreads)
    k_stencil_zb_c64(const BBlock<float2> *__restrict__ blocks, const BCoef *__restrict__ coef,
                     const int2 *__restrict__ work, const __grid_constant__ ZPairConst g,
                     const float *__restrict__ veff32, long Nd, int m, int deg, int in_sel,
                     int out_sel, int z_sel)
{
    const int w = blockIdx.z / g.nslab, slab = blockIdx.z % g.nslab;
    const int2 bc = work[w];
    const BBlock<float2> &B = blocks[bc.x];
    const BCoef cf = coef[(long)bc.x * m + deg];
    ZPairParams p;
    p.x = B.buf[in_sel]; p.ldx = B.ld[in_sel];
    p.out = B.buf[out_sel]; p.ldo = B.ld[out_sel];
    p.z = z_sel >= 0 ? B.buf[z_sel] : nullptr; p.ldz = z_sel >= 0 ? B.ld[z_sel] : 0;
    p.v32 = veff32 + (long)B.spin * Nd;
    p.c0 = (float)cf.c0; p.s1 = (float)cf.s1; p.s2 = (float)cf.s2;
#pragma unroll
    for (int i = 0; i < 9; i++) p.bf[i] = make_float2((float)B.bf[i].x, (float)B.bf[i].y);
    stencil_c64_pairs<R>(g, p, bc.y, slab);
}

// grid (image, column group); cg[y] = (block, first column)
template <typename CT, int MAXJ>
__global__ void __launch_bounds__(256)
    k_nl_project_zb(const BBlock<CT> *__restrict__ blocks, const int2 *__restrict__ cg,
                    int in_sel, const int *__restrict__ img_atom, const int *__restrict__ img_ndc,
                    const long *__restrict__ img_off, const long *__restrict__ img_chi_off,
                    const int *__restrict__ grid_pos, const double *__restrict__ chi,
                    const int *__restrict__ ip_displ, const double *__restrict__ gamma,
                    double dV)
{
    const int2 bc = cg[blockIdx.y];
    const BBlock<CT> &B = blocks[bc.x];
    nl_project_z_body<CT, MAXJ>(img_atom, img_ndc, img_off, img_chi_off, grid_pos, chi,
                                ip_displ, gamma, B.phase, B.ncol, B.buf[in_sel], B.ld[in_sel],
                                B.alpha, B.ncol, dV, blockIdx.x, bc.y);
}

// complex64 projection: block = (image g, group of kProjCols columns of one block), eight warps
// of four columns each. Lane = 8 c + p: column c of the warp, point phase p, so one load
// instruction reads eight consecutive points of four columns (coalesced) and one Chi row
// segment of eight points serves all four columns. The image's grid positions and Chi rows
// pass through shared memory in chunks of kProjChunk points (coalesced loads by the whole
// block; Chi stored point-major so a lane reads a point's values in 16-byte pieces), so the
// orbital loads wait on no other global load and several are in flight per lane. Each lane accumulates every projector; three shuffle steps sum the eight point phases
// (every lane ends with the totals) and lane p adds projectors p, p+8, p+16:
// alpha[row, n] += e^{i theta_g} dV Gamma_row sum (atomic across the images of one atom).
constexpr int kProjChunk = 256;  // points per staged chunk of the complex64 projection
template <int MAXJ>
__global__ void __launch_bounds__(256, 3)
    k_nl_project_zb_c64(const BBlock<float2> *__restrict__ blocks, const int2 *__restrict__ cg,
                        int in_sel, const int *__restrict__ img_atom,
                        const int *__restrict__ img_ndc, const long *__restrict__ img_off,
                        const long *__restrict__ img_chi_off, const int *__restrict__ grid_pos,
                        const float *__restrict__ chi, const int *__restrict__ ip_displ,
                        const double *__restrict__ gamma, double dV)
{
    const int g = blockIdx.x;
    const int2 bc = cg[blockIdx.y];
    const BBlock<float2> &B = blocks[bc.x];
    const int a = img_atom[g];
    const int np = ip_displ[a + 1] - ip_displ[a];
    const int ndc = img_ndc[g];
    const int *__restrict__ gp = grid_pos + img_off[g];
    const float *__restrict__ ch = chi + img_chi_off[g];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int p = lane & 7, c = lane >> 3;
    const int n = bc.y + wid * 4 + c;
    const bool on = n < B.ncol;
    const float2 *__restrict__ xc = B.buf[in_sel] + (long)(on ? n : bc.y) * B.ld[in_sel];
    // Chi of a chunk point-major, rows padded to a multiple of four floats: a lane reads one
    // point's values in 16-byte pieces, and the eight points a warp reads at once (rows
    // MAXJP floats apart, MAXJP = 4 mod 8) fall on distinct banks
    constexpr int MAXJP = (MAXJ + 3) / 4 * 4;
    static_assert(MAXJP % 8 == 4, "row pitch of the staged Chi values");
    __shared__ int sgp[kProjChunk];
    __shared__ __align__(16) float sch[kProjChunk * MAXJP];
    float2 acc[MAXJ];
#pragma unroll
    for (int jj = 0; jj < MAXJ; jj++) acc[jj] = make_float2(0.f, 0.f);
    for (int c0 = 0; c0 < ndc; c0 += kProjChunk) {
        const int cn = min(kProjChunk, ndc - c0);
        __syncthreads();  // the previous chunk is consumed
        for (int i = threadIdx.x; i < cn; i += 256) sgp[i] = __ldg(gp + c0 + i);
        for (int jj = 0; jj < MAXJP; jj++)
            for (int i = threadIdx.x; i < cn; i += 256)
                sch[i * MAXJP + jj] = jj < np ? __ldg(ch + (long)jj * ndc + c0 + i) : 0.f;
        __syncthreads();
#pragma unroll 2
        for (int ii = p; ii < cn; ii += 8) {
            const float2 xv = on ? __ldg(xc + sgp[ii]) : make_float2(0.f, 0.f);
            const float4 *cr = reinterpret_cast<const float4 *>(sch + ii * MAXJP);
#pragma unroll
            for (int u = 0; u < MAXJP / 4; u++) {
                const float4 c4 = cr[u];
                const float cv[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
                for (int w = 0; w < 4; w++) {
                    const int jj = 4 * u + w;
                    if (jj < MAXJ && jj < np) {
                        acc[jj].x = fmaf(cv[w], xv.x, acc[jj].x);
                        acc[jj].y = fmaf(cv[w], xv.y, acc[jj].y);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int jj = 0; jj < MAXJ; jj++) {
        if (jj < np) {
#pragma unroll
            for (int o = 4; o > 0; o >>= 1) {
                acc[jj].x += __shfl_xor_sync(0xffffffffu, acc[jj].x, o);
                acc[jj].y += __shfl_xor_sync(0xffffffffu, acc[jj].y, o);
            }
        }
    }
    if (!on) return;
    const double2 ph = B.phase[g];
#pragma unroll
    for (int jj = 0; jj < MAXJ; jj++) {
        if (jj < np && (jj & 7) == p) {
            const int row = ip_displ[a] + jj;
            const double f = dV * gamma[row];
            const double sr = acc[jj].x, si = acc[jj].y;
            float *dst = reinterpret_cast<float *>(B.alpha + (long)row * B.ncol + n);
            atomicAdd(dst, (float)(f * (ph.x * sr - ph.y * si)));
            atomicAdd(dst + 1, (float)(f * (ph.x * si + ph.y * sr)));
        }
    }
}

// the Chi table in a block's real precision
template <typename CT>
const typename Real<CT>::type *chi_z(const Nonlocal &nl)
{
    if constexpr (sizeof(CT) == 8)
        return nl.chi32;
    else
        return nl.chi64;
}

// staged, grouped: grid (chunk, column block, block); blocks with fewer columns return early
template <typename CT, int NPMAX>
__global__ void __launch_bounds__(kApplyChunkZ)
    k_nl_apply_zb_staged(const BBlock<CT> *__restrict__ blocks, const BCoef *__restrict__ coef,
                         int m, int deg, int out_sel, int ncov, const int *__restrict__ cov_pt,
                         const int *__restrict__ cov_ptr, const long *__restrict__ ent_chi,
                         const int4 *__restrict__ ent_meta, const int *__restrict__ ent_slot,
                         const int *__restrict__ chunk_row_ptr,
                         const int *__restrict__ chunk_rows,
                         const typename Real<CT>::type *__restrict__ chi)
{
    extern __shared__ __align__(16) unsigned char zsmem[];
    constexpr int CB = zapply_cb<CT>();
    const BBlock<CT> &B = blocks[blockIdx.z];
    const int n0 = blockIdx.y * CB;
    if (n0 >= B.ncol) return;  // uniform per thread block
    const double scale = coef[(long)blockIdx.z * m + deg].s1;
    nl_apply_z_staged_body<CT, CB, NPMAX>(ncov, cov_pt, cov_ptr, ent_chi, ent_meta, ent_slot,
                                          chunk_row_ptr, chunk_rows, chi, B.phase, B.ncol,
                                          B.alpha, B.ncol, scale, B.buf[out_sel],
                                          B.ld[out_sel], blockIdx.x, n0,
                                          reinterpret_cast<CT *>(zsmem));
}

// grid (covered-point chunk, block)
template <typename CT, int NPMAX>
__global__ void __launch_bounds__(256)
    k_nl_apply_zb(const BBlock<CT> *__restrict__ blocks, const BCoef *__restrict__ coef,
                  int m, int deg, int out_sel, int ncov, const int *__restrict__ cov_pt,
                  const int *__restrict__ cov_ptr, const long *__restrict__ ent_chi,
                  const int4 *__restrict__ ent_meta, const double *__restrict__ chi)
{
    const BBlock<CT> &B = blocks[blockIdx.y];
    const double scale = coef[(long)blockIdx.y * m + deg].s1;
    nl_apply_z_body<CT, NPMAX>(ncov, cov_pt, cov_ptr, ent_chi, ent_meta, chi, B.phase, B.ncol,
                               B.alpha, B.ncol, scale, B.buf[out_sel], B.ld[out_sel],
                               blockIdx.x * blockDim.x + threadIdx.x);
}

}  // namespace

// ------------------------------------------------------------------ host side

// device tables and the cached CUDA graph of the batched filter
struct BatchState {
    void *tables = nullptr;
    size_t tables_bytes = 0;
    cudaGraphExec_t exec = nullptr;
    std::vector<long> key;
    ~BatchState()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (tables) cudaFree(tables);
    }
};

struct KpointState {
    BatchState batch;
    long batch_launches = 0;         // kernels in the cached batched-filter graph
    double L[3] = {0, 0, 0};
    std::vector<double> img_coords;  // 3 * nimg
    double2 *img_phase = nullptr;    // device, nimg
    int nimg = 0;
};

static int kstate(sgpu_ctx *ctx, KpointState **out)
{
    if (!ctx->kp) {
        set_error("k-point call: sgpu_set_kpoint_geometry has not been called");
        return SGPU_ERR_STATE;
    }
    *out = ctx->kp;
    return SGPU_OK;
}

void kpoint_free(sgpu_ctx *ctx)
{
    if (ctx->kp) {
        if (ctx->kp->img_phase) cudaFree(ctx->kp->img_phase);
        delete ctx->kp;
        ctx->kp = nullptr;
    }
}

// per-image Bloch phases theta_g = -k . (floor(c_g / L) L) for k-point k
static int set_phases(sgpu_ctx *ctx, const double *k, cudaStream_t st)
{
    KpointState *ks;
    SGPU_TRY(kstate(ctx, &ks));
    if (ks->nimg == 0) return SGPU_OK;
    std::vector<double2> ph(ks->nimg);
    for (int g = 0; g < ks->nimg; g++) {
        const double *cg = &ks->img_coords[3 * g];
        double th = 0.0;
        for (int d = 0; d < 3; d++) th -= k[d] * (std::floor(cg[d] / ks->L[d]) * ks->L[d]);
        ph[g] = make_double2(std::cos(th), std::sin(th));
    }
    SGPU_CUDA_TRY(cudaMemcpyAsync(ks->img_phase, ph.data(), sizeof(double2) * ks->nimg,
                                  cudaMemcpyHostToDevice, st));
    return SGPU_OK;
}

template <typename CT>
static int stencil_z(sgpu_ctx *ctx, const double *k, int ncol, double a, double bv, double c,
                     const double *v, const float *v32, const CT *x, long ldx, CT *out,
                     long ldo, double s1, double s2, const CT *z, long ldz, cudaStream_t st)
{
    constexpr int R = 6;
    if (ctx->FDn != R) {
        set_error("stencil: only FD order 12 (radius 6) is built");
        return SGPU_ERR_ARG;
    }
    if (ncol <= 0) return SGPU_OK;
    KpointState *ks;
    SGPU_TRY(kstate(ctx, &ks));
    StencilZParams<CT> p;
    p.x = x; p.out = out; p.z = (z && s2 != 0.0) ? z : nullptr;
    p.v = (bv != 0.0) ? v : nullptr;
    p.v32 = (bv != 0.0) ? v32 : nullptr;
    p.ldx = ldx; p.ldo = ldo; p.ldz = ldz;
    p.Nx = ctx->Nx; p.Ny = ctx->Ny; p.Nz = ctx->Nz;
    for (int r = 0; r <= R; r++) {
        p.wx[r] = ctx->cx[r] * a;
        p.wy[r] = ctx->cy[r] * a;
        p.wz[r] = ctx->cz[r] * a;
    }
    double c0 = ctx->cx[0] * a;
    c0 += ctx->cy[0] * a;
    c0 += ctx->cz[0] * a;
    c0 += c;
    p.c0 = c0; p.bv = bv; p.s1 = s1; p.s2 = s2;
    p.k.kLx = k[0] * ks->L[0];
    p.k.kLy = k[1] * ks->L[1];
    p.k.kLz = k[2] * ks->L[2];
    if constexpr (sizeof(CT) == 8) {  // complex64: the pair kernel where it applies
        int PX2, PY;
        zpair_tile(ctx->Nx, ctx->Ny, R, &PX2, &PY);
        bool ok = ctx->zpair_on && zpair_ok(ctx->Nx, ctx->Ny, ctx->Nz, R, PX2, PY) &&
                  ldx % 2 == 0 && ldo % 2 == 0 && (!p.z || ldz % 2 == 0) &&
                  (uintptr_t)x % 16 == 0 && (uintptr_t)out % 16 == 0 &&
                  (!p.z || (uintptr_t)z % 16 == 0) && (!p.v32 || ctx->Nd % 2 == 0);
        if (ok) {
            ZPairParams zp;
            ZPairConst zg;
            zp.x = x; zp.out = out; zp.z = p.z; zp.v32 = p.v32;
            zp.ldx = ldx; zp.ldo = ldo; zp.ldz = ldz;
            zg.Nx = ctx->Nx; zg.Ny = ctx->Ny; zg.Nz = ctx->Nz;
            for (int r = 0; r <= R; r++) {
                zg.wx[r] = (float)p.wx[r]; zg.wy[r] = (float)p.wy[r]; zg.wz[r] = (float)p.wz[r];
            }
            // the potential scale bv multiplies the FP32 potential as in the generic kernel
            zp.c0 = (float)p.c0; zp.s1 = (float)p.s1; zp.s2 = (float)p.s2;
            const double kL[3] = {p.k.kLx, p.k.kLy, p.k.kLz};
            for (int a = 0; a < 3; a++)
                for (int d = -1; d <= 1; d++)
                    zp.bf[3 * a + d + 1] = make_float2((float)std::cos(d * kL[a]),
                                                       (float)std::sin(d * kL[a]));
            if (p.v32 && bv != 1.0) ok = false;  // the pair kernel takes bv = 1
            if (ok) {
                const size_t psm = zpair_smem(PX2, PY, R);
                SGPU_CUDA_TRY(cudaFuncSetAttribute(k_stencil_z_c64<R>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)psm));
                const int ptx = (ctx->Nx + 2 * PX2 - 1) / (2 * PX2), pty = (ctx->Ny + PY - 1) / PY;
                int nslab = 1;
                while ((long)ptx * pty * ncol * nslab < 152L * 8 && ctx->Nz / (nslab * 2) >= 8)
                    nslab *= 2;
                zg.zlen = (ctx->Nz + nslab - 1) / nslab;
                zg.nslab = nslab;
                const int maxz = 65535 / nslab;
                for (int c0i = 0; c0i < ncol; c0i += maxz) {
                    const int nc = std::min(maxz, ncol - c0i);
                    ZPairParams q = zp;
                    q.x = x + (long)c0i * ldx;
                    q.out = out + (long)c0i * ldo;
                    if (q.z) q.z = zp.z + (long)c0i * ldz;
                    ProfScope ps(ctx, SGPU_KERNEL_STENCIL, st);
                    k_stencil_z_c64<R><<<dim3(ptx, pty, nc * nslab), dim3(PX2, PY), psm, st>>>(zg, q);
                }
                SGPU_CUDA_TRY(cudaGetLastError());
                return SGPU_OK;
            }
        }
    }
    int BX, BY;
    zstencil_tile(ctx->Nx, ctx->Ny, R, zstencil_threads<CT>(), &BX, &BY);
    const size_t zsm = zstencil_smem<CT>(BX, BY, R);
    SGPU_CUDA_TRY(cudaFuncSetAttribute(k_stencil_z<CT, R>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zsm));
    const int tilesx = (ctx->Nx + BX - 1) / BX, tilesy = (ctx->Ny + BY - 1) / BY;
    long blocks1 = (long)tilesx * tilesy * ncol;
    int nslab = 1;
    while (blocks1 * nslab < 152L * 8 && ctx->Nz / (nslab * 2) >= 8) nslab *= 2;
    p.zlen = (ctx->Nz + nslab - 1) / nslab;
    p.nslab = nslab;
    const int maxz = 65535 / nslab;
    for (int c0i = 0; c0i < ncol; c0i += maxz) {
        const int nc = std::min(maxz, ncol - c0i);
        StencilZParams<CT> q = p;
        q.x = x + (long)c0i * ldx;
        q.out = out + (long)c0i * ldo;
        if (q.z) q.z = z + (long)c0i * ldz;
        ProfScope ps(ctx, SGPU_KERNEL_STENCIL, st);
        k_stencil_z<CT, R><<<dim3(tilesx, tilesy, nc * nslab), dim3(BX, BY), zsm, st>>>(q);
    }
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

template <typename CT>
static int nonlocal_z(sgpu_ctx *ctx, int ncol, const CT *x, long ldx, CT *out, long ldo,
                      double scale, cudaStream_t st)
{
    const Nonlocal &nl = ctx->nl;
    if (!ctx->has_nl || nl.ntot == 0 || ncol <= 0) return SGPU_OK;
    KpointState *ks;
    SGPU_TRY(kstate(ctx, &ks));
    if (ks->nimg != nl.nimg) {
        set_error("k-point call: image coordinates do not match the nonlocal set");
        return SGPU_ERR_STATE;
    }
    const long lda = ncol;
    CT *alpha = nullptr;
    SGPU_TRY(ws_get(ctx, WS_ALPHA, sizeof(CT) * (size_t)nl.ntot * lda, (void **)&alpha));
    SGPU_CUDA_TRY(cudaMemsetAsync(alpha, 0, sizeof(CT) * (size_t)nl.ntot * lda, st));
    const dim3 pg(nl.nimg, (ncol + 31) / 32);
    {
        ProfScope ps(ctx, SGPU_KERNEL_NL_PROJECT, st);
        if (nl.max_np <= 9)
            k_nl_project_z<CT, 9><<<pg, 256, 0, st>>>(nl.img_atom, nl.img_ndc, nl.img_off,
                nl.img_chi_off, nl.grid_pos, nl.chi64, nl.ip_displ, nl.gamma64, ks->img_phase,
                ncol, x, ldx, alpha, lda, ctx->dV);
        else if (nl.max_np <= 18)
            k_nl_project_z<CT, 18><<<pg, 256, 0, st>>>(nl.img_atom, nl.img_ndc, nl.img_off,
                nl.img_chi_off, nl.grid_pos, nl.chi64, nl.ip_displ, nl.gamma64, ks->img_phase,
                ncol, x, ldx, alpha, lda, ctx->dV);
        else {
            set_error("k-point nonlocal: more than 18 projectors per atom is not built");
            return SGPU_ERR_ARG;
        }
    }
    {
        ProfScope ps(ctx, SGPU_KERNEL_NL_APPLY, st);
        constexpr int CB = zapply_cb<CT>();
        const size_t stage = sizeof(CT) * (size_t)nl.max_chunk_rows * zstage_ld<CT, CB>();
        if (nl.nchunk > 0 && stage <= kZStageMax) {
            const dim3 sg(nl.nchunk, (ncol + CB - 1) / CB);
            auto launch = [&](auto kern) -> int {
                SGPU_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)std::max<size_t>(stage, 16)));
                kern<<<sg, kApplyChunkZ, std::max<size_t>(stage, 16), st>>>(
                    nl.ncov, nl.cov_pt, nl.cov_ptr, nl.ent_chi, nl.ent_meta, nl.ent_slot,
                    nl.chunk_row_ptr, nl.chunk_rows, chi_z<CT>(nl), ks->img_phase, ncol, alpha,
                    lda, scale, out, ldo);
                return SGPU_OK;
            };
            if (nl.max_np <= 9)
                SGPU_TRY(launch(k_nl_apply_z_staged<CT, 9>));
            else
                SGPU_TRY(launch(k_nl_apply_z_staged<CT, 18>));
        } else {
            const int blocks = (nl.ncov + 255) / 256;
            if (nl.max_np <= 9)
                k_nl_apply_z<CT, 9><<<blocks, 256, 0, st>>>(nl.ncov, nl.cov_pt, nl.cov_ptr,
                    nl.ent_chi, nl.ent_meta, nl.chi64, ks->img_phase, ncol, alpha, lda, scale, out, ldo);
            else
                k_nl_apply_z<CT, 18><<<blocks, 256, 0, st>>>(nl.ncov, nl.cov_pt, nl.cov_ptr,
                    nl.ent_chi, nl.ent_meta, nl.chi64, ks->img_phase, ncol, alpha, lda, scale, out, ldo);
        }
    }
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

// Hx = s1 * ((-0.5 Lap + Veff + c) x + Vnl x) + s2 * z at k-point k (per-image phases
// already set): the stencil writes every output point, then the nonlocal apply adds its term
// at the covered points.
template <typename CT>
int hamiltonian_z(sgpu_ctx *ctx, int spin, const double *k, int ncol, double c, const CT *x,
                  long ldx, CT *hx, long ldh, double s1, double s2, const CT *z, long ldz,
                  cudaStream_t st)
{
    if (spin < 0 || spin >= ctx->nspin_veff) {
        set_error("Hamiltonian (k-point): no local potential set for this spin block");
        return SGPU_ERR_STATE;
    }
    const bool f64 = sizeof(CT) == 16;
    const double *v = f64 ? ctx->veff64 + (long)spin * ctx->Nd : nullptr;
    const float *v32 = f64 ? nullptr : ctx->veff32 + (long)spin * ctx->Nd;
    SGPU_TRY(stencil_z<CT>(ctx, k, ncol, -0.5, 1.0, c, v, v32, x, ldx, hx, ldh, s1, s2, z, ldz, st));
    SGPU_TRY(nonlocal_z<CT>(ctx, ncol, x, ldx, hx, ldh, s1, st));
    return SGPU_OK;
}

template <typename CT>
int chebyshev_z(sgpu_ctx *ctx, int spin, const double *k, CT *X, long ldx, CT *Y, long ldy,
                int ncol, int m, double a, double b, double a0, cudaStream_t st)
{
    const double e = 0.5 * (b - a);
    const double c = 0.5 * (b + a);
    double sigma = e / (a0 - c);
    const double sigma1 = sigma;
    const double gamma = 2.0 / sigma1;
    const long Nd = ctx->Nd;
    CT *W = nullptr;
    const bool route = ((m - 1) % 2) == 1;  // same buffer routing as the real filter
    if (route) SGPU_TRY(ws_get(ctx, WS_STAGE_C, sizeof(CT) * (size_t)Nd * ncol, (void **)&W));
    CT *y0 = route ? W : Y;
    long ly0 = route ? Nd : ldy;
    SGPU_TRY(hamiltonian_z<CT>(ctx, spin, k, ncol, -c, X, ldx, y0, ly0, sigma1 / e, 0.0, nullptr, 0, st));
    CT *cur = y0, *prev = X;
    long ldc = ly0, ldp = ldx;
    for (int j = 1; j < m; j++) {
        const double sigma2 = 1.0 / (gamma - sigma);
        CT *dst = prev;
        long ldd = ldp;
        if (route && j == 1) { dst = Y; ldd = ldy; }
        if (route && j == 2) { dst = X; ldd = ldx; }
        SGPU_TRY(hamiltonian_z<CT>(ctx, spin, k, ncol, -c, cur, ldc, dst, ldd, 2.0 * sigma2 / e,
                                   -sigma * sigma2, prev, ldp, st));
        prev = cur; ldp = ldc;
        cur = dst; ldc = ldd;
        sigma = sigma2;
    }
    if (route && m == 2)
        SGPU_CUDA_TRY(cudaMemcpy2DAsync(X, sizeof(CT) * ldx, W, sizeof(CT) * Nd, sizeof(CT) * Nd,
                                        ncol, cudaMemcpyDeviceToDevice, st));
    return SGPU_OK;
}

// Batched filter: every block's degree j in one projection, one stencil and one apply launch;
// the launches of all m degrees are captured once in a CUDA graph (replayed while the call's
// shapes, buffers and workspaces repeat), and the per-call numbers go in through the tables.
template <typename CT>
static int chebyshev_batched(sgpu_ctx *ctx, int nblk, const sgpu_filter_block *blk, int m,
                             cudaStream_t st)
{
    constexpr int R = 6;
    KpointState *ks;
    SGPU_TRY(kstate(ctx, &ks));
    const Nonlocal &nl = ctx->nl;
    const bool has_nl = ctx->has_nl && nl.ntot > 0;
    if (has_nl && ks->nimg != nl.nimg) {
        set_error("batched filter: image coordinates do not match the nonlocal set");
        return SGPU_ERR_STATE;
    }
    if (has_nl && nl.max_np > 18) {
        set_error("batched filter: more than 18 projectors per atom is not built");
        return SGPU_ERR_ARG;
    }
    const long Nd = ctx->Nd;
    const bool route = ((m - 1) % 2) == 1;
    std::vector<long> coloff(nblk + 1, 0);
    for (int b = 0; b < nblk; b++) coloff[b + 1] = coloff[b] + blk[b].ncol;
    const long totcols = coloff[nblk];
    if (totcols == 0) return SGPU_OK;
    CT *W = nullptr, *alpha = nullptr;
    if (route) SGPU_TRY(ws_get(ctx, WS_STAGE_C, sizeof(CT) * (size_t)Nd * totcols, (void **)&W));
    if (has_nl)
        SGPU_TRY(ws_get(ctx, WS_ALPHA, sizeof(CT) * (size_t)nl.ntot * totcols, (void **)&alpha));

    // host copies of the tables: blocks | coef | work | column groups | phases
    std::vector<BBlock<CT>> hb(nblk);
    std::vector<BCoef> hc((size_t)nblk * m);
    std::vector<int2> hw, hg;
    const int nimg = has_nl ? nl.nimg : 0;
    std::vector<double2> hp((size_t)nblk * std::max(nimg, 1));
    int maxspin = 0;
    for (int b = 0; b < nblk; b++) {
        const sgpu_filter_block &f = blk[b];
        maxspin = std::max(maxspin, f.spin);
        BBlock<CT> &B = hb[b];
        B.buf[0] = reinterpret_cast<CT *>(f.X); B.ld[0] = f.ldi;
        B.buf[1] = reinterpret_cast<CT *>(f.Y); B.ld[1] = f.ldo;
        B.buf[2] = route ? W + (size_t)Nd * coloff[b] : nullptr; B.ld[2] = Nd;
        B.alpha = has_nl ? alpha + (size_t)nl.ntot * coloff[b] : nullptr;
        B.phase = nullptr;  // set after the table is placed
        for (int d = 0; d < 3; d++) B.kL[d] = f.k[d] * ks->L[d];
        for (int a = 0; a < 3; a++)
            for (int d = -1; d <= 1; d++)
                B.bf[3 * a + d + 1] = make_double2(std::cos(d * B.kL[a]), std::sin(d * B.kL[a]));
        B.ncol = f.ncol;
        B.spin = f.spin;
        // recurrence scalars of ChebyshevFiltering_kpt (src/eigenSolverKpt.c:458-550)
        const double e = 0.5 * (f.b - f.a), c = 0.5 * (f.b + f.a);
        double sigma = e / (f.a0 - c);
        const double sigma1 = sigma, gamma = 2.0 / sigma1;
        double c0 = ctx->cx[0] * -0.5;
        c0 += ctx->cy[0] * -0.5;
        c0 += ctx->cz[0] * -0.5;
        c0 += -c;
        for (int j = 0; j < m; j++) {
            BCoef &q = hc[(size_t)b * m + j];
            q.c0 = c0;
            if (j == 0) {
                q.s1 = sigma1 / e;
                q.s2 = 0.0;
            } else {
                const double sigma2 = 1.0 / (gamma - sigma);
                q.s1 = 2.0 * sigma2 / e;
                q.s2 = -sigma * sigma2;
                sigma = sigma2;
            }
        }
        for (int n = 0; n < f.ncol; n++) hw.push_back(make_int2(b, n));
        for (int n0 = 0; n0 < f.ncol; n0 += kProjCols) hg.push_back(make_int2(b, n0));
        for (int g = 0; g < nimg; g++) {
            const double *cgc = &ks->img_coords[3 * g];
            double th = 0.0;
            for (int d = 0; d < 3; d++) th -= f.k[d] * (std::floor(cgc[d] / ks->L[d]) * ks->L[d]);
            hp[(size_t)b * nimg + g] = make_double2(std::cos(th), std::sin(th));
        }
    }
    if (maxspin >= ctx->nspin_veff) {
        set_error("batched filter: a block's spin has no local potential");
        return SGPU_ERR_STATE;
    }
    auto align = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t ob = 0, oc = align(ob + sizeof(BBlock<CT>) * nblk),
                 ow = align(oc + sizeof(BCoef) * hc.size()),
                 og = align(ow + sizeof(int2) * hw.size()),
                 op = align(og + sizeof(int2) * hg.size()), oend = align(op + sizeof(double2) * hp.size());
    BatchState &bs = ks->batch;
    if (bs.tables_bytes < oend) {
        if (bs.exec) { cudaGraphExecDestroy(bs.exec); bs.exec = nullptr; }
        SGPU_CUDA_TRY(cudaStreamSynchronize(st));
        if (bs.tables) cudaFree(bs.tables);
        bs.tables = nullptr;
        bs.tables_bytes = 0;
        SGPU_CUDA_TRY(cudaMalloc(&bs.tables, oend));
        bs.tables_bytes = oend;
    }
    char *tb = static_cast<char *>(bs.tables);
    for (int b = 0; b < nblk; b++)
        hb[b].phase = reinterpret_cast<const double2 *>(tb + op) + (size_t)b * nimg;
    std::vector<char> pack(oend, 0);
    std::memcpy(pack.data() + ob, hb.data(), sizeof(BBlock<CT>) * nblk);
    std::memcpy(pack.data() + oc, hc.data(), sizeof(BCoef) * hc.size());
    std::memcpy(pack.data() + ow, hw.data(), sizeof(int2) * hw.size());
    std::memcpy(pack.data() + og, hg.data(), sizeof(int2) * hg.size());
    std::memcpy(pack.data() + op, hp.data(), sizeof(double2) * hp.size());
    SGPU_CUDA_TRY(cudaMemcpyAsync(tb, pack.data(), oend, cudaMemcpyHostToDevice, st));
    // the host staging buffer must outlive the copy
    SGPU_CUDA_TRY(cudaStreamSynchronize(st));
    const BBlock<CT> *dB = reinterpret_cast<const BBlock<CT> *>(tb + ob);
    const BCoef *dC = reinterpret_cast<const BCoef *>(tb + oc);
    const int2 *dW = reinterpret_cast<const int2 *>(tb + ow);
    const int2 *dG = reinterpret_cast<const int2 *>(tb + og);

    BConst cs;
    for (int r = 0; r <= R; r++) {
        cs.wx[r] = ctx->cx[r] * -0.5;
        cs.wy[r] = ctx->cy[r] * -0.5;
        cs.wz[r] = ctx->cz[r] * -0.5;
    }
    cs.Nx = ctx->Nx; cs.Ny = ctx->Ny; cs.Nz = ctx->Nz; cs.m = m; cs.Nd = Nd;
    cs.veff64 = ctx->veff64;
    cs.veff32 = ctx->veff32;
    int BX, BY;
    zstencil_tile(ctx->Nx, ctx->Ny, R, zstencil_threads<CT>(), &BX, &BY);
    size_t zsm = zstencil_smem<CT>(BX, BY, R);  // attribute set before any capture
    SGPU_CUDA_TRY(cudaFuncSetAttribute(k_stencil_zb<CT, R>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)zsm));
    // complex64: the pair kernel when its alignment and one-period conditions hold
    bool pairs = false;
    int PX2 = 0, PY = 0;
    if constexpr (sizeof(CT) == 8) {
        zpair_tile(ctx->Nx, ctx->Ny, R, &PX2, &PY);
        pairs = ctx->zpair_on && zpair_ok(ctx->Nx, ctx->Ny, ctx->Nz, R, PX2, PY) &&
                (uintptr_t)W % 16 == 0 && Nd % 2 == 0;
        for (int b = 0; b < nblk && pairs; b++)
            pairs = blk[b].ldi % 2 == 0 && blk[b].ldo % 2 == 0 &&
                    (uintptr_t)blk[b].X % 16 == 0 && (uintptr_t)blk[b].Y % 16 == 0;
        if (pairs) {
            BX = 2 * PX2;
            BY = PY;
            zsm = zpair_smem(PX2, PY, R);
            SGPU_CUDA_TRY(cudaFuncSetAttribute(k_stencil_zb_c64<R>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)zsm));
        }
    }
    const int tilesx = (ctx->Nx + BX - 1) / BX, tilesy = (ctx->Ny + BY - 1) / BY;
    int nslab = 1;
    while ((long)tilesx * tilesy * totcols * nslab < 152L * 8 && ctx->Nz / (nslab * 2) >= 8)
        nslab *= 2;
    cs.nslab = nslab;
    cs.zlen = (ctx->Nz + nslab - 1) / nslab;
    ZPairConst pg;  // launch-wide data of the complex64 pair kernel
    for (int r = 0; r <= R; r++) {
        pg.wx[r] = (float)cs.wx[r]; pg.wy[r] = (float)cs.wy[r]; pg.wz[r] = (float)cs.wz[r];
    }
    pg.Nx = cs.Nx; pg.Ny = cs.Ny; pg.Nz = cs.Nz; pg.nslab = cs.nslab; pg.zlen = cs.zlen;
    const long maxw = 65535 / nslab;
    const size_t abytes = has_nl ? sizeof(CT) * (size_t)nl.ntot * totcols : 0;
    int maxcol = 0;
    for (int b = 0; b < nblk; b++) maxcol = std::max(maxcol, blk[b].ncol);
    if (has_nl) {  // shared-memory size of the staged apply, set before any capture
        const size_t stage =
            sizeof(CT) * (size_t)nl.max_chunk_rows * zstage_ld<CT, zapply_cb<CT>()>();
        if (nl.nchunk > 0 && stage <= kZStageMax) {
            const int sm = (int)std::max<size_t>(stage, 16);
            SGPU_CUDA_TRY(cudaFuncSetAttribute(k_nl_apply_zb_staged<CT, 9>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
            SGPU_CUDA_TRY(cudaFuncSetAttribute(k_nl_apply_zb_staged<CT, 18>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
        }
    }

    auto issue = [&]() -> int {
        int cur = route ? 2 : 1, prev = 0;  // buffer ids: 0 X, 1 Y, 2 scratch
        for (int j = 0; j < m; j++) {
            int in, out, zsel;
            if (j == 0) {
                in = 0; out = cur; zsel = -1;
            } else {
                int dst = prev;
                if (route && j == 1) dst = 1;
                if (route && j == 2) dst = 0;
                in = cur; out = dst; zsel = prev;
                prev = cur;
                cur = dst;
            }
            if (has_nl) {
                SGPU_CUDA_TRY(cudaMemsetAsync(alpha, 0, abytes, st));
                ProfScope ps(ctx, SGPU_KERNEL_NL_PROJECT, st);
                const dim3 pg(nl.nimg, (unsigned)hg.size());
                if constexpr (sizeof(CT) == 8) {  // complex64: warp-per-column form
                    const auto *dB32 = reinterpret_cast<const BBlock<float2> *>(dB);
                    if (nl.max_np <= 9)
                        k_nl_project_zb_c64<9><<<pg, 256, 0, st>>>(dB32, dG, in, nl.img_atom,
                            nl.img_ndc, nl.img_off, nl.img_chi_off, nl.grid_pos, nl.chi32,
                            nl.ip_displ, nl.gamma64, ctx->dV);
                    else
                        k_nl_project_zb_c64<18><<<pg, 256, 0, st>>>(dB32, dG, in, nl.img_atom,
                            nl.img_ndc, nl.img_off, nl.img_chi_off, nl.grid_pos, nl.chi32,
                            nl.ip_displ, nl.gamma64, ctx->dV);
                } else if (nl.max_np <= 9)
                    k_nl_project_zb<CT, 9><<<pg, 256, 0, st>>>(dB, dG, in, nl.img_atom,
                        nl.img_ndc, nl.img_off, nl.img_chi_off, nl.grid_pos, nl.chi64,
                        nl.ip_displ, nl.gamma64, ctx->dV);
                else
                    k_nl_project_zb<CT, 18><<<pg, 256, 0, st>>>(dB, dG, in, nl.img_atom,
                        nl.img_ndc, nl.img_off, nl.img_chi_off, nl.grid_pos, nl.chi64,
                        nl.ip_displ, nl.gamma64, ctx->dV);
                ctx->launches++;
            }
            for (long w0 = 0; w0 < totcols; w0 += maxw) {
                const long nw = std::min(maxw, totcols - w0);
                ProfScope ps(ctx, SGPU_KERNEL_STENCIL, st);
                if constexpr (sizeof(CT) == 8) {
                    if (pairs) {
                        k_stencil_zb_c64<R><<<dim3(tilesx, tilesy, (unsigned)(nw * nslab)),
                                              dim3(PX2, PY), zsm, st>>>(
                            reinterpret_cast<const BBlock<float2> *>(dB), dC, dW + w0, pg,
                            ctx->veff32, Nd, m, j, in, out, zsel);
                        ctx->launches++;
                        continue;
                    }
                }
                k_stencil_zb<CT, R><<<dim3(tilesx, tilesy, (unsigned)(nw * nslab)),
                                      dim3(BX, BY), zsm, st>>>(dB, dC, dW + w0, cs, j, in, out,
                                                               zsel);
                ctx->launches++;
            }
            if (has_nl) {
                ProfScope ps(ctx, SGPU_KERNEL_NL_APPLY, st);
                constexpr int CB = zapply_cb<CT>();
                const size_t stage = sizeof(CT) * (size_t)nl.max_chunk_rows * zstage_ld<CT, CB>();
                if (nl.nchunk > 0 && stage <= kZStageMax) {
                    const dim3 sg(nl.nchunk, (unsigned)((maxcol + CB - 1) / CB), nblk);
                    const size_t sm = std::max<size_t>(stage, 16);
                    if (nl.max_np <= 9)
                        k_nl_apply_zb_staged<CT, 9><<<sg, kApplyChunkZ, sm, st>>>(
                            dB, dC, m, j, out, nl.ncov, nl.cov_pt, nl.cov_ptr, nl.ent_chi,
                            nl.ent_meta, nl.ent_slot, nl.chunk_row_ptr, nl.chunk_rows, chi_z<CT>(nl));
                    else
                        k_nl_apply_zb_staged<CT, 18><<<sg, kApplyChunkZ, sm, st>>>(
                            dB, dC, m, j, out, nl.ncov, nl.cov_pt, nl.cov_ptr, nl.ent_chi,
                            nl.ent_meta, nl.ent_slot, nl.chunk_row_ptr, nl.chunk_rows, chi_z<CT>(nl));
                } else {
                    const dim3 ag((nl.ncov + 255) / 256, nblk);
                    if (nl.max_np <= 9)
                        k_nl_apply_zb<CT, 9><<<ag, 256, 0, st>>>(dB, dC, m, j, out, nl.ncov,
                            nl.cov_pt, nl.cov_ptr, nl.ent_chi, nl.ent_meta, nl.chi64);
                    else
                        k_nl_apply_zb<CT, 18><<<ag, 256, 0, st>>>(dB, dC, m, j, out, nl.ncov,
                            nl.cov_pt, nl.cov_ptr, nl.ent_chi, nl.ent_meta, nl.chi64);
                }
                ctx->launches++;
            }
        }
        if (route && m == 2) {  // the degree-1 iterate is still in the scratch block
            for (int b = 0; b < nblk; b++)
                SGPU_CUDA_TRY(cudaMemcpy2DAsync(blk[b].X, sizeof(CT) * blk[b].ldi,
                                                W + (size_t)Nd * coloff[b], sizeof(CT) * Nd,
                                                sizeof(CT) * Nd, blk[b].ncol,
                                                cudaMemcpyDeviceToDevice, st));
        }
        SGPU_CUDA_TRY(cudaGetLastError());
        return SGPU_OK;
    };

    if (ctx->prof_on) return issue();  // per-launch events need plain launches
    std::vector<long> key = {(long)sizeof(CT), nblk, m, (long)(uintptr_t)tb, (long)(uintptr_t)W,
                             (long)(uintptr_t)alpha, (long)hg.size(), nslab, (long)pairs,
                             (long)(uintptr_t)ctx->veff64, (long)(uintptr_t)ctx->veff32};
    for (int b = 0; b < nblk; b++) {
        key.push_back(blk[b].ncol);
        key.push_back((long)(uintptr_t)blk[b].X);
        key.push_back((long)(uintptr_t)blk[b].Y);
    }
    if (!bs.exec || key != bs.key) {
        if (bs.exec) { cudaGraphExecDestroy(bs.exec); bs.exec = nullptr; }
        const long launches0 = ctx->launches;
        cudaGraph_t graph = nullptr;
        SGPU_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const int rc = issue();
        const cudaError_t ec = cudaStreamEndCapture(st, &graph);
        if (rc != SGPU_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        SGPU_CUDA_TRY(ec);
        const cudaError_t ei = cudaGraphInstantiate(&bs.exec, graph, 0);
        cudaGraphDestroy(graph);
        SGPU_CUDA_TRY(ei);
        bs.key = key;
        ks->batch_launches = ctx->launches - launches0;
        ctx->launches = launches0;
    }
    SGPU_CUDA_TRY(cudaGraphLaunch(bs.exec, st));
    ctx->launches += ks->batch_launches;
    return SGPU_OK;
}

template int hamiltonian_z<double2>(sgpu_ctx *, int, const double *, int, double, const double2 *,
                                    long, double2 *, long, double, double, const double2 *, long,
                                    cudaStream_t);
template int chebyshev_z<double2>(sgpu_ctx *, int, const double *, double2 *, long, double2 *,
                                  long, int, int, double, double, double, cudaStream_t);
template int chebyshev_z<float2>(sgpu_ctx *, int, const double *, float2 *, long, float2 *, long,
                                 int, int, double, double, double, cudaStream_t);

int kpoint_set_phases(sgpu_ctx *ctx, const double *k, cudaStream_t st) { return set_phases(ctx, k, st); }

// ---- Rayleigh-Ritz step at a k-point: DP_Project_Hamiltonian_kpt (src/eigenSolverKpt.c:676,
// Hp = Yᴴ HY and Mp = Yᴴ Y by ACCEL_ZGEMM / cblas_zgemm, :747-760),
// DP_Solve_Generalized_EigenProblem_kpt (:836, LAPACKE_zhegvd) and DP_Subspace_Rotation_kpt
// (:947, X = Y Q). The Ns x Ns products of these small blocks (C3: 64 states) go to cuBLAS
// (ZGEMM, or CGEMM for complex64 blocks), the eigenproblem to cuSOLVER zhegvd in complex128.

// Hp = Yᴴ HY, Mp = Yᴴ Y (ncol x ncol complex128, column-major, ld ncol)
template <typename CT>
int project_z(sgpu_ctx *ctx, int ncol, const CT *Y, long ldy, const CT *HY, long ldh,
              double2 *Hp, double2 *Mp, cudaStream_t st)
{
    SGPU_TRY(ensure_solver_handles(ctx));
    SGPU_CUBLAS_TRY(cublasSetStream(ctx->cublas, st));
    const int Nd = (int)ctx->Nd;
    if constexpr (sizeof(CT) == 16) {
        const cuDoubleComplex one = make_cuDoubleComplex(1.0, 0.0), zero = make_cuDoubleComplex(0.0, 0.0);
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        SGPU_CUBLAS_TRY(cublasZgemm(ctx->cublas, CUBLAS_OP_C, CUBLAS_OP_N, ncol, ncol, Nd, &one,
                                    Y, (int)ldy, Y, (int)ldy, &zero, Mp, ncol));
        SGPU_CUBLAS_TRY(cublasZgemm(ctx->cublas, CUBLAS_OP_C, CUBLAS_OP_N, ncol, ncol, Nd, &one,
                                    Y, (int)ldy, HY, (int)ldh, &zero, Hp, ncol));
    } else {
        float2 *tmp = nullptr;
        const size_t n2 = (size_t)ncol * ncol;
        SGPU_TRY(ws_get(ctx, WS_TC_PART, sizeof(float2) * 2 * n2, (void **)&tmp));
        const cuComplex one = make_cuComplex(1.f, 0.f), zero = make_cuComplex(0.f, 0.f);
        {
            ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
            SGPU_CUBLAS_TRY(cublasCgemm(ctx->cublas, CUBLAS_OP_C, CUBLAS_OP_N, ncol, ncol, Nd,
                                        &one, Y, (int)ldy, Y, (int)ldy, &zero, tmp, ncol));
            SGPU_CUBLAS_TRY(cublasCgemm(ctx->cublas, CUBLAS_OP_C, CUBLAS_OP_N, ncol, ncol, Nd,
                                        &one, Y, (int)ldy, HY, (int)ldh, &zero, tmp + n2, ncol));
        }
        SGPU_TRY(convert_cols<float, double>(reinterpret_cast<float *>(tmp), 2 * (long)n2,
                                             reinterpret_cast<double *>(Mp), 2 * (long)n2,
                                             2 * (long)n2, 1, st));
        SGPU_TRY(convert_cols<float, double>(reinterpret_cast<float *>(tmp + n2), 2 * (long)n2,
                                             reinterpret_cast<double *>(Hp), 2 * (long)n2,
                                             2 * (long)n2, 1, st));
    }
    return SGPU_OK;
}

// Hp q = lambda Mp q (upper triangles): Hp becomes Q, lambda (device) ascending
int generalized_eig_z(sgpu_ctx *ctx, int n, double2 *Hp, double2 *Mp, double *lambda_dev,
                      cudaStream_t st)
{
    SGPU_TRY(ensure_solver_handles(ctx));
    cusolverDnSetStream(ctx->cusolver, st);
    int lwork = 0;
    if (cusolverDnZhegvd_bufferSize(ctx->cusolver, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR,
                                    CUBLAS_FILL_MODE_UPPER, n, Hp, n, Mp, n, lambda_dev,
                                    &lwork) != CUSOLVER_STATUS_SUCCESS) {
        set_error("cusolverDnZhegvd_bufferSize failed");
        return SGPU_ERR_CUDA;
    }
    char *wsp = nullptr;
    SGPU_TRY(ws_get(ctx, WS_MISC, sizeof(double2) * ((size_t)lwork + 1) + 64, (void **)&wsp));
    double2 *work = reinterpret_cast<double2 *>(wsp);
    int *info = reinterpret_cast<int *>(wsp + sizeof(double2) * ((size_t)lwork + 1));
    {
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        if (cusolverDnZhegvd(ctx->cusolver, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR,
                             CUBLAS_FILL_MODE_UPPER, n, Hp, n, Mp, n, lambda_dev, work, lwork,
                             info) != CUSOLVER_STATUS_SUCCESS) {
            set_error("cusolverDnZhegvd failed to launch");
            return SGPU_ERR_CUDA;
        }
    }
    int hinfo = 0;
    SGPU_CUDA_TRY(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, st));
    SGPU_CUDA_TRY(cudaStreamSynchronize(st));
    if (hinfo != 0) {
        set_error("zhegvd: info = " + std::to_string(hinfo) +
                  (hinfo > n ? " (Mp is not positive definite)" : " (no convergence)"));
        return SGPU_ERR_LINALG;
    }
    return SGPU_OK;
}

// X = Y Q (Q ncol x ncol complex128, ld ncol)
template <typename CT>
int rotate_z(sgpu_ctx *ctx, int ncol, const CT *Y, long ldy, const double2 *Q, CT *X, long ldx,
             cudaStream_t st)
{
    SGPU_TRY(ensure_solver_handles(ctx));
    SGPU_CUBLAS_TRY(cublasSetStream(ctx->cublas, st));
    const int Nd = (int)ctx->Nd;
    if constexpr (sizeof(CT) == 16) {
        const cuDoubleComplex one = make_cuDoubleComplex(1.0, 0.0), zero = make_cuDoubleComplex(0.0, 0.0);
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        SGPU_CUBLAS_TRY(cublasZgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, Nd, ncol, ncol, &one,
                                    Y, (int)ldy, Q, ncol, &zero, X, (int)ldx));
    } else {
        float2 *q32 = nullptr;
        const long n2 = (long)ncol * ncol;
        SGPU_TRY(ws_get(ctx, WS_TC_PART, sizeof(float2) * n2, (void **)&q32));
        SGPU_TRY(convert_cols<double, float>(reinterpret_cast<const double *>(Q), 2 * n2,
                                             reinterpret_cast<float *>(q32), 2 * n2, 2 * n2, 1,
                                             st));
        const cuComplex one = make_cuComplex(1.f, 0.f), zero = make_cuComplex(0.f, 0.f);
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        SGPU_CUBLAS_TRY(cublasCgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, Nd, ncol, ncol, &one,
                                    Y, (int)ldy, q32, ncol, &zero, X, (int)ldx));
    }
    return SGPU_OK;
}

// Rayleigh-Ritz step of nblk blocks of equal width n in batched calls: H Y per block, then
// Hp = Yᴴ HY and Mp = Yᴴ Y for all blocks (batched ZGEMM / CGEMM), the generalized Hermitian
// eigenproblems Hp q = lambda Mp q reduced as zhegvd does (Mp = Uᴴ U by batched Cholesky,
// C = U⁻ᴴ Hp U⁻¹ by two batched triangular solves), all standard eigenproblems in one
// cusolverDnXsyevBatched call, Q = U⁻¹ V, and X = Y Q (batched). Ritz values land in lambda
// (host), block after block.
template <typename CT>
static int rr_batched(sgpu_ctx *ctx, int nblk, const sgpu_filter_block *blk, double *lambda,
                      cudaStream_t st)
{
    const int n = blk[0].ncol;
    const long n2 = (long)n * n;
    SGPU_TRY(ensure_solver_handles(ctx));
    SGPU_CUBLAS_TRY(cublasSetStream(ctx->cublas, st));
    cusolverDnSetStream(ctx->cusolver, st);
    // workspace: Hp, Mp (complex128, nblk n x n each), complex64 staging for CGEMM results,
    // eigenvalues, infos, pointer arrays
    char *ws = nullptr;
    const size_t zbytes = sizeof(double2) * 2 * (size_t)nblk * n2;
    const size_t cbytes = sizeof(CT) == 8 ? sizeof(float2) * 2 * (size_t)nblk * n2 : 0;
    const size_t wbytes = sizeof(double) * (size_t)nblk * n;
    const size_t ibytes = sizeof(int) * (size_t)(2 * nblk + 8);
    const size_t pbytes = sizeof(void *) * (size_t)(12 * nblk);
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t total = al(zbytes) + al(cbytes) + al(wbytes) + al(ibytes) + al(pbytes);
    SGPU_TRY(ws_get(ctx, WS_EIG, total, (void **)&ws));
    double2 *Hp = reinterpret_cast<double2 *>(ws), *Mp = Hp + (size_t)nblk * n2;
    char *q = ws + al(zbytes);
    float2 *Hc = reinterpret_cast<float2 *>(q), *Mc = Hc + (size_t)nblk * n2;
    q += al(cbytes);
    double *W = reinterpret_cast<double *>(q);
    q += al(wbytes);
    int *info = reinterpret_cast<int *>(q);
    q += al(ibytes);
    void **dptr = reinterpret_cast<void **>(q);
    // pointer arrays: Y, X (as HY and as the rotation output), Hp, Mp (or their complex64
    // staging), then the complex128 Hp, Mp for the solves
    std::vector<void *> hp(12 * (size_t)nblk);
    for (int b = 0; b < nblk; b++) {
        hp[b] = blk[b].Y;
        hp[nblk + b] = blk[b].X;
        hp[2 * nblk + b] = sizeof(CT) == 8 ? (void *)(Hc + b * n2) : (void *)(Hp + b * n2);
        hp[3 * nblk + b] = sizeof(CT) == 8 ? (void *)(Mc + b * n2) : (void *)(Mp + b * n2);
        hp[4 * nblk + b] = Hp + b * n2;
        hp[5 * nblk + b] = Mp + b * n2;
    }
    SGPU_CUDA_TRY(cudaMemcpyAsync(dptr, hp.data(), sizeof(void *) * 6 * nblk,
                                  cudaMemcpyHostToDevice, st));
    // H Y into X, block by block (each block's own k-point and spin)
    for (int b = 0; b < nblk; b++) {
        const sgpu_filter_block &f = blk[b];
        SGPU_TRY(set_phases(ctx, f.k, st));
        SGPU_TRY(hamiltonian_z<CT>(ctx, f.spin, f.k, n, 0.0, reinterpret_cast<CT *>(f.Y), f.ldo,
                                   reinterpret_cast<CT *>(f.X), f.ldi, 1.0, 0.0, nullptr, 0, st));
    }
    const int Nd = (int)ctx->Nd;
    {
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        if constexpr (sizeof(CT) == 16) {
            const cuDoubleComplex one = make_cuDoubleComplex(1.0, 0.0), zero = make_cuDoubleComplex(0.0, 0.0);
            auto P = [&](int i) { return reinterpret_cast<cuDoubleComplex **>(dptr + (size_t)i * nblk); };
            SGPU_CUBLAS_TRY(cublasZgemmBatched(ctx->cublas, CUBLAS_OP_C, CUBLAS_OP_N, n, n, Nd,
                                               &one, P(0), blk[0].ldo, P(0), blk[0].ldo, &zero,
                                               P(3), n, nblk));
            SGPU_CUBLAS_TRY(cublasZgemmBatched(ctx->cublas, CUBLAS_OP_C, CUBLAS_OP_N, n, n, Nd,
                                               &one, P(0), blk[0].ldo, P(1), blk[0].ldi, &zero,
                                               P(2), n, nblk));
        } else {
            const cuComplex one = make_cuComplex(1.f, 0.f), zero = make_cuComplex(0.f, 0.f);
            auto P = [&](int i) { return reinterpret_cast<cuComplex **>(dptr + (size_t)i * nblk); };
            SGPU_CUBLAS_TRY(cublasCgemmBatched(ctx->cublas, CUBLAS_OP_C, CUBLAS_OP_N, n, n, Nd,
                                               &one, P(0), blk[0].ldo, P(0), blk[0].ldo, &zero,
                                               P(3), n, nblk));
            SGPU_CUBLAS_TRY(cublasCgemmBatched(ctx->cublas, CUBLAS_OP_C, CUBLAS_OP_N, n, n, Nd,
                                               &one, P(0), blk[0].ldo, P(1), blk[0].ldi, &zero,
                                               P(2), n, nblk));
        }
    }
    if constexpr (sizeof(CT) == 8) {  // complex64 products to complex128 for the solves
        SGPU_TRY(convert_cols<float, double>(reinterpret_cast<float *>(Hc), 4 * nblk * n2,
                                             reinterpret_cast<double *>(Hp), 4 * nblk * n2,
                                             4 * nblk * n2, 1, st));
    }
    auto PZ = [&](int i) { return reinterpret_cast<cuDoubleComplex **>(dptr + (size_t)i * nblk); };
    {
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        // Mp = Uᴴ U
        if (cusolverDnZpotrfBatched(ctx->cusolver, CUBLAS_FILL_MODE_UPPER, n, PZ(5), n, info,
                                    nblk) != CUSOLVER_STATUS_SUCCESS) {
            set_error("cusolverDnZpotrfBatched failed to launch");
            return SGPU_ERR_CUDA;
        }
        const cuDoubleComplex one = make_cuDoubleComplex(1.0, 0.0);
        // C = U⁻ᴴ Hp U⁻¹
        SGPU_CUBLAS_TRY(cublasZtrsmBatched(ctx->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER,
                                           CUBLAS_OP_C, CUBLAS_DIAG_NON_UNIT, n, n, &one, PZ(5), n,
                                           PZ(4), n, nblk));
        SGPU_CUBLAS_TRY(cublasZtrsmBatched(ctx->cublas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_UPPER,
                                           CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, n, &one, PZ(5), n,
                                           PZ(4), n, nblk));
        // C V = V diag(lambda), all blocks in one call
        if (!ctx->xparams && cusolverDnCreateParams(&ctx->xparams) != CUSOLVER_STATUS_SUCCESS) {
            set_error("cusolverDnCreateParams failed");
            return SGPU_ERR_CUDA;
        }
        size_t dws = 0, hws = 0;
        if (cusolverDnXsyevBatched_bufferSize(ctx->cusolver, ctx->xparams, CUSOLVER_EIG_MODE_VECTOR,
                                              CUBLAS_FILL_MODE_UPPER, n, CUDA_C_64F, Hp, n,
                                              CUDA_R_64F, W, CUDA_C_64F, &dws, &hws,
                                              nblk) != CUSOLVER_STATUS_SUCCESS) {
            set_error("cusolverDnXsyevBatched_bufferSize failed");
            return SGPU_ERR_CUDA;
        }
        void *dwork = nullptr;
        SGPU_TRY(ws_get(ctx, WS_MISC, dws + 16, &dwork));
        if (ctx->xhost_bytes < hws) {
            free(ctx->xhost);
            ctx->xhost = hws ? malloc(hws) : nullptr;
            ctx->xhost_bytes = ctx->xhost ? hws : 0;
            if (hws && !ctx->xhost) {
                set_error("host workspace allocation failed");
                return SGPU_ERR_NOMEM;
            }
        }
        if (cusolverDnXsyevBatched(ctx->cusolver, ctx->xparams, CUSOLVER_EIG_MODE_VECTOR,
                                   CUBLAS_FILL_MODE_UPPER, n, CUDA_C_64F, Hp, n, CUDA_R_64F, W,
                                   CUDA_C_64F, dwork, dws, ctx->xhost, hws, info + nblk,
                                   nblk) != CUSOLVER_STATUS_SUCCESS) {
            set_error("cusolverDnXsyevBatched failed to launch");
            return SGPU_ERR_CUDA;
        }
        // Q = U⁻¹ V
        SGPU_CUBLAS_TRY(cublasZtrsmBatched(ctx->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER,
                                           CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, n, &one, PZ(5), n,
                                           PZ(4), n, nblk));
    }
    // X = Y Q
    {
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        if constexpr (sizeof(CT) == 16) {
            const cuDoubleComplex one = make_cuDoubleComplex(1.0, 0.0), zero = make_cuDoubleComplex(0.0, 0.0);
            auto P = [&](int i) { return reinterpret_cast<cuDoubleComplex **>(dptr + (size_t)i * nblk); };
            SGPU_CUBLAS_TRY(cublasZgemmBatched(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, Nd, n, n,
                                               &one, P(0), blk[0].ldo, P(4), n, &zero, P(1),
                                               blk[0].ldi, nblk));
        } else {
            SGPU_TRY(convert_cols<double, float>(reinterpret_cast<double *>(Hp), 2 * nblk * n2,
                                                 reinterpret_cast<float *>(Hc), 2 * nblk * n2,
                                                 2 * nblk * n2, 1, st));
            const cuComplex one = make_cuComplex(1.f, 0.f), zero = make_cuComplex(0.f, 0.f);
            auto P = [&](int i) { return reinterpret_cast<cuComplex **>(dptr + (size_t)i * nblk); };
            SGPU_CUBLAS_TRY(cublasCgemmBatched(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, Nd, n, n,
                                               &one, P(0), blk[0].ldo, P(2), n, &zero, P(1),
                                               blk[0].ldi, nblk));
        }
    }
    std::vector<int> hinfo(2 * nblk);
    SGPU_CUDA_TRY(cudaMemcpyAsync(lambda, W, sizeof(double) * (size_t)nblk * n,
                                  cudaMemcpyDeviceToHost, st));
    SGPU_CUDA_TRY(cudaMemcpyAsync(hinfo.data(), info, sizeof(int) * 2 * nblk,
                                  cudaMemcpyDeviceToHost, st));
    SGPU_CUDA_TRY(cudaStreamSynchronize(st));
    for (int b = 0; b < 2 * nblk; b++) {
        if (hinfo[b] != 0) {
            set_error(std::string(b < nblk ? "batched Cholesky of Mp" : "batched eigensolve") +
                      ": info = " + std::to_string(hinfo[b]) + " in block " +
                      std::to_string(b % nblk));
            return SGPU_ERR_LINALG;
        }
    }
    return SGPU_OK;
}

// One CheFSI pass over all (k, spin) blocks: the batched filter, then per block H Y into X,
// the projection, the eigenproblem and the rotation into X; lambda (host) receives each
// block's Ritz values, blocks one after another. Blocks of one width with common leading
// dimensions take the batched Rayleigh-Ritz step (ctx->rr_batched), others one block at a time.
template <typename CT>
int rayleigh_ritz_blocks(sgpu_ctx *ctx, int nblk, const sgpu_filter_block *blk, double *lambda,
                         cudaStream_t st)
{
    bool uniform = ctx->rr_batched && nblk > 0;
    for (int b = 1; b < nblk && uniform; b++)
        uniform = blk[b].ncol == blk[0].ncol && blk[b].ldi == blk[0].ldi &&
                  blk[b].ldo == blk[0].ldo;
    if (uniform && blk[0].ncol > 0) return rr_batched<CT>(ctx, nblk, blk, lambda, st);
    int nmax = 0;
    for (int b = 0; b < nblk; b++) nmax = std::max(nmax, blk[b].ncol);
    char *buf = nullptr;
    const size_t n2 = (size_t)nmax * nmax;
    SGPU_TRY(ws_get(ctx, WS_EIG, sizeof(double2) * 2 * n2 + sizeof(double) * nmax + 64,
                    (void **)&buf));
    double2 *Hp = reinterpret_cast<double2 *>(buf), *Mp = Hp + n2;
    double *dlam = reinterpret_cast<double *>(Mp + n2);
    long off = 0;
    for (int b = 0; b < nblk; b++) {
        const sgpu_filter_block &f = blk[b];
        if (f.ncol == 0) continue;
        CT *X = reinterpret_cast<CT *>(f.X);
        CT *Y = reinterpret_cast<CT *>(f.Y);
        SGPU_TRY(set_phases(ctx, f.k, st));
        SGPU_TRY(hamiltonian_z<CT>(ctx, f.spin, f.k, f.ncol, 0.0, Y, f.ldo, X, f.ldi, 1.0, 0.0,
                                   nullptr, 0, st));
        SGPU_TRY(project_z<CT>(ctx, f.ncol, Y, f.ldo, X, f.ldi, Hp, Mp, st));
        SGPU_TRY(generalized_eig_z(ctx, f.ncol, Hp, Mp, dlam, st));
        SGPU_TRY(rotate_z<CT>(ctx, f.ncol, Y, f.ldo, Hp, X, f.ldi, st));
        SGPU_CUDA_TRY(cudaMemcpyAsync(lambda + off, dlam, sizeof(double) * f.ncol,
                                      cudaMemcpyDeviceToHost, st));
        off += f.ncol;
    }
    SGPU_CUDA_TRY(cudaStreamSynchronize(st));
    return SGPU_OK;
}

template <typename CT>
int chefsi_batched(sgpu_ctx *ctx, int nblk, const sgpu_filter_block *blk, int m,
                   double *lambda, cudaStream_t st)
{
    SGPU_TRY(chebyshev_batched<CT>(ctx, nblk, blk, m, st));
    return rayleigh_ritz_blocks<CT>(ctx, nblk, blk, lambda, st);
}

template int chefsi_batched<double2>(sgpu_ctx *, int, const sgpu_filter_block *, int, double *,
                                     cudaStream_t);
template int chefsi_batched<float2>(sgpu_ctx *, int, const sgpu_filter_block *, int, double *,
                                    cudaStream_t);

// Graded pass: the complex64 filter of b32 (X -> Y), its result widened into b64's Y, the
// complex128 Rayleigh-Ritz step on b64 (Ritz vectors into b64's X), and those narrowed into
// b32's X for the next filter. The two descriptor sets describe the same blocks (same ncol,
// k-point and spin).
int chefsi_batched_graded(sgpu_ctx *ctx, int nblk, const sgpu_filter_block *b32,
                          const sgpu_filter_block *b64, int m, double *lambda, cudaStream_t st)
{
    SGPU_TRY(chebyshev_batched<float2>(ctx, nblk, b32, m, st));
    for (int b = 0; b < nblk; b++)
        if (b32[b].ncol > 0)
            SGPU_TRY((convert_cols<float, double>(
                reinterpret_cast<const float *>(b32[b].Y), 2L * b32[b].ldo,
                reinterpret_cast<double *>(b64[b].Y), 2L * b64[b].ldo, 2L * ctx->Nd,
                b32[b].ncol, st)));
    SGPU_TRY(rayleigh_ritz_blocks<double2>(ctx, nblk, b64, lambda, st));
    for (int b = 0; b < nblk; b++)
        if (b32[b].ncol > 0)
            SGPU_TRY((convert_cols<double, float>(
                reinterpret_cast<const double *>(b64[b].X), 2L * b64[b].ldi,
                reinterpret_cast<float *>(b32[b].X), 2L * b32[b].ldi, 2L * ctx->Nd,
                b32[b].ncol, st)));
    return SGPU_OK;
}

}  // namespace sgpu

using namespace sgpu;

namespace {
int kcheck(sgpu_ctx *ctx, int ncol, int ldi, int ldo)
{
    if (!ctx) {
        set_error("null context");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    if (ncol < 0 || ldi < ctx->Nd || ldo < ctx->Nd) {
        set_error("column block: need ncol >= 0 and leading dimensions >= Nd");
        return SGPU_ERR_ARG;
    }
    return SGPU_OK;
}

// complex column block to the device (interleaved doubles): device pointer with its ld
int zstage_in(sgpu_ctx *ctx, int slot, const double *x, int ld, int ncol, bool copy,
              double2 **d, long *ldd)
{
    if (is_device_ptr(x)) {
        *d = reinterpret_cast<double2 *>(const_cast<double *>(x));
        *ldd = ld;
        return SGPU_OK;
    }
    SGPU_TRY(ws_get(ctx, slot, sizeof(double2) * (size_t)ctx->Nd * (ncol > 0 ? ncol : 1),
                    (void **)d));
    if (copy && ncol > 0)
        SGPU_CUDA_TRY(cudaMemcpy2DAsync(*d, sizeof(double2) * ctx->Nd, x, sizeof(double2) * ld,
                                        sizeof(double2) * ctx->Nd, ncol, cudaMemcpyHostToDevice,
                                        ctx->stream));
    *ldd = ctx->Nd;
    return SGPU_OK;
}

int zstage_out(sgpu_ctx *ctx, const double2 *d, long ldd, double *y, int ld, int ncol)
{
    if ((const void *)d == (const void *)y || ncol <= 0) return SGPU_OK;
    SGPU_CUDA_TRY(cudaMemcpy2DAsync(y, sizeof(double2) * ld, d, sizeof(double2) * ldd,
                                    sizeof(double2) * ctx->Nd, ncol, cudaMemcpyDeviceToHost,
                                    ctx->stream));
    return SGPU_OK;
}
}  // namespace

extern "C" {

int sgpu_set_kpoint_geometry(sgpu_ctx *ctx, double Lx, double Ly, double Lz, int n_img,
                             const double *img_coords)
{
    if (!ctx || !(Lx > 0 && Ly > 0 && Lz > 0) || n_img < 0 || (n_img > 0 && !img_coords)) {
        set_error("sgpu_set_kpoint_geometry: bad arguments");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    kpoint_free(ctx);
    KpointState *ks = new KpointState();
    ks->L[0] = Lx; ks->L[1] = Ly; ks->L[2] = Lz;
    ks->nimg = n_img;
    ks->img_coords.assign(img_coords, img_coords + 3 * (size_t)n_img);
    if (n_img > 0 && cudaMalloc(&ks->img_phase, sizeof(double2) * n_img) != cudaSuccess) {
        delete ks;
        set_error("sgpu_set_kpoint_geometry: device allocation failed");
        return SGPU_ERR_NOMEM;
    }
    ctx->kp = ks;
    return SGPU_OK;
}

int sgpu_Lap_plus_diag_vec_mult_orth_kpt(sgpu_ctx *ctx, const double *k, int ncol, double a,
                                         double b, double c, const double *v, const double *x,
                                         int ldi, double *y, int ldo)
{
    SGPU_TRY(kcheck(ctx, ncol, ldi, ldo));
    if (ncol == 0) return SGPU_OK;
    double2 *dx, *dy;
    long lx, ly;
    SGPU_TRY(zstage_in(ctx, WS_STAGE_A, x, ldi, ncol, true, &dx, &lx));
    SGPU_TRY(zstage_in(ctx, WS_STAGE_B, y, ldo, ncol, false, &dy, &ly));
    double *dv = nullptr;
    if (v && !(std::fabs(b) < 1e-14)) {
        if (is_device_ptr(v)) {
            dv = const_cast<double *>(v);
        } else {
            SGPU_TRY(ws_get(ctx, WS_RHS, sizeof(double) * ctx->Nd, (void **)&dv));
            SGPU_CUDA_TRY(cudaMemcpyAsync(dv, v, sizeof(double) * ctx->Nd, cudaMemcpyHostToDevice,
                                          ctx->stream));
        }
    }
    SGPU_TRY(stencil_z<double2>(ctx, k, ncol, a, dv ? b : 0.0, c, dv, nullptr, dx, lx, dy, ly,
                                1.0, 0.0, nullptr, 0, ctx->stream));
    SGPU_TRY(zstage_out(ctx, dy, ly, y, ldo, ncol));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_Vnl_vec_mult_kpt(sgpu_ctx *ctx, const double *k, int ncol, const double *x, int ldi,
                          double *Hx, int ldo)
{
    SGPU_TRY(kcheck(ctx, ncol, ldi, ldo));
    if (ncol == 0 || !ctx->has_nl) return SGPU_OK;
    double2 *dx, *dh;
    long lx, lh;
    SGPU_TRY(zstage_in(ctx, WS_STAGE_A, x, ldi, ncol, true, &dx, &lx));
    SGPU_TRY(zstage_in(ctx, WS_STAGE_B, Hx, ldo, ncol, true, &dh, &lh));
    SGPU_TRY(set_phases(ctx, k, ctx->stream));
    SGPU_TRY(nonlocal_z<double2>(ctx, ncol, dx, lx, dh, lh, 1.0, ctx->stream));
    SGPU_TRY(zstage_out(ctx, dh, lh, Hx, ldo, ncol));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_Hamiltonian_vectors_mult_kpt(sgpu_ctx *ctx, int spin, const double *k, int ncol,
                                      double c, const double *x, int ldi, double *Hx, int ldo)
{
    SGPU_TRY(kcheck(ctx, ncol, ldi, ldo));
    if (ncol == 0) return SGPU_OK;
    double2 *dx, *dh;
    long lx, lh;
    SGPU_TRY(zstage_in(ctx, WS_STAGE_A, x, ldi, ncol, true, &dx, &lx));
    SGPU_TRY(zstage_in(ctx, WS_STAGE_B, Hx, ldo, ncol, false, &dh, &lh));
    SGPU_TRY(set_phases(ctx, k, ctx->stream));
    SGPU_TRY(hamiltonian_z<double2>(ctx, spin, k, ncol, c, dx, lx, dh, lh, 1.0, 0.0, nullptr, 0,
                                    ctx->stream));
    SGPU_TRY(zstage_out(ctx, dh, lh, Hx, ldo, ncol));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_ChebyshevFiltering_kpt(sgpu_ctx *ctx, int spin, const double *k, double *X, int ldi,
                                double *Y, int ldo, int ncol, int m, double a, double b,
                                double a0, int precision)
{
    SGPU_TRY(kcheck(ctx, ncol, ldi, ldo));
    if (precision != SGPU_PREC_FP64 && precision != SGPU_PREC_FP32) {
        set_error("ChebyshevFiltering_kpt: precision must be SGPU_PREC_FP64 or SGPU_PREC_FP32");
        return SGPU_ERR_ARG;
    }
    if (!(b > a) || !(a > a0) || m < 1) {
        set_error("ChebyshevFiltering_kpt: need a0 < a < b and m >= 1");
        return SGPU_ERR_ARG;
    }
    if (ncol == 0) return SGPU_OK;
    double2 *dX, *dY;
    long lX, lY;
    SGPU_TRY(zstage_in(ctx, WS_STAGE_A, X, ldi, ncol, true, &dX, &lX));
    SGPU_TRY(zstage_in(ctx, WS_STAGE_B, Y, ldo, ncol, false, &dY, &lY));
    SGPU_TRY(set_phases(ctx, k, ctx->stream));
    SGPU_CUDA_TRY(cudaEventRecord(ctx->ev0, ctx->stream));
    if (precision == SGPU_PREC_FP64) {
        SGPU_TRY(chebyshev_z<double2>(ctx, spin, k, dX, lX, dY, lY, ncol, m, a, b, a0, ctx->stream));
    } else {
        float2 *fX = nullptr;
        const size_t fb = sizeof(float2) * (size_t)ctx->Nd * ncol;
        SGPU_TRY(ws_get(ctx, WS_MISC, 2 * fb, (void **)&fX));
        float2 *fY = fX + (size_t)ctx->Nd * ncol;
        SGPU_TRY(convert_cols<double, float>(reinterpret_cast<double *>(dX), 2 * lX,
                                             reinterpret_cast<float *>(fX), 2 * ctx->Nd,
                                             2 * ctx->Nd, ncol, ctx->stream));
        SGPU_TRY(chebyshev_z<float2>(ctx, spin, k, fX, ctx->Nd, fY, ctx->Nd, ncol, m, a, b, a0,
                                     ctx->stream));
        SGPU_TRY(convert_cols<float, double>(reinterpret_cast<float *>(fX), 2 * ctx->Nd,
                                             reinterpret_cast<double *>(dX), 2 * lX,
                                             2 * ctx->Nd, ncol, ctx->stream));
        SGPU_TRY(convert_cols<float, double>(reinterpret_cast<float *>(fY), 2 * ctx->Nd,
                                             reinterpret_cast<double *>(dY), 2 * lY,
                                             2 * ctx->Nd, ncol, ctx->stream));
        ctx->launches += 3;
    }
    SGPU_CUDA_TRY(cudaEventRecord(ctx->ev1, ctx->stream));
    SGPU_TRY(zstage_out(ctx, dX, lX, X, ldi, ncol));
    SGPU_TRY(zstage_out(ctx, dY, lY, Y, ldo, ncol));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    SGPU_CUDA_TRY(cudaEventElapsedTime(&ctx->last_filter_ms, ctx->ev0, ctx->ev1));
    return SGPU_OK;
}

// argument checks shared by the batched filter and the batched CheFSI pass
static int batched_check(sgpu_ctx *ctx, int nblk, const sgpu_filter_block *blocks, int m,
                         int precision)
{
    if (!ctx || nblk < 0 || (nblk > 0 && !blocks) || m < 1) {
        set_error("ChebyshevFiltering_batched: need a context, nblk >= 0 blocks and m >= 1");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    if (precision != SGPU_PREC_FP64 && precision != SGPU_PREC_FP32) {
        set_error("ChebyshevFiltering_batched: precision must be SGPU_PREC_FP64 (complex128) or "
                  "SGPU_PREC_FP32 (complex64)");
        return SGPU_ERR_ARG;
    }
    for (int b = 0; b < nblk; b++) {
        const sgpu_filter_block &f = blocks[b];
        if (f.ncol < 0 || f.ldi < ctx->Nd || f.ldo < ctx->Nd || f.spin < 0) {
            set_error("ChebyshevFiltering_batched: block " + std::to_string(b) +
                      ": need ncol >= 0, spin >= 0 and leading dimensions >= Nd");
            return SGPU_ERR_ARG;
        }
        if (f.ncol > 0 && (!is_device_ptr(f.X) || !is_device_ptr(f.Y))) {
            set_error("ChebyshevFiltering_batched: block " + std::to_string(b) +
                      ": X and Y must be device memory");
            return SGPU_ERR_ARG;
        }
        if (!(f.b > f.a) || !(f.a > f.a0)) {
            set_error("ChebyshevFiltering_batched: block " + std::to_string(b) +
                      ": need a0 < a < b");
            return SGPU_ERR_ARG;
        }
    }
    return SGPU_OK;
}

// complex Ns x Ns matrix to the device (interleaved doubles, ld n)
static int zmat_in(sgpu_ctx *ctx, int slot, const double *h, int n, bool copy, double2 **d)
{
    if (is_device_ptr(h)) {
        *d = reinterpret_cast<double2 *>(const_cast<double *>(h));
        return SGPU_OK;
    }
    SGPU_TRY(ws_get(ctx, slot, sizeof(double2) * (size_t)n * n, (void **)d));
    if (copy)
        SGPU_CUDA_TRY(cudaMemcpyAsync(*d, h, sizeof(double2) * (size_t)n * n,
                                      cudaMemcpyHostToDevice, ctx->stream));
    return SGPU_OK;
}

static int zmat_out(sgpu_ctx *ctx, const double2 *d, double *h, int n)
{
    if ((const void *)d == (const void *)h) return SGPU_OK;
    SGPU_CUDA_TRY(cudaMemcpyAsync(h, d, sizeof(double2) * (size_t)n * n, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    return SGPU_OK;
}

int sgpu_Project_Hamiltonian_kpt(sgpu_ctx *ctx, int spin, const double *k, const double *Y,
                                 int ldi, double *HY, int ldo, int ncol, double *Hp, double *Mp)
{
    SGPU_TRY(kcheck(ctx, ncol, ldi, ldo));
    if (!k || !Hp || !Mp) {
        set_error("Project_Hamiltonian_kpt: null argument");
        return SGPU_ERR_ARG;
    }
    if (ncol == 0) return SGPU_OK;
    double2 *dY, *dH, *dHp, *dMp;
    long lY, lH;
    SGPU_TRY(zstage_in(ctx, WS_STAGE_A, Y, ldi, ncol, true, &dY, &lY));
    SGPU_TRY(zstage_in(ctx, WS_STAGE_B, HY, ldo, ncol, false, &dH, &lH));
    SGPU_TRY(zmat_in(ctx, WS_POIS, Hp, ncol, false, &dHp));
    SGPU_TRY(zmat_in(ctx, WS_MIX, Mp, ncol, false, &dMp));
    SGPU_TRY(kpoint_set_phases(ctx, k, ctx->stream));
    SGPU_TRY(hamiltonian_z<double2>(ctx, spin, k, ncol, 0.0, dY, lY, dH, lH, 1.0, 0.0, nullptr,
                                    0, ctx->stream));
    SGPU_TRY(project_z<double2>(ctx, ncol, dY, lY, dH, lH, dHp, dMp, ctx->stream));
    SGPU_TRY(zstage_out(ctx, dH, lH, HY, ldo, ncol));
    SGPU_TRY(zmat_out(ctx, dHp, Hp, ncol));
    SGPU_TRY(zmat_out(ctx, dMp, Mp, ncol));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_Solve_Generalized_EigenProblem_kpt(sgpu_ctx *ctx, int Ns, double *Hp, double *Mp,
                                            double *lambda)
{
    if (!ctx || Ns <= 0 || !Hp || !Mp || !lambda) {
        set_error("Solve_Generalized_EigenProblem_kpt: bad arguments");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    double2 *dHp, *dMp;
    SGPU_TRY(zmat_in(ctx, WS_POIS, Hp, Ns, true, &dHp));
    SGPU_TRY(zmat_in(ctx, WS_MIX, Mp, Ns, true, &dMp));
    double *dl = lambda;
    if (!is_device_ptr(lambda)) SGPU_TRY(ws_get(ctx, WS_RED, sizeof(double) * Ns, (void **)&dl));
    SGPU_TRY(generalized_eig_z(ctx, Ns, dHp, dMp, dl, ctx->stream));
    SGPU_TRY(zmat_out(ctx, dHp, Hp, Ns));
    SGPU_TRY(zmat_out(ctx, dMp, Mp, Ns));
    if (dl != lambda)
        SGPU_CUDA_TRY(cudaMemcpyAsync(lambda, dl, sizeof(double) * Ns, cudaMemcpyDeviceToHost,
                                      ctx->stream));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_Subspace_Rotation_kpt(sgpu_ctx *ctx, const double *Y, int ldi, const double *Q,
                               int ncol, double *X, int ldo)
{
    SGPU_TRY(kcheck(ctx, ncol, ldi, ldo));
    if (!Q) {
        set_error("Subspace_Rotation_kpt: null Q");
        return SGPU_ERR_ARG;
    }
    if (ncol == 0) return SGPU_OK;
    double2 *dY, *dX, *dQ;
    long lY, lX;
    SGPU_TRY(zstage_in(ctx, WS_STAGE_A, Y, ldi, ncol, true, &dY, &lY));
    SGPU_TRY(zstage_in(ctx, WS_STAGE_B, X, ldo, ncol, false, &dX, &lX));
    SGPU_TRY(zmat_in(ctx, WS_POIS, Q, ncol, true, &dQ));
    SGPU_TRY(rotate_z<double2>(ctx, ncol, dY, lY, dQ, dX, lX, ctx->stream));
    SGPU_TRY(zstage_out(ctx, dX, lX, X, ldo, ncol));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_CheFSI_batched(sgpu_ctx *ctx, int nblk, const sgpu_filter_block *blocks, int m,
                        int precision, double *lambda)
{
    SGPU_TRY(batched_check(ctx, nblk, blocks, m, precision));
    if (nblk == 0) return SGPU_OK;
    if (!lambda) {
        set_error("CheFSI_batched: null lambda");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaEventRecord(ctx->ev0, ctx->stream));
    if (precision == SGPU_PREC_FP64)
        SGPU_TRY(chefsi_batched<double2>(ctx, nblk, blocks, m, lambda, ctx->stream));
    else
        SGPU_TRY(chefsi_batched<float2>(ctx, nblk, blocks, m, lambda, ctx->stream));
    SGPU_CUDA_TRY(cudaEventRecord(ctx->ev1, ctx->stream));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    SGPU_CUDA_TRY(cudaEventElapsedTime(&ctx->last_filter_ms, ctx->ev0, ctx->ev1));
    return SGPU_OK;
}

int sgpu_ChebyshevFiltering_batched(sgpu_ctx *ctx, int nblk, const sgpu_filter_block *blocks,
                                    int m, int precision)
{
    SGPU_TRY(batched_check(ctx, nblk, blocks, m, precision));
    if (nblk == 0) return SGPU_OK;
    SGPU_CUDA_TRY(cudaEventRecord(ctx->ev0, ctx->stream));
    if (precision == SGPU_PREC_FP64)
        SGPU_TRY(chebyshev_batched<double2>(ctx, nblk, blocks, m, ctx->stream));
    else
        SGPU_TRY(chebyshev_batched<float2>(ctx, nblk, blocks, m, ctx->stream));
    SGPU_CUDA_TRY(cudaEventRecord(ctx->ev1, ctx->stream));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    SGPU_CUDA_TRY(cudaEventElapsedTime(&ctx->last_filter_ms, ctx->ev0, ctx->ev1));
    return SGPU_OK;
}

}  // extern "C"
