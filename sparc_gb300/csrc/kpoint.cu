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
#include <vector>

#include "sgpu_internal.h"

namespace sgpu {
namespace {

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

template <typename CT>
__device__ __forceinline__ CT phase(double theta)
{
    double s, c;
    sincos(theta, &s, &c);
    using R = typename Real<CT>::type;
    return CT{(R)c, (R)s};
}

// one point per thread, z-register queue, shared plane with x/y halo (as the real kernel);
// every fetched value is multiplied by the Bloch factor of its unwrapped position
template <typename CT, int R, int BX, int BY>
__global__ void __launch_bounds__(BX *BY) k_stencil_z(const StencilZParams<CT> p)
{
    using RT = typename Real<CT>::type;
    __shared__ CT s[BY + 2 * R][BX + 2 * R];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    const int col = blockIdx.z / p.nslab;
    const int slab = blockIdx.z - col * p.nslab;
    const int zs = slab * p.zlen;
    const int ze = min(zs + p.zlen, p.Nz);
    if (zs >= ze) return;
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
    auto zload = [&](int kr) {  // own column at unwrapped plane kr
        const CT val = __ldg(xc + own + (long)wrapz(kr, p.Nz) * NxNy);
        return cmul(cmul(val, f_own), phase<CT>(floordiv(kr, p.Nz) * p.k.kLz));
    };
    CT q[2 * R + 1];
#pragma unroll
    for (int m = 0; m < 2 * R; m++) q[m] = zload(zs - R + m);
    for (int k = zs; k < ze; k++) {
        q[2 * R] = zload(k + R);
        const long pk = (long)k * NxNy;
        __syncthreads();
        s[ty + R][tx + R] = q[R];
        if (hx) {
            s[ty + R][tx] = cmul(__ldg(xc + pk + hxl), f_xl);
            s[ty + R][tx + BX + R] = cmul(__ldg(xc + pk + hxr), f_xr);
        }
        if (hy) {
            s[ty][tx + R] = cmul(__ldg(xc + pk + hyl), f_yl);
            s[ty + BY + R][tx + R] = cmul(__ldg(xc + pk + hyr), f_yr);
        }
        __syncthreads();
        if (active) {
            CT res = cscale(q[R], (RT)p.c0);
#pragma unroll
            for (int r = 1; r <= R; r++) {
                const CT rx = cscale(cadd(s[ty + R][tx + R - r], s[ty + R][tx + R + r]), (RT)p.wx[r]);
                const CT ry = cscale(cadd(s[ty + R - r][tx + R], s[ty + R + r][tx + R]), (RT)p.wy[r]);
                const CT rz = cscale(cadd(q[R - r], q[R + r]), (RT)p.wz[r]);
                res = cadd(res, cadd(cadd(rx, ry), rz));
            }
            const long pt = own + pk;
            if (p.v) res = cadd(res, cscale(q[R], (RT)(p.bv * p.v[pt])));
            if (p.v32) res = cadd(res, cscale(q[R], (RT)p.bv * p.v32[pt]));
            CT o = cscale(res, (RT)p.s1);
            if (zc) o = cadd(o, cscale(zc[pt], (RT)p.s2));
            oc[pt] = o;
        }
#pragma unroll
        for (int m = 0; m < 2 * R; m++) q[m] = q[m + 1];
    }
}

// projection: block = (atom image g, group of 32 columns), threads stride over the image's
// points; alpha[row * lda + n] += e^{i theta_g} dV Gamma_row sum_i Chi[i, j] x[gp_i, n]
template <typename CT, int MAXJ>
__global__ void __launch_bounds__(256)
    k_nl_project_z(const int *__restrict__ img_atom, const int *__restrict__ img_ndc,
                   const long *__restrict__ img_off, const long *__restrict__ img_chi_off,
                   const int *__restrict__ grid_pos, const double *__restrict__ chi,
                   const int *__restrict__ ip_displ, const double *__restrict__ gamma,
                   const double2 *__restrict__ img_phase, int ncol, const CT *__restrict__ x,
                   long ldx, CT *__restrict__ alpha, long lda, double dV)
{
    using RT = typename Real<CT>::type;
    constexpr int NC = 32, PG = 8;  // 32 columns x 8 point groups
    const int g = blockIdx.x;
    const int n0 = blockIdx.y * NC;
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

// apply: one thread per covered point, all columns; Hx[p] += s1 e^{-i theta_g} Chi alpha
template <typename CT, int NPMAX>
__global__ void __launch_bounds__(256)
    k_nl_apply_z(int ncov, const int *__restrict__ cov_pt, const int *__restrict__ cov_ptr,
                 const long *__restrict__ ent_chi, const int4 *__restrict__ ent_meta,
                 const double *__restrict__ chi, const double2 *__restrict__ img_phase,
                 int ncol, const CT *__restrict__ alpha, long lda, double scale,
                 CT *__restrict__ out, long ldo)
{
    using RT = typename Real<CT>::type;
    const int cidx = blockIdx.x * blockDim.x + threadIdx.x;
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

}  // namespace

// ------------------------------------------------------------------ host side

struct KpointState {
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
    constexpr int R = 6, BX = 32, BY = 8;
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
        k_stencil_z<CT, R, BX, BY><<<dim3(tilesx, tilesy, nc * nslab), dim3(BX, BY), 0, st>>>(q);
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
        const int blocks = (nl.ncov + 255) / 256;
        if (nl.max_np <= 9)
            k_nl_apply_z<CT, 9><<<blocks, 256, 0, st>>>(nl.ncov, nl.cov_pt, nl.cov_ptr,
                nl.ent_chi, nl.ent_meta, nl.chi64, ks->img_phase, ncol, alpha, lda, scale, out, ldo);
        else
            k_nl_apply_z<CT, 18><<<blocks, 256, 0, st>>>(nl.ncov, nl.cov_pt, nl.cov_ptr,
                nl.ent_chi, nl.ent_meta, nl.chi64, ks->img_phase, ncol, alpha, lda, scale, out, ldo);
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

template int hamiltonian_z<double2>(sgpu_ctx *, int, const double *, int, double, const double2 *,
                                    long, double2 *, long, double, double, const double2 *, long,
                                    cudaStream_t);
template int chebyshev_z<double2>(sgpu_ctx *, int, const double *, double2 *, long, double2 *,
                                  long, int, int, double, double, double, cudaStream_t);
template int chebyshev_z<float2>(sgpu_ctx *, int, const double *, float2 *, long, float2 *, long,
                                 int, int, double, double, double, cudaStream_t);

int kpoint_set_phases(sgpu_ctx *ctx, const double *k, cudaStream_t st) { return set_phases(ctx, k, st); }

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

}  // extern "C"
