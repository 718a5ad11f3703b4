// Radius-6 finite-difference stencil for an orthogonal periodic grid, fused with the diagonal
// (local potential), the shift and the Chebyshev three-term update:
//
//   out[:, n] = s1 * ( a*Lap + bv*diag(v) + c*I ) x[:, n]  +  s2 * z[:, n]
//
// This one kernel serves Lap_plus_diag_vec_mult_orth (src/lapVecRoutines.c:306, with
// s1 = 1, s2 = 0), the local part of Hamiltonian_vectors_mult
// (src/hamiltonianVecRoutines.c:45, a = -0.5, bv = 1) and each degree of ChebyshevFiltering
// (src/eigenSolver.c:722-798, s1 = 2*sigma2/e, s2 = -sigma*sigma2, z = X), so the recurrence
// costs no extra pass over HBM.
//
// Layout: column-major blocks with leading dimension ld, grid index i + j*Nx + k*Nx*Ny.
// Each thread block owns a BX x BY tile of an xy-plane for one column and marches along z:
// the z-neighbours of a thread's point live in a register queue of 2R+1 values, the current
// plane plus its x/y halo lives in shared memory, and periodic images are resolved by
// wrapping indices while loading (no ghost-extended copy, unlike the reference's x_ex).
#include "sgpu_internal.h"

namespace sgpu {
namespace {

template <typename T>
struct StencilParams {
    const T *__restrict__ x;
    T *__restrict__ out;
    const T *__restrict__ z;
    const T *__restrict__ v;
    long ldx, ldo, ldz;
    int Nx, Ny, Nz, nslab, zlen;
    T wx[kMaxFDn + 1], wy[kMaxFDn + 1], wz[kMaxFDn + 1];
    T c0, bv, s1, s2;
};

__device__ __forceinline__ int wrapi(int i, int n)
{
    i %= n;
    return i < 0 ? i + n : i;
}

template <typename T, int R, int BX, int BY>
__global__ void __launch_bounds__(BX *BY)
    k_stencil_orth(const StencilParams<T> p)
{
    __shared__ T s[BY + 2 * R][BX + 2 * R];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    const int col = blockIdx.z / p.nslab;
    const int slab = blockIdx.z - col * p.nslab;
    const int zs = slab * p.zlen;
    const int ze = min(zs + p.zlen, p.Nz);
    if (zs >= ze) return;

    const int i = x0 + tx, j = y0 + ty;
    const bool active = (i < p.Nx) && (j < p.Ny);
    const int gi = wrapi(i, p.Nx), gj = wrapi(j, p.Ny);
    const long NxNy = (long)p.Nx * p.Ny;

    const T *__restrict__ xc = p.x + (long)col * p.ldx;
    const long own = gi + (long)gj * p.Nx;

    // halo source offsets within a plane (x-halo: left/right; y-halo: top/bottom)
    long hxl = 0, hxr = 0, hyl = 0, hyr = 0;
    if (tx < R) {
        hxl = wrapi(x0 - R + tx, p.Nx) + (long)gj * p.Nx;
        hxr = wrapi(x0 + BX + tx, p.Nx) + (long)gj * p.Nx;
    }
    if (ty < R) {
        hyl = gi + (long)wrapi(y0 - R + ty, p.Ny) * p.Nx;
        hyr = gi + (long)wrapi(y0 + BY + ty, p.Ny) * p.Nx;
    }

    T q[2 * R + 1];
#pragma unroll
    for (int m = 0; m < 2 * R; m++) q[m] = __ldg(xc + own + (long)wrapi(zs - R + m, p.Nz) * NxNy);

    for (int k = zs; k < ze; k++) {
        q[2 * R] = __ldg(xc + own + (long)wrapi(k + R, p.Nz) * NxNy);
        const long pk = (long)k * NxNy;
        __syncthreads();  // previous plane fully consumed
        s[ty + R][tx + R] = q[R];
        if (tx < R) {
            s[ty + R][tx] = __ldg(xc + pk + hxl);
            s[ty + R][tx + BX + R] = __ldg(xc + pk + hxr);
        }
        if (ty < R) {
            s[ty][tx + R] = __ldg(xc + pk + hyl);
            s[ty + BY + R][tx + R] = __ldg(xc + pk + hyr);
        }
        __syncthreads();
        if (active) {
            T res = p.c0 * q[R];
#pragma unroll
            for (int r = 1; r <= R; r++) {
                T rx = (s[ty + R][tx + R - r] + s[ty + R][tx + R + r]) * p.wx[r];
                T ry = (s[ty + R - r][tx + R] + s[ty + R + r][tx + R]) * p.wy[r];
                T rz = (q[R - r] + q[R + r]) * p.wz[r];
                res += rx + ry + rz;
            }
            const long pt = own + pk;
            if (p.v) res += p.bv * (__ldg(p.v + pt) * q[R]);
            T o = p.s1 * res;
            if (p.z) o += p.s2 * p.z[(long)col * p.ldz + pt];
            p.out[(long)col * p.ldo + pt] = o;
        }
#pragma unroll
        for (int m = 0; m < 2 * R; m++) q[m] = q[m + 1];
    }
}

}  // namespace

template <typename T>
int launch_stencil(sgpu_ctx *ctx, int ncol, double a, double bv, double c, const T *v,
                   const T *x, long ldx, T *out, long ldo, double s1, double s2, const T *z,
                   long ldz, cudaStream_t st)
{
    constexpr int R = 6, BX = 32, BY = 8;
    if (ctx->FDn != R) {
        set_error("stencil: only FD order 12 (radius 6) is built");
        return SGPU_ERR_ARG;
    }
    if (ncol <= 0) return SGPU_OK;
    StencilParams<T> p;
    p.x = x; p.out = out; p.z = z; p.v = v;
    p.ldx = ldx; p.ldo = ldo; p.ldz = ldz;
    p.Nx = ctx->Nx; p.Ny = ctx->Ny; p.Nz = ctx->Nz;
    for (int r = 0; r <= R; r++) {
        p.wx[r] = (T)(ctx->cx[r] * a);
        p.wy[r] = (T)(ctx->cy[r] * a);
        p.wz[r] = (T)(ctx->cz[r] * a);
    }
    // centre weight as the reference forms it: a*wx0 + a*wy0 + a*wz0 + c
    double c0 = ctx->cx[0] * a;
    c0 += ctx->cy[0] * a;
    c0 += ctx->cz[0] * a;
    c0 += c;
    p.c0 = (T)c0;
    p.bv = (T)bv; p.s1 = (T)s1; p.s2 = (T)s2;
    if (!v || fabs(bv) < 1e-14) p.v = nullptr;
    if (!z || s2 == 0.0) p.z = nullptr;

    const int tilesx = (ctx->Nx + BX - 1) / BX, tilesy = (ctx->Ny + BY - 1) / BY;
    // split z into slabs until there are enough blocks to fill 152 SMs several times over
    long blocks1 = (long)tilesx * tilesy * ncol;
    int nslab = 1;
    while (blocks1 * nslab < 152L * 8 && ctx->Nz / (nslab * 2) >= 8) nslab *= 2;
    p.zlen = (ctx->Nz + nslab - 1) / nslab;
    p.nslab = nslab;
    const int maxz = 65535 / nslab;
    for (int c0i = 0; c0i < ncol; c0i += maxz) {
        int nc = ncol - c0i < maxz ? ncol - c0i : maxz;
        StencilParams<T> q = p;
        q.x = x + (long)c0i * ldx;
        q.out = out + (long)c0i * ldo;
        if (q.z) q.z = z + (long)c0i * ldz;
        dim3 grid(tilesx, tilesy, nc * nslab), block(BX, BY);
        ProfScope ps(ctx, SGPU_KERNEL_STENCIL, st);
        k_stencil_orth<T, R, BX, BY><<<grid, block, 0, st>>>(q);
    }
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

template int launch_stencil<double>(sgpu_ctx *, int, double, double, double, const double *,
                                    const double *, long, double *, long, double, double,
                                    const double *, long, cudaStream_t);
template int launch_stencil<float>(sgpu_ctx *, int, double, double, double, const float *,
                                   const float *, long, float *, long, double, double,
                                   const float *, long, cudaStream_t);

}  // namespace sgpu
