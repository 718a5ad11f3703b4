// Atomic forces after the SCF: the finite-difference gradient of grid blocks, the nonlocal
// force from the projections of the orbitals and of their gradients, and the removal of the
// mean force. The local (pseudocharge) and core-correction forces live in setup.cu beside the
// pseudocharge code they share.
//
// Restates, for orthogonal periodic cells at the Gamma point:
//   Gradient_vectors_dir              src/gradVecRoutines.c:33 (D1 stencil, radius FDn)
//   Calculate_nonlocal_forces_linear  src/forces.c:750
//   Compute_Integral_psi_Chi          src/forces.c:849
//   Compute_Integral_Chi_Dpsi         src/forces.c:890
//   Compute_force_nloc_by_integrals   src/forces.c:926
//   Symmetrize_forces                 src/forces.c:1399
#include <vector>

#include "sgpu_internal.h"

namespace sgpu {
namespace {

struct D1Row {
    double w[kMaxFDn + 1];
};

// out = D1 x along one direction with periodic wrap: one thread per grid point and column
__global__ void __launch_bounds__(256) k_gradient(const double *__restrict__ x, long ldx,
                                                  double *__restrict__ out, long ldo, int Nx,
                                                  int Ny, int Nz, int dir, int FDn, D1Row c)
{
    const long Nd = (long)Nx * Ny * Nz;
    const int col = blockIdx.y;
    const double *xc = x + (long)col * ldx;
    double *oc = out + (long)col * ldo;
    for (long p = (long)blockIdx.x * blockDim.x + threadIdx.x; p < Nd;
         p += (long)gridDim.x * blockDim.x) {
        const int i = (int)(p % Nx), j = (int)((p / Nx) % Ny), k = (int)(p / ((long)Nx * Ny));
        const int n = dir == 0 ? Nx : dir == 1 ? Ny : Nz;
        const int q = dir == 0 ? i : dir == 1 ? j : k;
        const long stride = dir == 0 ? 1 : dir == 1 ? Nx : (long)Nx * Ny;
        const long base = p - (long)q * stride;
        double s = 0.0;
        for (int r = 1; r <= FDn; r++) {
            int qp = q + r, qm = q - r;
            qp -= qp >= n ? n : 0;  // r <= FDn < n: at most one wrap
            qm += qm < 0 ? n : 0;
            s += (xc[base + (long)qp * stride] - xc[base + (long)qm * stride]) * c.w[r];
        }
        oc[p] = s;
    }
}

// F[atom, d] -= 2 occfac sum_n occ[n] sum_{rows j of atom} alpha[j, n] beta_d[j, n]
// (alpha carries dV Gamma_j, beta_d the plain <Chi_j, d psi_n / dx_d>): one block per atom
__global__ void __launch_bounds__(256) k_nl_force_reduce(const int *__restrict__ ip_displ,
                                                         const double *__restrict__ alpha,
                                                         const double *__restrict__ beta,
                                                         long lda, long bstride, int ncol,
                                                         const double *__restrict__ occ,
                                                         double fac, double *__restrict__ F)
{
    __shared__ double red[3][8];
    const int atom = blockIdx.x;
    const int r0 = ip_displ[atom], nr = ip_displ[atom + 1] - r0;
    double s[3] = {0.0, 0.0, 0.0};
    for (int e = threadIdx.x; e < nr * ncol; e += blockDim.x) {
        const int row = r0 + e / ncol, n = e % ncol;
        const double a = alpha[(long)row * lda + n] * occ[n];
#pragma unroll
        for (int d = 0; d < 3; d++) s[d] += a * beta[d * bstride + (long)row * lda + n];
    }
#pragma unroll
    for (int d = 0; d < 3; d++) {
        double v = s[d];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) red[d][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[threadIdx.x][w];
        F[3 * atom + threadIdx.x] = -fac * t;
    }
}

__global__ void k_fill(double *x, long n, double v)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x)
        x[i] = v;
}

}  // namespace

int launch_gradient(sgpu_ctx *ctx, int ncol, const double *x, long ldx, double *out, long ldo,
                    int dir, const double *w, cudaStream_t st)
{
    if (ncol <= 0) return SGPU_OK;
    if (dir < 0 || dir > 2) {
        set_error("gradient: direction must be 0, 1 or 2");
        return SGPU_ERR_ARG;
    }
    const int n = dir == 0 ? ctx->Nx : dir == 1 ? ctx->Ny : ctx->Nz;
    if (n <= ctx->FDn) {
        set_error("gradient: the grid must have more than FDn points in each direction");
        return SGPU_ERR_ARG;
    }
    D1Row c{};
    for (int r = 0; r <= ctx->FDn; r++) c.w[r] = w[r];
    const long blocks = std::min<long>((ctx->Nd + 255) / 256, 2048);
    for (int c0 = 0; c0 < ncol; c0 += 65535) {
        const int nc = std::min(65535, ncol - c0);
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        k_gradient<<<dim3((unsigned)blocks, nc), 256, 0, st>>>(x + (long)c0 * ldx, ldx,
                                                               out + (long)c0 * ldo, ldo, ctx->Nx,
                                                               ctx->Ny, ctx->Nz, dir, ctx->FDn, c);
    }
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

}  // namespace sgpu

using namespace sgpu;

extern "C" {

int sgpu_Calculate_nonlocal_forces(sgpu_ctx *ctx, int ncol, const double *X, int ldi,
                                   const double *occ, double occfac, const double *cell,
                                   double *forces)
{
    if (!ctx || ncol <= 0 || !X || ldi < ctx->Nd || !occ || !cell || !forces) {
        set_error("sgpu_Calculate_nonlocal_forces: bad arguments");
        return SGPU_ERR_ARG;
    }
    if (!ctx->has_nl) {
        set_error("sgpu_Calculate_nonlocal_forces: no projectors (sgpu_set_nonlocal or "
                  "sgpu_CalculateNonlocalProjectors first)");
        return SGPU_ERR_STATE;
    }
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const Nonlocal &nl = ctx->nl;
    const long Nd = ctx->Nd;
    const long lda = nonlocal_alpha_ld(ncol, (int)sizeof(double));
    const long asz = (long)nl.ntot * lda;
    const bool dev_x = is_device_ptr(X);
    const double h[3] = {cell[0] / ctx->Nx, cell[1] / ctx->Ny, cell[2] / ctx->Nz};
    // alpha (4 blocks: psi, d psi/dx, dy, dz), gradient block, occupations, ones, forces, and a
    // device copy of X when it is in host memory
    const size_t n = 4 * asz + (size_t)Nd * ncol + ncol + nl.ntot + 3 * (size_t)nl.natom +
                     (dev_x ? 0 : (size_t)Nd * ncol);
    double *buf = nullptr;
    SGPU_CUDA_TRY(cudaMallocAsync(&buf, sizeof(double) * n, st));
    double *alpha = buf, *dX = alpha + 4 * asz, *docc = dX + (size_t)Nd * ncol,
           *ones = docc + ncol, *dF = ones + nl.ntot, *xs = dF + 3 * nl.natom;
    const double *xd = X;
    long ldx = ldi;
    int rc = SGPU_OK;
    do {
        if (!dev_x) {
            if (cudaMemcpy2DAsync(xs, sizeof(double) * Nd, X, sizeof(double) * ldi,
                                  sizeof(double) * Nd, ncol, cudaMemcpyHostToDevice,
                                  st) != cudaSuccess) {
                rc = SGPU_ERR_CUDA; break;
            }
            xd = xs;
            ldx = Nd;
        }
        if (cudaMemsetAsync(alpha, 0, sizeof(double) * 4 * asz, st) != cudaSuccess ||
            cudaMemcpyAsync(docc, occ, sizeof(double) * ncol, cudaMemcpyDefault, st) != cudaSuccess) {
            rc = SGPU_ERR_CUDA; break;
        }
        k_fill<<<64, 256, 0, st>>>(ones, nl.ntot, 1.0);
        // alpha_J = dV Gamma Chi_J^T psi (Compute_Integral_psi_Chi, Gamma folded in here)
        if ((rc = launch_nonlocal_project<double>(ctx, ncol, xd, ldx, alpha, lda, st)) != SGPU_OK)
            break;
        const double *cc[3] = {ctx->cx, ctx->cy, ctx->cz};
        for (int d = 0; d < 3 && rc == SGPU_OK; d++) {
            double w[kMaxFDn + 1] = {0.0};
            for (int r = 1; r <= ctx->FDn; r++) w[r] = cc[d][r] * h[d] * r * 0.5;
            rc = launch_gradient(ctx, ncol, xd, ldx, dX, Nd, d, w, st);
            // beta_d = Chi^T d psi / dx_d (Compute_Integral_Chi_Dpsi)
            if (rc == SGPU_OK)
                rc = launch_nonlocal_project_plain(ctx, ncol, dX, Nd, alpha + (d + 1) * asz, lda,
                                                   ones, st);
        }
        if (rc != SGPU_OK) break;
        {
            ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
            k_nl_force_reduce<<<nl.natom, 256, 0, st>>>(nl.ip_displ, alpha, alpha + asz, lda,
                                                        asz, ncol, docc, 2.0 * occfac, dF);
        }
        if (cudaGetLastError() != cudaSuccess) { rc = SGPU_ERR_CUDA; break; }
        std::vector<double> f(3 * nl.natom);
        if (cudaMemcpyAsync(f.data(), dF, sizeof(double) * f.size(), cudaMemcpyDeviceToHost,
                            st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            rc = SGPU_ERR_CUDA; break;
        }
        for (size_t i = 0; i < f.size(); i++) forces[i] += f[i];
    } while (0);
    cudaFreeAsync(buf, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == SGPU_OK) rc = SGPU_ERR_CUDA;
    if (rc == SGPU_ERR_CUDA) set_error("sgpu_Calculate_nonlocal_forces: CUDA error");
    return rc;
}

int sgpu_Gradient_vectors_dir(sgpu_ctx *ctx, int ncol, const double *cell, const double *x,
                              int ldi, double *Dx, int ldo, int dir)
{
    if (!ctx || ncol < 0 || !cell || !x || !Dx || ldi < ctx->Nd || ldo < ctx->Nd || dir < 0 ||
        dir > 2) {
        set_error("sgpu_Gradient_vectors_dir: bad arguments");
        return SGPU_ERR_ARG;
    }
    if (ncol == 0) return SGPU_OK;
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const long Nd = ctx->Nd;
    const bool dx_ = is_device_ptr(x), dy_ = is_device_ptr(Dx);
    double *buf = nullptr;
    const size_t n = (dx_ ? 0 : (size_t)Nd * ncol) + (dy_ ? 0 : (size_t)Nd * ncol);
    if (n) SGPU_CUDA_TRY(cudaMallocAsync(&buf, sizeof(double) * n, st));
    const double *xd = x;
    double *yd = Dx;
    long lx = ldi, ly = ldo;
    int rc = SGPU_OK;
    do {
        double *p = buf;
        if (!dx_) {
            if (cudaMemcpy2DAsync(p, sizeof(double) * Nd, x, sizeof(double) * ldi,
                                  sizeof(double) * Nd, ncol, cudaMemcpyHostToDevice,
                                  st) != cudaSuccess) {
                rc = SGPU_ERR_CUDA; break;
            }
            xd = p; lx = Nd; p += (size_t)Nd * ncol;
        }
        if (!dy_) { yd = p; ly = Nd; }
        const double *cc = dir == 0 ? ctx->cx : dir == 1 ? ctx->cy : ctx->cz;
        const double h = cell[dir] / (dir == 0 ? ctx->Nx : dir == 1 ? ctx->Ny : ctx->Nz);
        double w[kMaxFDn + 1] = {0.0};
        for (int r = 1; r <= ctx->FDn; r++) w[r] = cc[r] * h * r * 0.5;
        if ((rc = launch_gradient(ctx, ncol, xd, lx, yd, ly, dir, w, st)) != SGPU_OK) break;
        if (!dy_ && cudaMemcpy2DAsync(Dx, sizeof(double) * ldo, yd, sizeof(double) * Nd,
                                      sizeof(double) * Nd, ncol, cudaMemcpyDeviceToHost,
                                      st) != cudaSuccess) {
            rc = SGPU_ERR_CUDA; break;
        }
    } while (0);
    if (buf) cudaFreeAsync(buf, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == SGPU_OK) rc = SGPU_ERR_CUDA;
    if (rc == SGPU_ERR_CUDA) set_error("sgpu_Gradient_vectors_dir: CUDA error");
    return rc;
}

int sgpu_Symmetrize_forces(int n_atom, double *forces)
{
    if (n_atom <= 0 || !forces) {
        set_error("sgpu_Symmetrize_forces: bad arguments");
        return SGPU_ERR_ARG;
    }
    double m[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < n_atom; i++)
        for (int d = 0; d < 3; d++) m[d] += forces[3 * i + d];
    for (int d = 0; d < 3; d++) m[d] /= n_atom;
    for (int i = 0; i < n_atom; i++)
        for (int d = 0; d < 3; d++) forces[3 * i + d] -= m[d];
    return SGPU_OK;
}

}  // extern "C"
