// SCF-side device operations in FP64: reductions, electron density, LDA (PW92) exchange-
// correlation, the AAR linear solver (Poisson and Kerker), periodic-Pulay density mixing.
//
// Reference functions restated here (one process, orthogonal periodic cell):
//   CalculateDensity_psi       src/electronDensity.c:104-205
//   slater / pw / add_rho_core src/exchangeCorrelation.c:459, :475, :1254; Calculate_Exc :429
//   AAR                        src/linearSolver.c:37-165
//   AndersonExtrapolation etc. src/mixing.c:48-140 (dgelsd on the m x m normal equations)
//   Jacobi_preconditioner      src/electrostatics.c:1682-1709
//   Calculate_elecstPotential  src/electrostatics.c:1593-1680 (RHS 4*pi*(b + rho), mean shift)
//   Mixing_periodic_pulay      src/mixing.c:213-455, Kerker_precond :462-528
//   Evaluate_scf_error         src/electronicGroundState.c:1160-1195
// The grid-sized work runs on the device; only m x m Anderson systems (m = history length)
// and scalars cross to the host.
#include <algorithm>
#include <cmath>
#include <vector>

#include "sgpu_internal.h"

namespace sgpu {
namespace {

constexpr int kRedBlocks = 152 * 4;
constexpr int kMaxHist = 16;

__global__ void k_dot_partial(const double *__restrict__ a, const double *__restrict__ b, long n,
                              double *__restrict__ part)
{
    double s = 0.0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x)
        s += a[i] * (b ? b[i] : 1.0);
    __shared__ double sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_sum_partials(const double *__restrict__ part, int np, double *__restrict__ out)
{
    __shared__ double sh[256];
    double s = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

inline int egrid(long n)
{
    long g = (n + 255) / 256;
    return (int)std::max<long>(1, std::min<long>(g, 152L * 16));
}

// rho[i] = sum_n w[n] * psi[i + n*ld]^2   (w[n] = occfac * g_n / dV)
template <typename T>
__global__ void k_density(const T *__restrict__ psi, long ld, int ncol,
                          const double *__restrict__ w, double *__restrict__ rho, long Nd)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < Nd;
         i += (long)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int n = 0; n < ncol; n++) {
            const double v = (double)psi[i + (long)n * ld];
            s += w[n] * v * v;
        }
        rho[i] = s;
    }
}

// complex columns (re, im interleaved): rho[i] (+)= sum_n w_n |psi[i, n]|^2
template <typename CT>
__global__ void k_density_z(const CT *__restrict__ psi, long ld, int ncol,
                            const double *__restrict__ w, double *__restrict__ rho, long Nd,
                            int accumulate)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < Nd;
         i += (long)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int n = 0; n < ncol; n++) {
            const CT v = psi[i + (long)n * ld];
            const double re = (double)v.x, im = (double)v.y;
            s += w[n] * (re * re + im * im);
        }
        rho[i] = accumulate ? rho[i] + s : s;
    }
}

// LDA: Slater exchange + Perdew-Wang 92 correlation on rho + rho_core (clamped at rhotol).
// vxc = vx + vc, exc = ex + ec (energy per particle). Constants are the published values of
// the functional (J. P. Perdew and Y. Wang, PRB 45, 13244 (1992)).
__global__ void k_lda_pw(const double *__restrict__ rho, const double *__restrict__ rho_core,
                         double rhotol, double *__restrict__ vxc, double *__restrict__ exc,
                         long n)
{
    const double C2 = 0.738558766382022;    // 3/4 (3/pi)^(1/3)
    const double C3 = 0.9847450218426965;   // (3/pi)^(1/3)
    const double C31 = 0.6203504908993999;  // (3/(4 pi))^(1/3)
    const double A = 0.031091, alpha1 = 0.21370;
    const double beta1 = 7.5957, beta2 = 3.5876, beta3 = 1.6382, beta4 = 0.49294;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        double r = rho[i] + (rho_core ? rho_core[i] : 0.0);
        if (r < rhotol) r = rhotol;
        const double rc = cbrt(r);
        const double ex = -C2 * rc, vx = -C3 * rc;
        const double rs = C31 / rc;
        const double rsq = sqrt(rs);
        const double den = 2.0 * A * (beta1 * rsq + beta2 * rs + beta3 * rs * rsq + beta4 * rs * rs);
        const double G1 = log(1.0 + 1.0 / den);
        const double ec = -2.0 * A * (1.0 + alpha1 * rs) * G1;
        const double dden = A * (beta1 / rsq + 2.0 * beta2 + 3.0 * beta3 * rsq + 4.0 * beta4 * rs);
        const double vc = ec - (rs / 3.0) * (-2.0 * A * alpha1 * G1 +
                                              (2.0 * A * (1.0 + alpha1 * rs) * dden) / (den * (den + 1.0)));
        vxc[i] = vx + vc;
        exc[i] = ex + ec;
    }
}

// PW92 correlation energy per particle of one parameter set (unpolarised, fully polarised
// or the spin stiffness), G(rs) = -2A (1 + a1 rs) ln(1 + 1 / (2A (b1 rs^1/2 + b2 rs +
// b3 rs^3/2 + b4 rs^2))), and its rs derivative
__device__ __forceinline__ void pw92_g(double rs, double rsq, double A, double a1, double b1,
                                       double b2, double b3, double b4, double *g, double *dg)
{
    const double q1 = 2.0 * A * (b1 * rsq + b2 * rs + b3 * rs * rsq + b4 * rs * rs);
    const double dq1 = A * (b1 / rsq + 2.0 * b2 + 3.0 * b3 * rsq + 4.0 * b4 * rs);
    const double lg = log(1.0 + 1.0 / q1);
    const double q0 = -2.0 * A * (1.0 + a1 * rs);
    *g = q0 * lg;
    *dg = -2.0 * A * a1 * lg - q0 * dq1 / (q1 * (q1 + 1.0));
}

// LSDA: spin-polarised Slater exchange + PW92 correlation (J. P. Perdew and Y. Wang, PRB 45,
// 13244 (1992), eqs. 8-10 and table I) on the spin densities (up, dn) with half the model
// core density added to each and each clamped at rhotol; the total is their sum. The spin
// interpolation f(zeta) takes zeta scaled by 1 - 1e-6, which keeps it finite at full
// polarisation, as the reference's pw_spin does. Outputs Vxc_up, Vxc_dn and
// exc = ex + ec per particle of the total density.
__global__ void k_lsda_pw(const double *__restrict__ up_in, const double *__restrict__ dn_in,
                          const double *__restrict__ rho_core, double rhotol,
                          double *__restrict__ vxc_up, double *__restrict__ vxc_dn,
                          double *__restrict__ exc, long n)
{
    const double kx = 0.9305257363491000;     // (3/4) (6/pi)^(1/3): ex_s = -kx rho_s^(1/3)
    const double C31 = 0.6203504908993999;    // (3/(4 pi))^(1/3)
    const double fpp0_inv = 1.0 / 1.709921;   // 1 / f''(0)
    const double fden = 1.0 / (2.0 * 1.2599210498948732 - 2.0);  // 1 / (2^(4/3) - 2)
    const double az = 1.0 - 1.0e-6;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        const double hc = rho_core ? 0.5 * rho_core[i] : 0.0;
        double ru = up_in[i] + hc, rd = dn_in[i] + hc;
        if (ru < rhotol) ru = rhotol;
        if (rd < rhotol) rd = rhotol;
        const double r = ru + rd;
        const double cu = cbrt(ru), cd = cbrt(rd);
        // exchange: E_x = sum_s -kx rho_s^(4/3)
        const double exu = -kx * cu, exd = -kx * cd;
        const double ex = (exu * ru + exd * rd) / r;
        const double vxu = (4.0 / 3.0) * exu, vxd = (4.0 / 3.0) * exd;
        // correlation
        const double rs = C31 / cbrt(r);
        const double rsq = sqrt(rs);
        double e0, de0, e1, de1, am, dam;   // am = -alpha_c
        pw92_g(rs, rsq, 0.031091, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294, &e0, &de0);
        pw92_g(rs, rsq, 0.015545, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517, &e1, &de1);
        pw92_g(rs, rsq, 0.016887, 0.11125, 10.357, 3.6231, 0.88026, 0.49671, &am, &dam);
        const double z = (ru - rd) / r;
        const double zp = 1.0 + az * z, zm = 1.0 - az * z;
        const double czp = cbrt(zp), czm = cbrt(zm);
        const double f = (zp * czp + zm * czm - 2.0) * fden;
        const double df = (4.0 / 3.0) * az * (czp - czm) * fden;
        const double z3 = z * z * z, z4 = z3 * z;
        // ec = e0 - am f (1 - z^4) / f''(0) + (e1 - e0) f z^4
        const double ec = e0 - am * fpp0_inv * f * (1.0 - z4) + (e1 - e0) * f * z4;
        const double dec_drs = de0 - dam * fpp0_inv * f * (1.0 - z4) + (de1 - de0) * f * z4;
        const double dec_dz = -am * fpp0_inv * (df * (1.0 - z4) - 4.0 * z3 * f) +
                              (e1 - e0) * (df * z4 + 4.0 * z3 * f);
        const double base = ec - (rs / 3.0) * dec_drs - z * dec_dz;
        vxc_up[i] = vxu + base + dec_dz;
        vxc_dn[i] = vxd + base - dec_dz;
        exc[i] = ex + ec;
    }
}

// AAR bookkeeping for one iteration (after the residual r is known):
//   f = minv * r; if hist >= 0: X[:,hist] = x - x_old, F[:,hist] = f - f_old;
//   x_old = x; f_old = f; if richardson: x = x_old + omega * f
__global__ void k_aar_step(long n, double minv, double omega, int hist, int richardson,
                           double *__restrict__ x, const double *__restrict__ r,
                           double *__restrict__ f, double *__restrict__ x_old,
                           double *__restrict__ f_old, double *__restrict__ X,
                           double *__restrict__ F)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        const double fi = minv * r[i];
        const double xi = x[i];
        if (hist >= 0) {
            X[(long)hist * n + i] = xi - x_old[i];
            F[(long)hist * n + i] = fi - f_old[i];
        }
        x_old[i] = xi;
        f_old[i] = fi;
        f[i] = fi;
        if (richardson) x[i] = xi + omega * fi;
    }
}

struct Gam {
    double g[kMaxHist];
};

// x_wavg = x_k - X*Gamma, f_wavg = f_k - F*Gamma; out = x_wavg + beta * f_wavg (AAR), or the
// two averages separately (mixing, when xw / fw are given)
__global__ void k_anderson(long n, int m, Gam gam, double beta, const double *__restrict__ xk,
                           const double *__restrict__ fk, const double *__restrict__ X,
                           const double *__restrict__ F, double *__restrict__ out,
                           double *__restrict__ xw, double *__restrict__ fw)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        double xa = xk[i], fa = fk[i];
        for (int j = 0; j < m; j++) {
            xa -= gam.g[j] * X[(long)j * n + i];
            fa -= gam.g[j] * F[(long)j * n + i];
        }
        if (out) out[i] = xa + beta * fa;
        if (xw) xw[i] = xa;
        if (fw) fw[i] = fa;
    }
}

__global__ void k_axpby(long n, double a, const double *__restrict__ x, double b,
                        const double *__restrict__ y, double *__restrict__ z)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x)
        z[i] = a * x[i] + (y ? b * y[i] : 0.0);
}

__global__ void k_shift(long n, double *__restrict__ x, const double *__restrict__ sum,
                        double scale)
{
    const double s = *sum * scale;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x)
        x[i] -= s;
}

// rhs = 4 pi (b + rho)
__global__ void k_poisson_rhs(long n, const double *__restrict__ b,
                              const double *__restrict__ rho, double *__restrict__ rhs)
{
    const double fpi = 4.0 * M_PI;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x)
        rhs[i] = fpi * (b[i] + rho[i]);
}

// x = max(x, 0); flag set if any was negative
// x += (*a - *b) * scale: the shift that gives x the integral *a in place of *b
__global__ void k_shift_to(long n, double *__restrict__ x, const double *__restrict__ a,
                           const double *__restrict__ b, double scale)
{
    const double s = (*a - *b) * scale;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x)
        x[i] += s;
}

__global__ void k_clamp_neg(long n, double *__restrict__ x, int *__restrict__ flag)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        if (x[i] < 0.0) {
            x[i] = 0.0;
            *flag = 1;
        }
    }
}

__global__ void k_scale_by(long n, double *__restrict__ x, const double *__restrict__ sum,
                           double num)
{
    const double s = num / *sum;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x)
        x[i] *= s;
}

// sbuf[0] += out^2, sbuf[1] += (out - in)^2 partials
__global__ void k_err_partial(const double *__restrict__ out, const double *__restrict__ in,
                              long n, double *__restrict__ part)
{
    double s0 = 0.0, s1 = 0.0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        const double t = out[i] - in[i];
        s0 += out[i] * out[i];
        s1 += t * t;
    }
    __shared__ double sh0[256], sh1[256];
    sh0[threadIdx.x] = s0;
    sh1[threadIdx.x] = s1;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            sh0[threadIdx.x] += sh0[threadIdx.x + o];
            sh1[threadIdx.x] += sh1[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = sh0[0];
        part[2 * blockIdx.x + 1] = sh1[0];
    }
}

// Symmetric positive semi-definite pseudo-inverse solve of A g = b (m x m), restating the
// minimum-norm least-squares solution of LAPACK dgelsd with rcond = machine epsilon: singular
// values below eps * s_max are dropped. Cyclic Jacobi eigen-decomposition (A = V S Vᵀ).
void spd_pinv_solve(int m, const double *Ain, const double *b, double *g)
{
    std::vector<double> A(Ain, Ain + (size_t)m * m), V((size_t)m * m, 0.0);
    for (int i = 0; i < m; i++) V[(size_t)i * m + i] = 1.0;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0;
        for (int p = 0; p < m; p++)
            for (int q = p + 1; q < m; q++) off += A[(size_t)q * m + p] * A[(size_t)q * m + p];
        if (off < 1e-300) break;
        for (int p = 0; p < m; p++) {
            for (int q = p + 1; q < m; q++) {
                const double apq = A[(size_t)q * m + p];
                if (apq == 0.0) continue;
                const double app = A[(size_t)p * m + p], aqq = A[(size_t)q * m + q];
                const double theta = (aqq - app) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) /
                                 (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < m; k++) {  // columns p, q
                    const double akp = A[(size_t)p * m + k], akq = A[(size_t)q * m + k];
                    A[(size_t)p * m + k] = c * akp - s * akq;
                    A[(size_t)q * m + k] = s * akp + c * akq;
                }
                for (int k = 0; k < m; k++) {  // rows p, q
                    const double apk = A[(size_t)k * m + p], aqk = A[(size_t)k * m + q];
                    A[(size_t)k * m + p] = c * apk - s * aqk;
                    A[(size_t)k * m + q] = s * apk + c * aqk;
                }
                for (int k = 0; k < m; k++) {
                    const double vkp = V[(size_t)p * m + k], vkq = V[(size_t)q * m + k];
                    V[(size_t)p * m + k] = c * vkp - s * vkq;
                    V[(size_t)q * m + k] = s * vkp + c * vkq;
                }
            }
        }
    }
    double smax = 0.0;
    for (int i = 0; i < m; i++) smax = std::max(smax, std::fabs(A[(size_t)i * m + i]));
    const double thr = 2.220446049250313e-16 * smax;
    for (int i = 0; i < m; i++) g[i] = 0.0;
    for (int k = 0; k < m; k++) {
        const double s = A[(size_t)k * m + k];
        if (std::fabs(s) <= thr || s == 0.0) continue;
        double vb = 0.0;
        for (int i = 0; i < m; i++) vb += V[(size_t)k * m + i] * b[i];
        for (int i = 0; i < m; i++) g[i] += V[(size_t)k * m + i] * vb / s;
    }
}

}  // namespace

int dot_dev(sgpu_ctx *ctx, const double *a, const double *b, long n, double *d_out,
            cudaStream_t st)
{
    double *part = nullptr;
    SGPU_TRY(ws_get(ctx, WS_RED, sizeof(double) * (kRedBlocks * 2 + 8), (void **)&part));
    k_dot_partial<<<kRedBlocks, 256, 0, st>>>(a, b, n, part);
    k_sum_partials<<<1, 256, 0, st>>>(part, kRedBlocks, d_out);
    ctx->launches += 2;
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

int dot_host(sgpu_ctx *ctx, const double *a, const double *b, long n, double *out,
             cudaStream_t st)
{
    double *part = nullptr;
    SGPU_TRY(ws_get(ctx, WS_RED, sizeof(double) * (kRedBlocks * 2 + 8), (void **)&part));
    double *res = part + kRedBlocks * 2;
    SGPU_TRY(dot_dev(ctx, a, b, n, res, st));
    SGPU_CUDA_TRY(cudaMemcpyAsync(out, res, sizeof(double), cudaMemcpyDeviceToHost, st));
    SGPU_CUDA_TRY(cudaStreamSynchronize(st));
    return SGPU_OK;
}

template <typename T>
int density_dev(sgpu_ctx *ctx, const T *psi, long ld, int ncol, const double *w_dev,
                double *rho, cudaStream_t st)
{
    ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
    k_density<T><<<egrid(ctx->Nd), 256, 0, st>>>(psi, ld, ncol, w_dev, rho, ctx->Nd);
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}
template int density_dev<double>(sgpu_ctx *, const double *, long, int, const double *,
                                 double *, cudaStream_t);
template int density_dev<float>(sgpu_ctx *, const float *, long, int, const double *, double *,
                                cudaStream_t);

template <typename CT>
int density_z_dev(sgpu_ctx *ctx, const CT *psi, long ld, int ncol, const double *w_dev,
                  double *rho, bool accumulate, cudaStream_t st)
{
    ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
    k_density_z<CT><<<egrid(ctx->Nd), 256, 0, st>>>(psi, ld, ncol, w_dev, rho, ctx->Nd,
                                                    accumulate ? 1 : 0);
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}
template int density_z_dev<double2>(sgpu_ctx *, const double2 *, long, int, const double *,
                                    double *, bool, cudaStream_t);
template int density_z_dev<float2>(sgpu_ctx *, const float2 *, long, int, const double *,
                                   double *, bool, cudaStream_t);

int lda_pw_dev(sgpu_ctx *ctx, const double *rho, const double *rho_core, double rhotol,
               double *vxc, double *exc, cudaStream_t st)
{
    ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
    k_lda_pw<<<egrid(ctx->Nd), 256, 0, st>>>(rho, rho_core, rhotol, vxc, exc, ctx->Nd);
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

int lsda_pw_dev(sgpu_ctx *ctx, const double *up, const double *dn, const double *rho_core,
                double rhotol, double *vxc_up, double *vxc_dn, double *exc, cudaStream_t st)
{
    ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
    k_lsda_pw<<<egrid(ctx->Nd), 256, 0, st>>>(up, dn, rho_core, rhotol, vxc_up, vxc_dn, exc,
                                              ctx->Nd);
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

int axpby_dev(sgpu_ctx *ctx, long n, double a, const double *x, double b, const double *y,
              double *z, cudaStream_t st)
{
    k_axpby<<<egrid(n), 256, 0, st>>>(n, a, x, b, y, z);
    ctx->launches++;
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

int poisson_rhs_dev(sgpu_ctx *ctx, const double *b, const double *rho, double *rhs,
                    cudaStream_t st)
{
    k_poisson_rhs<<<egrid(ctx->Nd), 256, 0, st>>>(ctx->Nd, b, rho, rhs);
    ctx->launches++;
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

// subtract the mean (periodic Poisson solution / Kerker with zero screening)
int remove_mean_dev(sgpu_ctx *ctx, double *x, cudaStream_t st)
{
    double *part = nullptr;
    SGPU_TRY(ws_get(ctx, WS_RED, sizeof(double) * (kRedBlocks * 2 + 8), (void **)&part));
    double *res = part + kRedBlocks * 2 + 1;
    SGPU_TRY(dot_dev(ctx, x, nullptr, ctx->Nd, res, st));
    k_shift<<<egrid(ctx->Nd), 256, 0, st>>>(ctx->Nd, x, res, 1.0 / (double)ctx->Nd);
    ctx->launches++;
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

int scf_error_dev(sgpu_ctx *ctx, const double *out, const double *in, double *err,
                  cudaStream_t st, long n)
{
    double *part = nullptr;
    SGPU_TRY(ws_get(ctx, WS_RED, sizeof(double) * (kRedBlocks * 2 + 8), (void **)&part));
    k_err_partial<<<kRedBlocks, 256, 0, st>>>(out, in, n > 0 ? n : ctx->Nd, part);
    ctx->launches++;
    std::vector<double> h(2 * kRedBlocks);
    SGPU_CUDA_TRY(cudaMemcpyAsync(h.data(), part, sizeof(double) * 2 * kRedBlocks,
                                  cudaMemcpyDeviceToHost, st));
    SGPU_CUDA_TRY(cudaStreamSynchronize(st));
    double s0 = 0.0, s1 = 0.0;
    for (int i = 0; i < kRedBlocks; i++) { s0 += h[2 * i]; s1 += h[2 * i + 1]; }
    *err = std::sqrt(s1 / s0);
    return SGPU_OK;
}

// Anderson coefficients: Gamma = pinv(Fᵀ F) Fᵀ f (m x m normal equations on the host)
static int anderson_gamma(sgpu_ctx *ctx, long n, int m, const double *F, const double *f,
                          Gam *gam, cudaStream_t st)
{
    double *part = nullptr;
    SGPU_TRY(ws_get(ctx, WS_RED, sizeof(double) * (kRedBlocks * 2 + 8 + kMaxHist * (kMaxHist + 1)),
                    (void **)&part));
    double *ftf = part + kRedBlocks * 2 + 8;
    double *ftb = ftf + kMaxHist * kMaxHist;
    // Fᵀ F and Fᵀ f with deterministic device reductions
    for (int i = 0; i < m; i++) {
        for (int j = i; j < m; j++) SGPU_TRY(dot_dev(ctx, F + (long)i * n, F + (long)j * n, n, ftf + i * m + j, st));
        SGPU_TRY(dot_dev(ctx, F + (long)i * n, f, n, ftb + i, st));
    }
    double h[kMaxHist * (kMaxHist + 1)];
    SGPU_CUDA_TRY(cudaMemcpyAsync(h, ftf, sizeof(double) * kMaxHist * (kMaxHist + 1),
                                  cudaMemcpyDeviceToHost, st));
    SGPU_CUDA_TRY(cudaStreamSynchronize(st));
    double A[kMaxHist * kMaxHist], b[kMaxHist];
    for (int i = 0; i < m; i++) {
        for (int j = i; j < m; j++) A[(size_t)j * m + i] = A[(size_t)i * m + j] = h[i * m + j];
        b[i] = h[kMaxHist * kMaxHist + i];
    }
    spd_pinv_solve(m, A, b, gam->g);
    return SGPU_OK;
}

// AAR for  b + (Lap + c) x = 0  with the Jacobi preconditioner, restating AAR
// (src/linearSolver.c:37-165) with poisson_residual and Jacobi_preconditioner. The residual
// norm is evaluated at Anderson steps only, as in the reference. Returns the iteration count.
int aar_dev(sgpu_ctx *ctx, double c, double *x, const double *b, double omega, double beta,
            int m, int p, double tol, int max_iter, int *iters, cudaStream_t st)
{
    if (m < 1 || m > kMaxHist || p < 1) {
        set_error("AAR: history length must be in [1, 16] and p >= 1");
        return SGPU_ERR_ARG;
    }
    const long N = ctx->Nd;
    double *w = nullptr;
    SGPU_TRY(ws_get(ctx, WS_POIS, sizeof(double) * (size_t)N * (4 + 2 * m), (void **)&w));
    double *r = w, *x_old = w + N, *f = w + 2 * N, *f_old = w + 3 * N;
    double *X = w + 4 * N, *F = w + (4 + m) * N;
    SGPU_CUDA_TRY(cudaMemsetAsync(X, 0, sizeof(double) * (size_t)N * 2 * m, st));
    SGPU_CUDA_TRY(cudaMemcpyAsync(x_old, x, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
    double bnorm2 = 0.0;
    SGPU_TRY(dot_host(ctx, b, b, N, &bnorm2, st));
    double minv = ctx->cx[0] + ctx->cy[0] + ctx->cz[0] + c;
    if (std::fabs(minv) < 1e-14) minv = 1.0;
    minv = -1.0 / minv;
    // r = b + (Lap + c) x
    SGPU_TRY(launch_stencil<double>(ctx, 1, 1.0, 0.0, c, nullptr, x, N, r, N, 1.0, 1.0, b, N, st));
    tol *= std::sqrt(bnorm2);
    double rnorm = tol + 1.0;
    int it = 0;
    while (rnorm > tol && it < max_iter) {
        const int hist = it > 0 ? (it - 1) % m : -1;
        const bool anderson = ((it + 1) % p == 0) && it > 0;
        k_aar_step<<<egrid(N), 256, 0, st>>>(N, minv, omega, hist, anderson ? 0 : 1, x, r, f,
                                             x_old, f_old, X, F);
        ctx->launches++;
        if (anderson) {
            Gam gam;
            SGPU_TRY(anderson_gamma(ctx, N, m, F, f, &gam, st));
            k_anderson<<<egrid(N), 256, 0, st>>>(N, m, gam, beta, x_old, f, X, F, x, nullptr,
                                                 nullptr);
            ctx->launches++;
            SGPU_TRY(launch_stencil<double>(ctx, 1, 1.0, 0.0, c, nullptr, x, N, r, N, 1.0, 1.0,
                                            b, N, st));
            double r2 = 0.0;
            SGPU_TRY(dot_host(ctx, r, r, N, &r2, st));
            rnorm = std::sqrt(r2);
        } else {
            SGPU_TRY(launch_stencil<double>(ctx, 1, 1.0, 0.0, c, nullptr, x, N, r, N, 1.0, 1.0,
                                            b, N, st));
        }
        it++;
    }
    SGPU_CUDA_TRY(cudaGetLastError());
    if (iters) *iters = it;
    if (rnorm > tol) {
        set_error("AAR: no convergence in " + std::to_string(max_iter) + " iterations");
        return SGPU_ERR_NOT_CONVERGED;
    }
    return SGPU_OK;
}

// phi: -Lap phi = 4 pi (b + rho), zero mean (Calculate_elecstPotential, periodic cell).
// phi holds the initial guess on entry.
int poisson_dev(sgpu_ctx *ctx, const double *rho, const double *b, double *phi, double tol,
                int max_iter, int *iters, cudaStream_t st)
{
    const long N = ctx->Nd;
    double *rhs = nullptr;
    SGPU_TRY(ws_get(ctx, WS_RHS, sizeof(double) * (size_t)N, (void **)&rhs));
    SGPU_TRY(poisson_rhs_dev(ctx, b, rho, rhs, st));
    int rc = aar_dev(ctx, 0.0, phi, rhs, 0.6, 0.6, 7, 6, tol, max_iter, iters, st);
    if (rc != SGPU_OK && rc != SGPU_ERR_NOT_CONVERGED) return rc;
    SGPU_TRY(remove_mean_dev(ctx, phi, st));
    return SGPU_OK;  // non-convergence is a warning in the reference (src/linearSolver.c)
}

// Kerker: Pf = a (L - kTF^2)^-1 (L - idiemac kTF^2) f, solved with AAR (src/mixing.c:462-528).
// Pf holds the initial guess on entry (the previous call's result, as in the reference).
int kerker_dev(sgpu_ctx *ctx, const double *f, double a, double kTF, double idiemac,
               double tol, double *Pf, cudaStream_t st)
{
    const long N = ctx->Nd;
    double *Lf = nullptr;
    SGPU_TRY(ws_get(ctx, WS_RHS, sizeof(double) * (size_t)N, (void **)&Lf));
    SGPU_TRY(launch_stencil<double>(ctx, 1, 1.0, 0.0, -kTF * kTF * idiemac, nullptr, f, N, Lf, N,
                                    1.0, 0.0, nullptr, 0, st));
    int rc = aar_dev(ctx, -kTF * kTF, Pf, Lf, 0.6, 0.6, 7, 6, tol, 1000, nullptr, st);
    if (rc != SGPU_OK && rc != SGPU_ERR_NOT_CONVERGED) return rc;
    if (std::fabs(kTF) < 1e-14) SGPU_TRY(remove_mean_dev(ctx, Pf, st));
    SGPU_TRY(axpby_dev(ctx, N, -a, Pf, 0.0, nullptr, Pf, st));
    return SGPU_OK;
}

// ---------------------------------------------------------------- Pulay mixing state

MixState::~MixState()
{
    if (buf) cudaFree(buf);
}

int mixing_init(sgpu_ctx *ctx, const MixParams &prm, const double *x0)
{
    if (prm.m < 1 || prm.m > kMaxHist) {
        set_error("mixing: history length must be in [1, 16]");
        return SGPU_ERR_ARG;
    }
    if (prm.nspden != 1 && prm.nspden != 2) {
        set_error("mixing: Nspden must be 1 or 2");
        return SGPU_ERR_ARG;
    }
    const long N = ctx->Nd * prm.nspden;  // length of the mixed vector
    MixState *ms = ctx->mix;
    if (!ms || ms->m != prm.m || ms->prm.nspden != prm.nspden) {
        delete ms;
        ms = new MixState();
        ctx->mix = ms;
        ms->m = prm.m;
        ms->prm.nspden = prm.nspden;
        if (cudaMalloc(&ms->buf, sizeof(double) * (size_t)N * (8 + 2 * prm.m)) != cudaSuccess) {
            set_error("mixing: device allocation failed");
            delete ms;
            ctx->mix = nullptr;
            return SGPU_ERR_NOMEM;
        }
    }
    ms->prm = prm;
    double *b = ms->buf;
    ms->x_k = b; ms->x_km1 = b + N; ms->f_k = b + 2 * N; ms->f_km1 = b + 3 * N;
    ms->Pf = b + 4 * N; ms->x_wavg = b + 5 * N; ms->f_wavg = b + 6 * N; ms->tmp = b + 7 * N;
    ms->R = b + 8 * N; ms->F = b + (8 + prm.m) * N;
    SGPU_CUDA_TRY(cudaMemsetAsync(ms->buf, 0, sizeof(double) * (size_t)N * (8 + 2 * prm.m),
                                  ctx->stream));
    SGPU_CUDA_TRY(cudaMemcpyAsync(ms->x_k, x0, sizeof(double) * N, cudaMemcpyDefault,
                                  ctx->stream));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

// One periodic-Pulay step of density mixing (Mixing_periodic_pulay, src/mixing.c:213-450):
// g (the output density of this SCF iteration; with collinear spin the vector [rho, magz]
// of 2 Nd values) is replaced in place by the next input x_{k+1}. With spin, the total density
// residual is preconditioned as without (Kerker or amix), the magnetization residual by
// amix_mag alone (MixingPrecondMag = 0), and each preconditioned part is shifted to keep the
// integral of its residual (src/mixing.c:376-385).
int mixing_step(sgpu_ctx *ctx, int iter_count, double *g, cudaStream_t st)
{
    MixState *ms = ctx->mix;
    if (!ms) {
        set_error("mixing: sgpu_mixing_init has not been called");
        return SGPU_ERR_STATE;
    }
    const MixParams &p = ms->prm;
    const long Nd = ctx->Nd;
    const long N = Nd * p.nspden;
    const int m = ms->m;
    const bool pulay = ((iter_count + 1) % p.pulay_freq == 0) && iter_count > 0;
    const double amix = pulay ? p.beta : p.omega;
    const double amix_mag = pulay ? p.beta_mag : p.omega_mag;
    if (iter_count > 0)
        SGPU_CUDA_TRY(cudaMemcpyAsync(ms->f_km1, ms->f_k, sizeof(double) * N,
                                      cudaMemcpyDeviceToDevice, st));
    SGPU_TRY(axpby_dev(ctx, N, 1.0, g, -1.0, ms->x_k, ms->f_k, st));
    if (iter_count > 0) {
        const int ih = (iter_count - 1) % m;
        if (p.restart && ih == 0 && m > 1) {  // keep only the newest difference
            SGPU_CUDA_TRY(cudaMemsetAsync(ms->R + N, 0, sizeof(double) * N * (m - 1), st));
            SGPU_CUDA_TRY(cudaMemsetAsync(ms->F + N, 0, sizeof(double) * N * (m - 1), st));
        }
        SGPU_TRY(axpby_dev(ctx, N, 1.0, ms->x_k, -1.0, ms->x_km1, ms->R + (long)ih * N, st));
        SGPU_TRY(axpby_dev(ctx, N, 1.0, ms->f_k, -1.0, ms->f_km1, ms->F + (long)ih * N, st));
    }
    if (pulay) {
        Gam gam;
        SGPU_TRY(anderson_gamma(ctx, N, m, ms->F, ms->f_k, &gam, st));
        k_anderson<<<egrid(N), 256, 0, st>>>(N, m, gam, 0.0, ms->x_k, ms->f_k, ms->R, ms->F,
                                             nullptr, ms->x_wavg, ms->f_wavg);
        ctx->launches++;
    } else {
        SGPU_CUDA_TRY(cudaMemcpyAsync(ms->x_wavg, ms->x_k, sizeof(double) * N,
                                      cudaMemcpyDeviceToDevice, st));
        SGPU_CUDA_TRY(cudaMemcpyAsync(ms->f_wavg, ms->f_k, sizeof(double) * N,
                                      cudaMemcpyDeviceToDevice, st));
    }
    if (p.kerker) {
        SGPU_TRY(kerker_dev(ctx, ms->f_wavg, amix, p.kTF, p.idiemac, p.precond_tol, ms->Pf, st));
    } else {
        SGPU_TRY(axpby_dev(ctx, Nd, amix, ms->f_wavg, 0.0, nullptr, ms->Pf, st));
    }
    int *flag = nullptr;
    double *part = nullptr;
    SGPU_TRY(ws_get(ctx, WS_RED, sizeof(double) * (kRedBlocks * 2 + 8 + kMaxHist * (kMaxHist + 1)),
                    (void **)&part));
    flag = reinterpret_cast<int *>(part + kRedBlocks * 2 + 4);
    double *sum = part + kRedBlocks * 2 + 2;
    if (p.nspden == 2) {
        SGPU_TRY(axpby_dev(ctx, Nd, amix_mag, ms->f_wavg + Nd, 0.0, nullptr, ms->Pf + Nd, st));
        // per component: Pf += (sum f_wavg - sum Pf) / Nd
        double *sums = nullptr;
        SGPU_TRY(ws_get(ctx, WS_ALPHA2, sizeof(double) * 8, (void **)&sums));
        for (int c = 0; c < 2; c++) {
            double *sf = sums + c * 2, *sp = sf + 1;
            SGPU_TRY(dot_dev(ctx, ms->f_wavg + c * Nd, nullptr, Nd, sf, st));
            SGPU_TRY(dot_dev(ctx, ms->Pf + c * Nd, nullptr, Nd, sp, st));
            k_shift_to<<<egrid(Nd), 256, 0, st>>>(Nd, ms->Pf + c * Nd, sf, sp, 1.0 / (double)Nd);
            ctx->launches++;
        }
    }
    // x_{k+1} = x_wavg + Pf, clamp negative densities, renormalise to the electron count
    SGPU_TRY(axpby_dev(ctx, N, 1.0, ms->x_wavg, 1.0, ms->Pf, g, st));
    SGPU_CUDA_TRY(cudaMemsetAsync(flag, 0, sizeof(int), st));
    k_clamp_neg<<<egrid(Nd), 256, 0, st>>>(Nd, g, flag);
    SGPU_TRY(dot_dev(ctx, g, nullptr, Nd, sum, st));
    // scale = -NegCharge / (dV * sum)
    k_scale_by<<<egrid(Nd), 256, 0, st>>>(Nd, g, sum, -p.neg_charge / ctx->dV);
    ctx->launches += 2;
    SGPU_CUDA_TRY(cudaMemcpyAsync(ms->x_km1, ms->x_k, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
    SGPU_CUDA_TRY(cudaMemcpyAsync(ms->x_k, g, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

}  // namespace sgpu
