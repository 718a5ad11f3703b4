// CheFSI SCF on the device, and the C ABI for the Rayleigh-Ritz and SCF-side rows.
//
// The driver restates the reference's single-point SCF for an orthogonal, periodic,
// Gamma-point, spin-unpolarised system with an LDA functional and density mixing:
//   scf / scf_loop               src/electronicGroundState.c:607-1155
//   eigSolve_CheFSI / CheFSI     src/eigenSolver.c:150-263 / :269-445
//   Chebyshevfilter_constants    src/eigenSolver.c:589-715 (Lanczos :1920-2129)
//   Calculate_occupation         src/occupation.c:43 (Fermi level by Brent's method, :291)
//   Calculate_Free_Energy        src/energy.c:41-200 (Eband :205, entropy :241, :296)
// Everything grid-sized stays on the device; per SCF iteration only the Ns eigenvalues, a few
// scalars (energy terms, SCF error) and the m x m Anderson systems come back to the host.
//
// Mixed precision (SGPU_PREC_FP32): while the SCF error is above fp64_switch_error the orbital
// block is FP32, the filter runs in FP32 and the projection / rotation products are
// FP32-accurate split products on the tensor cores (rr_tc.cu); the eigenproblem, Poisson, XC,
// mixing and all energy reductions stay FP64. Below the threshold (or once the FP32 error stalls) the block
// is widened to FP64 and the remaining iterations are either the plain FP64 path or, with
// graded_tail, an FP32 filter whose last degrees run in FP64 followed by an FP64
// Rayleigh-Ritz step (chebyshev_graded).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <functional>
#include <vector>

#include "sgpu_internal.h"

namespace sgpu {

__global__ void k_init_orbitals(double *X, long n, unsigned long long seed)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        // splitmix64 of (seed, index) -> uniform [-0.5, 0.5)
        unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(i + 1);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        X[i] = (double)(z >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    }
}

void init_orbitals(sgpu_ctx *ctx, double *X, long n, unsigned long long seed, int blocks,
                   cudaStream_t st)
{
    k_init_orbitals<<<blocks, 256, 0, st>>>(X, n, seed);
    ctx->launches++;
}

double smearing(double beta, double lam, double ef, int type)
{
    return type ? 0.5 * (1.0 - std::erf(beta * (lam - ef))) : 1.0 / (1.0 + std::exp(beta * (lam - ef)));
}

// Brent root finding for sum_n w_n f(lambda_n) = Nelectron (Numerical-Recipes style
// bracketing with inverse quadratic interpolation, as local_Calculate_FermiLevel does; w_n is
// occfac at the Gamma point and occfac * kptWts / Nkpts at k-points, src/occupation.c:445-466)
double fermi_level(const std::vector<double> &lam, const std::vector<double> &w, double nelec,
                   double beta, int type, double x1, double x2, double tol, int max_iter,
                   int *status)
{
    auto g = [&](double ef) {
        double s = 0.0;
        for (size_t i = 0; i < lam.size(); i++) s += w[i] * smearing(beta, lam[i], ef, type);
        return s - nelec;
    };
    double a = std::min(x1, x2), b = std::max(x1, x2), c = b, d = 0, e = 0;
    double fa = g(a), fb = g(b), fc;
    int ext = 0;
    while (fa * fb > 0.0 && ext++ < 10) {
        const double w = b - a;
        a -= w / 2.0;
        b += w / 2.0;
        c = b;
        fa = g(a);
        fb = g(b);
    }
    *status = (fa * fb > 0.0) ? 1 : 0;
    if (*status) return b;
    fc = fb;
    const double EPS = 1e-16;
    for (int it = 1; it <= max_iter; it++) {
        if ((fb > 0.0 && fc > 0.0) || (fb < 0.0 && fc < 0.0)) {
            c = a; fc = fa; e = d = b - a;
        }
        if (std::fabs(fc) < std::fabs(fb)) {
            a = b; b = c; c = a; fa = fb; fb = fc; fc = fa;
        }
        const double tol1 = 2.0 * EPS * std::fabs(b) + 0.5 * tol;
        const double xm = 0.5 * (c - b);
        if (std::fabs(xm) <= tol1 || std::fabs(fb) < EPS) return b;
        if (std::fabs(e) >= tol1 && std::fabs(fa) > std::fabs(fb)) {
            double p, q, r;
            const double s = fb / fa;
            if (a == c) {
                p = 2.0 * xm * s;
                q = 1.0 - s;
            } else {
                q = fa / fc;
                r = fb / fc;
                p = s * (2.0 * xm * q * (q - r) - (b - a) * (r - 1.0));
                q = (q - 1.0) * (r - 1.0) * (s - 1.0);
            }
            if (p > 0.0) q = -q;
            p = std::fabs(p);
            const double min1 = 3.0 * xm * q - std::fabs(tol1 * q), min2 = std::fabs(e * q);
            if (2.0 * p < std::min(min1, min2)) {
                e = d;
                d = p / q;
            } else {
                d = xm;
                e = d;
            }
        } else {
            d = xm;
            e = d;
        }
        a = b;
        fa = fb;
        b += (std::fabs(d) > tol1) ? d : (xm > 0 ? std::fabs(tol1) : -std::fabs(tol1));
        fb = g(b);
    }
    return b;
}

namespace {

// Extreme eigenvalues of the symmetric tridiagonal matrix (diag a[0..n-1], off b[0..n-2]) by
// Sturm-sequence bisection
void tridiag_extremes(int n, const double *a, const double *b, double *lo, double *hi)
{
    double gl = a[0], gu = a[0];
    for (int i = 0; i < n; i++) {
        const double r = (i > 0 ? std::fabs(b[i - 1]) : 0.0) + (i < n - 1 ? std::fabs(b[i]) : 0.0);
        gl = std::min(gl, a[i] - r);
        gu = std::max(gu, a[i] + r);
    }
    auto count_below = [&](double x) {  // eigenvalues < x
        int cnt = 0;
        double q = a[0] - x;
        if (q < 0) cnt++;
        for (int i = 1; i < n; i++) {
            if (q == 0.0) q = 1e-300;
            q = a[i] - x - b[i - 1] * b[i - 1] / q;
            if (q < 0) cnt++;
        }
        return cnt;
    };
    auto kth = [&](int k) {  // k-th smallest (0-based)
        double l = gl, u = gu;
        for (int it = 0; it < 200 && u - l > 1e-14 * std::max(1.0, std::fabs(u) + std::fabs(l)); it++) {
            const double mid = 0.5 * (l + u);
            if (count_below(mid) > k) u = mid; else l = mid;
        }
        return 0.5 * (l + u);
    };
    *lo = kth(0);
    *hi = kth(n - 1);
}

}  // namespace

// Lanczos estimate of the extreme eigenvalues of a symmetric operator on vectors of len
// doubles, restating Lanczos (src/eigenSolver.c:1920-2129): stop when both extremes change by
// less than tol. A Hermitian H_k acting on complex vectors stored as interleaved (re, im)
// doubles runs through the same recurrence (Lanczos_kpt, src/eigenSolverKpt.c:1361): its
// coefficients are real and Re(x^H y) is the dot product of the interleaved arrays.
int lanczos_run(sgpu_ctx *ctx, long len, const std::function<int(const double *, double *)> &apply,
                const double *x0, double tol, int maxit, double *eigmin, double *eigmax,
                cudaStream_t st)
{
    const long N = len;
    double *v = nullptr;
    SGPU_TRY(ws_get(ctx, WS_SCF2, sizeof(double) * (size_t)N * 3, (void **)&v));
    double *Vjm1 = v, *Vj = v + N, *Vjp1 = v + 2 * N;
    SGPU_CUDA_TRY(cudaMemcpyAsync(Vjm1, x0, sizeof(double) * N, cudaMemcpyDefault, st));
    double nrm2 = 0.0;
    SGPU_TRY(dot_host(ctx, Vjm1, Vjm1, N, &nrm2, st));
    SGPU_TRY(axpby_dev(ctx, N, 1.0 / std::sqrt(nrm2), Vjm1, 0.0, nullptr, Vjm1, st));
    SGPU_TRY(apply(Vjm1, Vj));
    std::vector<double> a(maxit + 2), b(maxit + 2);
    SGPU_TRY(dot_host(ctx, Vjm1, Vj, N, &a[0], st));
    SGPU_TRY(axpby_dev(ctx, N, 1.0, Vj, -a[0], Vjm1, Vj, st));
    SGPU_TRY(dot_host(ctx, Vj, Vj, N, &nrm2, st));
    b[0] = std::sqrt(nrm2);
    if (b[0] == 0.0) {
        set_error("Lanczos: the start vector is an eigenvector");
        return SGPU_ERR_LINALG;
    }
    SGPU_TRY(axpby_dev(ctx, N, 1.0 / b[0], Vj, 0.0, nullptr, Vj, st));
    double emin = 0.0, emax = 0.0, pmin = 0.0, pmax = 0.0;
    double errmin = tol + 1.0, errmax = tol + 1.0;
    int j = 0;
    while ((errmin > tol || errmax > tol) && j < maxit) {
        SGPU_TRY(apply(Vj, Vjp1));
        SGPU_TRY(dot_host(ctx, Vj, Vjp1, N, &a[j + 1], st));
        // Vjp1 -= a[j+1] Vj + b[j] Vjm1 ; Vjm1 = Vj
        SGPU_TRY(axpby_dev(ctx, N, 1.0, Vjp1, -a[j + 1], Vj, Vjp1, st));
        SGPU_TRY(axpby_dev(ctx, N, 1.0, Vjp1, -b[j], Vjm1, Vjp1, st));
        SGPU_CUDA_TRY(cudaMemcpyAsync(Vjm1, Vj, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        SGPU_TRY(dot_host(ctx, Vjp1, Vjp1, N, &nrm2, st));
        b[j + 1] = std::sqrt(nrm2);
        if (b[j + 1] == 0.0) break;
        SGPU_TRY(axpby_dev(ctx, N, 1.0 / b[j + 1], Vjp1, 0.0, nullptr, Vj, st));
        tridiag_extremes(j + 2, a.data(), b.data(), &emin, &emax);
        errmin = std::fabs(emin - pmin);
        errmax = std::fabs(emax - pmax);
        pmin = emin;
        pmax = emax;
        j++;
    }
    *eigmin = emin;
    *eigmax = emax;
    return SGPU_OK;
}

// Lanczos on the Gamma-point H of one spin block
int lanczos_dev(sgpu_ctx *ctx, int spin, const double *x0, double tol, int maxit,
                double *eigmin, double *eigmax, cudaStream_t st)
{
    const long N = ctx->Nd;
    auto apply = [&](const double *in, double *out) {
        return hamiltonian_dev<double>(ctx, spin, 1, 0.0, in, N, out, N, 1.0, 0.0, nullptr, 0, st);
    };
    return lanczos_run(ctx, N, apply, x0, tol, maxit, eigmin, eigmax, st);
}

}  // namespace sgpu

using namespace sgpu;

namespace {

// stage an Nd-vector (or ncol x Nd block, leading dim Nd) to a device scratch slot
int stage_vec(sgpu_ctx *ctx, int slot, const double *p, long n, double **out)
{
    if (is_device_ptr(p)) {
        *out = const_cast<double *>(p);
        return SGPU_OK;
    }
    SGPU_TRY(ws_get(ctx, slot, sizeof(double) * (size_t)(n > 0 ? n : 1), (void **)out));
    if (p && n > 0)
        SGPU_CUDA_TRY(cudaMemcpyAsync(*out, p, sizeof(double) * n, cudaMemcpyHostToDevice,
                                      ctx->stream));
    return SGPU_OK;
}

int unstage_vec(sgpu_ctx *ctx, const double *d, double *p, long n)
{
    if (d == p || n <= 0) return SGPU_OK;
    SGPU_CUDA_TRY(cudaMemcpyAsync(p, d, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    return SGPU_OK;
}

int check(sgpu_ctx *ctx)
{
    if (!ctx) {
        set_error("null context");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    return SGPU_OK;
}

}  // namespace

extern "C" {

int sgpu_Project_Hamiltonian(sgpu_ctx *ctx, int spin, const double *Y, int ldi, double *HY,
                             int ldo, int ncol, double *Hp, double *Mp)
{
    SGPU_TRY(check(ctx));
    if (ncol <= 0 || ldi < ctx->Nd || ldo < ctx->Nd) {
        set_error("Project_Hamiltonian: need ncol > 0 and leading dimensions >= Nd");
        return SGPU_ERR_ARG;
    }
    double *dY, *dHY, *dHp, *dMp;
    const bool hy = !is_device_ptr(Y), hh = !is_device_ptr(HY);
    long ly = ldi, lh = ldo;
    if (hy) {
        SGPU_TRY(ws_get(ctx, WS_STAGE_A, sizeof(double) * (size_t)ctx->Nd * ncol, (void **)&dY));
        SGPU_CUDA_TRY(cudaMemcpy2DAsync(dY, sizeof(double) * ctx->Nd, Y, sizeof(double) * ldi,
                                        sizeof(double) * ctx->Nd, ncol, cudaMemcpyHostToDevice,
                                        ctx->stream));
        ly = ctx->Nd;
    } else {
        dY = const_cast<double *>(Y);
    }
    if (hh) {
        SGPU_TRY(ws_get(ctx, WS_STAGE_B, sizeof(double) * (size_t)ctx->Nd * ncol, (void **)&dHY));
        lh = ctx->Nd;
    } else {
        dHY = HY;
    }
    const long n2 = (long)ncol * ncol;
    SGPU_TRY(stage_vec(ctx, WS_SCF, Hp, 2 * n2, &dHp));  // scratch for both when host
    dMp = is_device_ptr(Mp) ? Mp : dHp + n2;
    if (is_device_ptr(Hp) && !is_device_ptr(Mp)) {
        SGPU_TRY(ws_get(ctx, WS_SCF2, sizeof(double) * n2, (void **)&dMp));
    }
    SGPU_TRY(hamiltonian_dev<double>(ctx, spin, ncol, 0.0, dY, ly, dHY, lh, 1.0, 0.0, nullptr, 0,
                                     ctx->stream));
    SGPU_TRY(project_f64(ctx, ncol, dY, ly, dHY, lh, dHp, dMp, ctx->stream));
    if (hh)
        SGPU_CUDA_TRY(cudaMemcpy2DAsync(HY, sizeof(double) * ldo, dHY, sizeof(double) * lh,
                                        sizeof(double) * ctx->Nd, ncol, cudaMemcpyDeviceToHost,
                                        ctx->stream));
    SGPU_TRY(unstage_vec(ctx, dHp, Hp, n2));
    SGPU_TRY(unstage_vec(ctx, dMp, Mp, n2));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_Project_Hamiltonian_std(sgpu_ctx *ctx, int spin, double *Y, int ldi, double *HY,
                                 int ldo, int ncol, double *Hp)
{
    SGPU_TRY(check(ctx));
    if (ncol <= 0 || ldi < ctx->Nd || ldo < ctx->Nd || !Y || !HY || !Hp) {
        set_error("Project_Hamiltonian_std: need ncol > 0, arrays and leading dimensions >= Nd");
        return SGPU_ERR_ARG;
    }
    double *dY, *dHY, *dHp;
    const bool hy = !is_device_ptr(Y), hh = !is_device_ptr(HY);
    long ly = ldi, lh = ldo;
    if (hy) {
        SGPU_TRY(ws_get(ctx, WS_STAGE_A, sizeof(double) * (size_t)ctx->Nd * ncol, (void **)&dY));
        SGPU_CUDA_TRY(cudaMemcpy2DAsync(dY, sizeof(double) * ctx->Nd, Y, sizeof(double) * ldi,
                                        sizeof(double) * ctx->Nd, ncol, cudaMemcpyHostToDevice,
                                        ctx->stream));
        ly = ctx->Nd;
    } else {
        dY = Y;
    }
    if (hh) {
        SGPU_TRY(ws_get(ctx, WS_STAGE_B, sizeof(double) * (size_t)ctx->Nd * ncol, (void **)&dHY));
        lh = ctx->Nd;
    } else {
        dHY = HY;
    }
    const long n2 = (long)ncol * ncol;
    SGPU_TRY(stage_vec(ctx, WS_SCF, Hp, n2, &dHp));
    SGPU_TRY(cholqr_f64(ctx, ncol, dY, ly, ctx->stream));
    SGPU_TRY(hamiltonian_dev<double>(ctx, spin, ncol, 0.0, dY, ly, dHY, lh, 1.0, 0.0, nullptr, 0,
                                     ctx->stream));
    {
        SGPU_CUBLAS_TRY(cublasSetStream(ctx->cublas, ctx->stream));
        const double one = 1.0, zero = 0.0;
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, ctx->stream);
        SGPU_CUBLAS_TRY(cublasDgemm(ctx->cublas, CUBLAS_OP_T, CUBLAS_OP_N, ncol, ncol,
                                    (int)ctx->Nd, &one, dY, (int)ly, dHY, (int)lh, &zero, dHp,
                                    ncol));
    }
    if (hy)
        SGPU_CUDA_TRY(cudaMemcpy2DAsync(Y, sizeof(double) * ldi, dY, sizeof(double) * ly,
                                        sizeof(double) * ctx->Nd, ncol, cudaMemcpyDeviceToHost,
                                        ctx->stream));
    if (hh)
        SGPU_CUDA_TRY(cudaMemcpy2DAsync(HY, sizeof(double) * ldo, dHY, sizeof(double) * lh,
                                        sizeof(double) * ctx->Nd, ncol, cudaMemcpyDeviceToHost,
                                        ctx->stream));
    SGPU_TRY(unstage_vec(ctx, dHp, Hp, n2));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_Solve_Standard_EigenProblem(sgpu_ctx *ctx, int Ns, double *Hp, double *lambda)
{
    SGPU_TRY(check(ctx));
    if (Ns <= 0 || !Hp || !lambda) {
        set_error("Solve_Standard_EigenProblem: bad arguments");
        return SGPU_ERR_ARG;
    }
    const long n2 = (long)Ns * Ns;
    double *dH, *dl;
    SGPU_TRY(stage_vec(ctx, WS_SCF, Hp, n2, &dH));
    SGPU_TRY(stage_vec(ctx, WS_SCF2, is_device_ptr(lambda) ? lambda : nullptr, Ns, &dl));
    SGPU_TRY(standard_eig(ctx, Ns, dH, dl, ctx->stream));
    SGPU_TRY(unstage_vec(ctx, dH, Hp, n2));
    SGPU_TRY(unstage_vec(ctx, dl, lambda, Ns));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_Solve_Generalized_EigenProblem(sgpu_ctx *ctx, int Ns, double *Hp, double *Mp,
                                        double *lambda)
{
    SGPU_TRY(check(ctx));
    if (Ns <= 0) {
        set_error("Solve_Generalized_EigenProblem: Ns must be positive");
        return SGPU_ERR_ARG;
    }
    const long n2 = (long)Ns * Ns;
    double *dH, *dM, *dl;
    SGPU_TRY(stage_vec(ctx, WS_SCF, Hp, n2, &dH));
    SGPU_TRY(stage_vec(ctx, WS_SCF2, Mp, n2, &dM));
    SGPU_TRY(stage_vec(ctx, WS_RHS, lambda, Ns, &dl));
    int rc = generalized_eig(ctx, Ns, dH, dM, dl, ctx->stream);
    if (rc != SGPU_OK) return rc;
    SGPU_TRY(unstage_vec(ctx, dH, Hp, n2));
    SGPU_TRY(unstage_vec(ctx, dM, Mp, n2));
    SGPU_TRY(unstage_vec(ctx, dl, lambda, Ns));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_Subspace_Rotation(sgpu_ctx *ctx, const double *Y, int ldi, const double *Q, int ncol,
                           double *X, int ldo)
{
    SGPU_TRY(check(ctx));
    if (ncol <= 0 || ldi < ctx->Nd || ldo < ctx->Nd) {
        set_error("Subspace_Rotation: need ncol > 0 and leading dimensions >= Nd");
        return SGPU_ERR_ARG;
    }
    double *dY, *dX, *dQ;
    long ly = ldi, lx = ldo;
    if (!is_device_ptr(Y)) {
        SGPU_TRY(ws_get(ctx, WS_STAGE_A, sizeof(double) * (size_t)ctx->Nd * ncol, (void **)&dY));
        SGPU_CUDA_TRY(cudaMemcpy2DAsync(dY, sizeof(double) * ctx->Nd, Y, sizeof(double) * ldi,
                                        sizeof(double) * ctx->Nd, ncol, cudaMemcpyHostToDevice,
                                        ctx->stream));
        ly = ctx->Nd;
    } else {
        dY = const_cast<double *>(Y);
    }
    const bool hx = !is_device_ptr(X);
    if (hx) {
        SGPU_TRY(ws_get(ctx, WS_STAGE_B, sizeof(double) * (size_t)ctx->Nd * ncol, (void **)&dX));
        lx = ctx->Nd;
    } else {
        dX = X;
    }
    SGPU_TRY(stage_vec(ctx, WS_SCF, Q, (long)ncol * ncol, &dQ));
    SGPU_TRY(rotate_f64(ctx, ncol, dY, ly, dQ, dX, lx, ctx->stream));
    if (hx)
        SGPU_CUDA_TRY(cudaMemcpy2DAsync(X, sizeof(double) * ldo, dX, sizeof(double) * lx,
                                        sizeof(double) * ctx->Nd, ncol, cudaMemcpyDeviceToHost,
                                        ctx->stream));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

// FP32 orbital blocks (device): the Rayleigh-Ritz products of the mixed SCF's FP32 phase, Hp
// and Mp (or Q) FP64 on the host or the device.
int sgpu_Project_Hamiltonian_f32(sgpu_ctx *ctx, int spin, const float *Y, int ldi, float *HY,
                                 int ldo, int ncol, double *Hp, double *Mp)
{
    SGPU_TRY(check(ctx));
    if (ncol <= 0 || ldi < ctx->Nd || ldo < ctx->Nd || !Y || !HY || !Hp || !Mp) {
        set_error("Project_Hamiltonian_f32: need ncol > 0, arrays and leading dimensions >= Nd");
        return SGPU_ERR_ARG;
    }
    if (!is_device_ptr(Y) || !is_device_ptr(HY)) {
        set_error("Project_Hamiltonian_f32: Y and HY must be device FP32 blocks");
        return SGPU_ERR_ARG;
    }
    const long n2 = (long)ncol * ncol;
    double *dHp, *dMp;
    SGPU_TRY(stage_vec(ctx, WS_SCF, Hp, 2 * n2, &dHp));
    dMp = is_device_ptr(Mp) ? Mp : dHp + n2;
    if (is_device_ptr(Hp) && !is_device_ptr(Mp))
        SGPU_TRY(ws_get(ctx, WS_SCF2, sizeof(double) * n2, (void **)&dMp));
    SGPU_TRY(hamiltonian_dev<float>(ctx, spin, ncol, 0.0, Y, ldi, HY, ldo, 1.0, 0.0, nullptr, 0,
                                    ctx->stream));
    SGPU_TRY(project_f32(ctx, ncol, Y, ldi, HY, ldo, dHp, dMp, ctx->stream));
    SGPU_TRY(unstage_vec(ctx, dHp, Hp, n2));
    SGPU_TRY(unstage_vec(ctx, dMp, Mp, n2));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_Subspace_Rotation_f32(sgpu_ctx *ctx, const float *Y, int ldi, const double *Q, int ncol,
                               float *X, int ldo)
{
    SGPU_TRY(check(ctx));
    if (ncol <= 0 || ldi < ctx->Nd || ldo < ctx->Nd || !Y || !Q || !X) {
        set_error("Subspace_Rotation_f32: need ncol > 0, arrays and leading dimensions >= Nd");
        return SGPU_ERR_ARG;
    }
    if (!is_device_ptr(Y) || !is_device_ptr(X)) {
        set_error("Subspace_Rotation_f32: Y and X must be device FP32 blocks");
        return SGPU_ERR_ARG;
    }
    double *dQ;
    SGPU_TRY(stage_vec(ctx, WS_SCF, Q, (long)ncol * ncol, &dQ));
    SGPU_TRY(rotate_f32(ctx, ncol, Y, ldi, dQ, X, ldo, ctx->stream));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_CalculateDensity_psi(sgpu_ctx *ctx, const double *psi, int ld, int ncol,
                              const double *occ, double occfac, double *rho)
{
    SGPU_TRY(check(ctx));
    if (ncol <= 0 || ld < ctx->Nd || !occ) {
        set_error("CalculateDensity_psi: need ncol > 0, ld >= Nd and occupations");
        return SGPU_ERR_ARG;
    }
    double *dpsi, *drho, *dw;
    long lp = ld;
    if (!is_device_ptr(psi)) {
        SGPU_TRY(ws_get(ctx, WS_STAGE_A, sizeof(double) * (size_t)ctx->Nd * ncol, (void **)&dpsi));
        SGPU_CUDA_TRY(cudaMemcpy2DAsync(dpsi, sizeof(double) * ctx->Nd, psi, sizeof(double) * ld,
                                        sizeof(double) * ctx->Nd, ncol, cudaMemcpyHostToDevice,
                                        ctx->stream));
        lp = ctx->Nd;
    } else {
        dpsi = const_cast<double *>(psi);
    }
    std::vector<double> w(ncol);
    std::vector<double> occh(ncol);
    if (is_device_ptr(occ))
        SGPU_CUDA_TRY(cudaMemcpy(occh.data(), occ, sizeof(double) * ncol, cudaMemcpyDeviceToHost));
    else
        std::copy(occ, occ + ncol, occh.begin());
    for (int n = 0; n < ncol; n++) w[n] = occfac * occh[n] / ctx->dV;
    SGPU_TRY(ws_get(ctx, WS_SCF, sizeof(double) * ncol, (void **)&dw));
    SGPU_CUDA_TRY(cudaMemcpyAsync(dw, w.data(), sizeof(double) * ncol, cudaMemcpyHostToDevice,
                                  ctx->stream));
    SGPU_TRY(stage_vec(ctx, WS_RHS, is_device_ptr(rho) ? rho : nullptr, ctx->Nd, &drho));
    SGPU_TRY(density_dev<double>(ctx, dpsi, lp, ncol, dw, drho, ctx->stream));
    SGPU_TRY(unstage_vec(ctx, drho, rho, ctx->Nd));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_Calculate_Vxc_LDA_PW(sgpu_ctx *ctx, const double *rho, const double *rho_core,
                              double xc_rhotol, double *vxc, double *exc)
{
    SGPU_TRY(check(ctx));
    double *dr, *dc = nullptr, *dv, *de;
    SGPU_TRY(stage_vec(ctx, WS_STAGE_A, rho, ctx->Nd, &dr));
    if (rho_core) SGPU_TRY(stage_vec(ctx, WS_STAGE_B, rho_core, ctx->Nd, &dc));
    double *out = nullptr;
    SGPU_TRY(ws_get(ctx, WS_STAGE_C, sizeof(double) * 2 * (size_t)ctx->Nd, (void **)&out));
    dv = is_device_ptr(vxc) ? vxc : out;
    de = is_device_ptr(exc) ? exc : out + ctx->Nd;
    SGPU_TRY(lda_pw_dev(ctx, dr, dc, xc_rhotol, dv, de, ctx->stream));
    SGPU_TRY(unstage_vec(ctx, dv, vxc, ctx->Nd));
    SGPU_TRY(unstage_vec(ctx, de, exc, ctx->Nd));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_AAR(sgpu_ctx *ctx, double c, double *x, const double *b, double omega, double beta,
             int m, int p, double tol, int max_iter, int *iters)
{
    SGPU_TRY(check(ctx));
    double *dx, *db;
    SGPU_TRY(stage_vec(ctx, WS_STAGE_A, x, ctx->Nd, &dx));
    SGPU_TRY(stage_vec(ctx, WS_STAGE_B, b, ctx->Nd, &db));
    const int rc = aar_dev(ctx, c, dx, db, omega, beta, m, p, tol, max_iter, iters, ctx->stream);
    if (rc != SGPU_OK && rc != SGPU_ERR_NOT_CONVERGED) return rc;
    SGPU_TRY(unstage_vec(ctx, dx, x, ctx->Nd));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return rc;
}

int sgpu_Calculate_elecstPotential(sgpu_ctx *ctx, const double *rho, const double *b,
                                   double *phi, double tol, int max_iter, int *iters)
{
    SGPU_TRY(check(ctx));
    double *dr, *db, *dp;
    SGPU_TRY(stage_vec(ctx, WS_STAGE_A, rho, ctx->Nd, &dr));
    SGPU_TRY(stage_vec(ctx, WS_STAGE_B, b, ctx->Nd, &db));
    SGPU_TRY(stage_vec(ctx, WS_STAGE_C, phi, ctx->Nd, &dp));
    SGPU_TRY(poisson_dev(ctx, dr, db, dp, tol, max_iter, iters, ctx->stream));
    SGPU_TRY(unstage_vec(ctx, dp, phi, ctx->Nd));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_Mixing_init(sgpu_ctx *ctx, int history, int pulay_frequency, int pulay_restart,
                     double mixing_parameter, double mixing_parameter_simple, int kerker,
                     double kTF, double idiemac, double tol_precond, double neg_charge,
                     const double *rho_in)
{
    SGPU_TRY(check(ctx));
    MixParams prm;
    prm.m = history;
    prm.pulay_freq = std::max(1, pulay_frequency);
    prm.restart = pulay_restart;
    prm.beta = mixing_parameter;
    prm.omega = mixing_parameter_simple;
    prm.kerker = kerker;
    prm.kTF = kTF;
    prm.idiemac = idiemac;
    prm.precond_tol = tol_precond;
    prm.neg_charge = neg_charge;
    return mixing_init(ctx, prm, rho_in);
}

int sgpu_Calculate_Vxc_LSDA_PW(sgpu_ctx *ctx, const double *rho_up, const double *rho_dn,
                               const double *rho_core, double xc_rhotol, double *vxc,
                               double *exc)
{
    SGPU_TRY(check(ctx));
    const long N = ctx->Nd;
    double *du, *dd, *dc = nullptr;
    SGPU_TRY(stage_vec(ctx, WS_STAGE_A, rho_up, N, &du));
    SGPU_TRY(stage_vec(ctx, WS_STAGE_B, rho_dn, N, &dd));
    if (rho_core) SGPU_TRY(stage_vec(ctx, WS_RHS, rho_core, N, &dc));
    double *out = nullptr;
    SGPU_TRY(ws_get(ctx, WS_STAGE_C, sizeof(double) * 3 * (size_t)N, (void **)&out));
    double *dv = is_device_ptr(vxc) ? vxc : out;
    double *de = is_device_ptr(exc) ? exc : out + 2 * N;
    SGPU_TRY(lsda_pw_dev(ctx, du, dd, dc, xc_rhotol, dv, dv + N, de, ctx->stream));
    SGPU_TRY(unstage_vec(ctx, dv, vxc, 2 * N));
    SGPU_TRY(unstage_vec(ctx, de, exc, N));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_Mixing_init_spin(sgpu_ctx *ctx, int history, int pulay_frequency, int pulay_restart,
                          double mixing_parameter, double mixing_parameter_simple,
                          double mixing_parameter_mag, double mixing_parameter_simple_mag,
                          int kerker, double kTF, double idiemac, double tol_precond,
                          double neg_charge, const double *rho_in, const double *mag_in)
{
    SGPU_TRY(check(ctx));
    if (!rho_in || !mag_in) {
        set_error("sgpu_Mixing_init_spin: null density or magnetization");
        return SGPU_ERR_ARG;
    }
    MixParams prm;
    prm.m = history;
    prm.pulay_freq = std::max(1, pulay_frequency);
    prm.restart = pulay_restart;
    prm.beta = mixing_parameter;
    prm.omega = mixing_parameter_simple;
    prm.kerker = kerker;
    prm.kTF = kTF;
    prm.idiemac = idiemac;
    prm.precond_tol = tol_precond;
    prm.neg_charge = neg_charge;
    prm.nspden = 2;
    prm.beta_mag = mixing_parameter_mag;
    prm.omega_mag = mixing_parameter_simple_mag;
    const long N = ctx->Nd;
    double *x0 = nullptr;
    SGPU_TRY(ws_get(ctx, WS_STAGE_A, sizeof(double) * 2 * (size_t)N, (void **)&x0));
    SGPU_CUDA_TRY(cudaMemcpyAsync(x0, rho_in, sizeof(double) * N, cudaMemcpyDefault, ctx->stream));
    SGPU_CUDA_TRY(cudaMemcpyAsync(x0 + N, mag_in, sizeof(double) * N, cudaMemcpyDefault,
                                  ctx->stream));
    return mixing_init(ctx, prm, x0);
}

int sgpu_Mixing_periodic_pulay_spin(sgpu_ctx *ctx, int iter_count, double *rho, double *mag)
{
    SGPU_TRY(check(ctx));
    if (!ctx->mix || ctx->mix->prm.nspden != 2) {
        set_error("sgpu_Mixing_periodic_pulay_spin: call sgpu_Mixing_init_spin first");
        return SGPU_ERR_STATE;
    }
    const long N = ctx->Nd;
    double *g = nullptr;
    SGPU_TRY(ws_get(ctx, WS_STAGE_A, sizeof(double) * 2 * (size_t)N, (void **)&g));
    SGPU_CUDA_TRY(cudaMemcpyAsync(g, rho, sizeof(double) * N, cudaMemcpyDefault, ctx->stream));
    SGPU_CUDA_TRY(cudaMemcpyAsync(g + N, mag, sizeof(double) * N, cudaMemcpyDefault, ctx->stream));
    SGPU_TRY(mixing_step(ctx, iter_count, g, ctx->stream));
    SGPU_CUDA_TRY(cudaMemcpyAsync(rho, g, sizeof(double) * N, cudaMemcpyDefault, ctx->stream));
    SGPU_CUDA_TRY(cudaMemcpyAsync(mag, g + N, sizeof(double) * N, cudaMemcpyDefault, ctx->stream));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_Mixing_periodic_pulay(sgpu_ctx *ctx, int iter_count, double *rho)
{
    SGPU_TRY(check(ctx));
    if (ctx->mix && ctx->mix->prm.nspden != 1) {
        set_error("sgpu_Mixing_periodic_pulay: the history was set up for spin "
                  "(use sgpu_Mixing_periodic_pulay_spin)");
        return SGPU_ERR_STATE;
    }
    double *dr;
    SGPU_TRY(stage_vec(ctx, WS_STAGE_A, rho, ctx->Nd, &dr));
    SGPU_TRY(mixing_step(ctx, iter_count, dr, ctx->stream));
    SGPU_TRY(unstage_vec(ctx, dr, rho, ctx->Nd));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_Evaluate_scf_error(sgpu_ctx *ctx, const double *rho_out, const double *rho_in,
                            double *error)
{
    SGPU_TRY(check(ctx));
    double *a, *b;
    SGPU_TRY(stage_vec(ctx, WS_STAGE_A, rho_out, ctx->Nd, &a));
    SGPU_TRY(stage_vec(ctx, WS_STAGE_B, rho_in, ctx->Nd, &b));
    return scf_error_dev(ctx, a, b, error, ctx->stream);
}

int sgpu_Lanczos(sgpu_ctx *ctx, int spin, const double *x0, double tol, int maxit,
                 double *eigmin, double *eigmax)
{
    SGPU_TRY(check(ctx));
    return lanczos_dev(ctx, spin, x0, tol, maxit, eigmin, eigmax, ctx->stream);
}

// ---------------------------------------------------------------------------- SCF

int sgpu_scf(sgpu_ctx *ctx, const sgpu_scf_params *prm, const double *b, const double *rho_init,
             const double *rho_core, double *rho_out, double *lambda_out, double *occ_out,
             sgpu_scf_result *res)
{
    SGPU_TRY(check(ctx));
    if (!prm || !b || !rho_init || !res) {
        set_error("sgpu_scf: null argument");
        return SGPU_ERR_ARG;
    }
    const int Ns = prm->Nstates;
    if (Ns <= 0 || prm->cheb_degree < 1) {
        set_error("sgpu_scf: need Nstates > 0 and a Chebyshev degree >= 1");
        return SGPU_ERR_ARG;
    }
    if (prm->precision != SGPU_PREC_FP64 && prm->precision != SGPU_PREC_FP32) {
        set_error("sgpu_scf: precision must be SGPU_PREC_FP64 or SGPU_PREC_FP32");
        return SGPU_ERR_ARG;
    }
    if (prm->spin_typ != 0) {
        set_error("sgpu_scf: spin-polarised runs go through sgpu_scf_kpt (a k = 0 grid for the "
                  "Gamma point)");
        return SGPU_ERR_ARG;
    }
    if (prm->graded_tail < 0 || prm->graded_tail > 1 ||
        (prm->graded_tail == 1 &&
         (prm->tail_fp64_degrees < 0 || prm->tail_fp64_degrees >= prm->cheb_degree))) {
        set_error("sgpu_scf: graded_tail must be 0 or 1, and tail_fp64_degrees in "
                  "[0, cheb_degree) for 1");
        return SGPU_ERR_ARG;
    }
    auto t0 = std::chrono::steady_clock::now();
    cudaStream_t st = ctx->stream;
    const long N = ctx->Nd;
    const long nb = N * (long)Ns;

    // persistent device vectors of the SCF (SPARC_OBJ fields of the same role)
    double *vec = nullptr;
    SGPU_CUDA_TRY(cudaMalloc(&vec, sizeof(double) * (size_t)N * 8 + sizeof(double) * 4 * (size_t)Ns * Ns + 4096));
    struct Guard { double *p; ~Guard() { if (p) cudaFree(p); } } guard{vec};
    double *d_b = vec, *d_core = vec + N, *d_rho = vec + 2 * N, *d_phi = vec + 3 * N;
    double *d_vxc = vec + 4 * N, *d_exc = vec + 5 * N, *d_veff = vec + 6 * N, *d_rhoout = vec + 7 * N;
    double *d_Hp = vec + 8 * N, *d_Mp = d_Hp + (long)Ns * Ns, *d_lam = d_Mp + (long)Ns * Ns;
    double *d_w = d_lam + Ns;
    SGPU_CUDA_TRY(cudaMemcpyAsync(d_b, b, sizeof(double) * N, cudaMemcpyDefault, st));
    if (rho_core)
        SGPU_CUDA_TRY(cudaMemcpyAsync(d_core, rho_core, sizeof(double) * N, cudaMemcpyDefault, st));
    SGPU_CUDA_TRY(cudaMemcpyAsync(d_rho, rho_init, sizeof(double) * N, cudaMemcpyDefault, st));
    SGPU_CUDA_TRY(cudaMemsetAsync(d_phi, 0, sizeof(double) * N, st));
    const double *core = rho_core ? d_core : nullptr;

    // orbital blocks: FP64 X, Y always; FP32 pair while in mixed mode
    double *X64 = nullptr, *Y64 = nullptr;
    float *X32 = nullptr, *Y32 = nullptr;
    SGPU_CUDA_TRY(cudaMalloc(&X64, sizeof(double) * (size_t)nb));
    struct G2 { double *p; ~G2() { if (p) cudaFree(p); } } gx{X64};
    SGPU_CUDA_TRY(cudaMalloc(&Y64, sizeof(double) * (size_t)nb));
    struct G3 { double *p; ~G3() { if (p) cudaFree(p); } } gy{Y64};
    bool mixed = prm->precision == SGPU_PREC_FP32;
    if (mixed) {
        SGPU_CUDA_TRY(cudaMalloc(&X32, sizeof(float) * (size_t)nb * 2));
        Y32 = X32 + nb;
    }
    struct G4 { float *p; ~G4() { if (p) cudaFree(p); } } g32{X32};
    if (mixed && !ctx->stencil_tuned)  // tuned at the block width the filter runs at
        SGPU_TRY(sgpu_autotune(ctx, Ns, nullptr, nullptr));
    init_orbitals(ctx, X64, nb, prm->seed, 152 * 8, st);
    if (mixed) SGPU_TRY(convert_cols<double, float>(X64, nb, X32, nb, nb, 1, st));

    const double occfac = 2.0;  // spin-unpolarised
    const double neg_charge = -prm->Nelectron;
    int pits = 0;
    // initial potential (scf(), src/electronicGroundState.c:677-704)
    SGPU_TRY(poisson_dev(ctx, d_rho, d_b, d_phi, prm->tol_poisson, prm->maxit_poisson, &pits, st));
    SGPU_TRY(lda_pw_dev(ctx, d_rho, core, prm->xc_rhotol, d_vxc, d_exc, st));
    SGPU_TRY(axpby_dev(ctx, N, 1.0, d_phi, 1.0, d_vxc, d_veff, st));
    SGPU_TRY(sgpu_set_veff(ctx, 1, d_veff));
    MixParams mp;
    mp.m = prm->mixing_history;
    mp.pulay_freq = std::max(1, prm->pulay_freq);
    mp.restart = prm->pulay_restart;
    mp.beta = prm->mixing_param;
    mp.omega = prm->mixing_param_simple;
    mp.kerker = prm->kerker;
    mp.kTF = prm->kerker_kTF;
    mp.idiemac = prm->kerker_idiemac;
    mp.precond_tol = prm->tol_precond;
    mp.neg_charge = neg_charge;
    SGPU_TRY(mixing_init(ctx, mp, d_rho));

    std::vector<double> lam(Ns), occ(Ns, 0.0);
    double eigmin = 0.0, eigmax = 0.0, efermi = 0.0, error = prm->tol_scf + 1.0;
    double Etot = 0, Eband = 0, E1 = 0, E2 = 0, E3 = 0, Exc = 0, Entropy = 0;
    int scf = 0, switch_iter = mixed ? -1 : 0;
    // after the switch: plain FP64, or the graded filter with FP64 Rayleigh-Ritz
    bool graded = false;
    double best_error = 1e300;
    int stall = 0;
    double filter_ms = 0.0;
    const int m = prm->cheb_degree;
    while (scf < prm->maxit_scf) {
        // ---- eigSolve_CheFSI
        int count = scf == 0 ? 0 : prm->rho_trigger + (scf - 1) * prm->nchefsi;
        const int cend = prm->rho_trigger + scf * prm->nchefsi;
        for (; count < cend; count++) {
            double cutoff;
            if (count == 0) {
                // Lanczos on H from a random start vector, then the reference's safety margins
                double *x0 = nullptr;
                SGPU_TRY(ws_get(ctx, WS_SCF, sizeof(double) * N, (void **)&x0));
                init_orbitals(ctx, x0, N, prm->seed ^ 0x5bd1e995ull, 152, st);
                SGPU_TRY(lanczos_dev(ctx, 0, x0, prm->tol_lanczos, 1000, &eigmin, &eigmax, st));
                eigmax *= 1.01;
                eigmin -= 0.1;
                cutoff = 0.5 * (eigmin + eigmax);
            } else {
                if (count >= prm->rho_trigger) eigmin = lam[0];
                cutoff = lam[Ns - 1] + 0.1;
            }
            cudaEvent_t e0 = ctx->ev0, e1 = ctx->ev1;
            SGPU_CUDA_TRY(cudaEventRecord(e0, st));
            if (mixed) {
                SGPU_TRY(chebyshev_dev<float>(ctx, 0, X32, N, Y32, N, Ns, m, cutoff, eigmax, eigmin, st));
                // HY into X (the reference reuses Xorb for HY), then project in FP32 products
                SGPU_TRY(hamiltonian_dev<float>(ctx, 0, Ns, 0.0, Y32, N, X32, N, 1.0, 0.0, nullptr, 0, st));
                SGPU_TRY(project_f32(ctx, Ns, Y32, N, X32, N, d_Hp, d_Mp, st));
            } else if (graded) {
                SGPU_TRY(chebyshev_graded(ctx, 0, X32, Y32, X64, Y64, Ns, m,
                                          prm->tail_fp64_degrees, cutoff, eigmax, eigmin, st));
                SGPU_TRY(hamiltonian_dev<double>(ctx, 0, Ns, 0.0, Y64, N, X64, N, 1.0, 0.0, nullptr, 0, st));
                if (ctx->rr_tc)  // FP64-accurate split products on the tensor cores
                    SGPU_TRY(tc_project<double>(ctx, Ns, Y64, N, X64, N, d_Hp, d_Mp, true, st));
                else
                    SGPU_TRY(project_f64(ctx, Ns, Y64, N, X64, N, d_Hp, d_Mp, st));
            } else {
                SGPU_TRY(chebyshev_dev<double>(ctx, 0, X64, N, Y64, N, Ns, m, cutoff, eigmax, eigmin, st));
                SGPU_TRY(hamiltonian_dev<double>(ctx, 0, Ns, 0.0, Y64, N, X64, N, 1.0, 0.0, nullptr, 0, st));
                SGPU_TRY(project_f64(ctx, Ns, Y64, N, X64, N, d_Hp, d_Mp, st));
            }
            SGPU_CUDA_TRY(cudaEventRecord(e1, st));
            SGPU_TRY(generalized_eig(ctx, Ns, d_Hp, d_Mp, d_lam, st));
            float ms = 0.f;
            SGPU_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
            filter_ms += ms;
            if (mixed) {
                SGPU_TRY(rotate_f32(ctx, Ns, Y32, N, d_Hp, X32, N, st));
            } else if (graded && ctx->rr_tc) {
                SGPU_TRY(tc_rotate<double>(ctx, Ns, Y64, N, d_Hp, Ns, X64, N, true, st));
                SGPU_TRY(convert_cols<double, float>(X64, nb, X32, nb, nb, 1, st));
            } else {
                SGPU_TRY(rotate_f64(ctx, Ns, Y64, N, d_Hp, X64, N, st));
                // the graded filter starts from an FP32 copy of the rotated orbitals
                if (graded) SGPU_TRY(convert_cols<double, float>(X64, nb, X32, nb, nb, 1, st));
            }
            SGPU_CUDA_TRY(cudaMemcpyAsync(lam.data(), d_lam, sizeof(double) * Ns,
                                          cudaMemcpyDeviceToHost, st));
            SGPU_CUDA_TRY(cudaStreamSynchronize(st));
            int fst = 0;
            efermi = fermi_level(lam, std::vector<double>(Ns, occfac), prm->Nelectron, prm->Beta,
                                 prm->elec_T_type, lam[0] - 1.0, lam[Ns - 1] + 1.0, 1e-12, 100,
                                 &fst);
            if (fst) {
                set_error("sgpu_scf: cannot bracket the Fermi level");
                return SGPU_ERR_LINALG;
            }
            for (int n = 0; n < Ns; n++) occ[n] = smearing(prm->Beta, lam[n], efermi, prm->elec_T_type);
        }
        // ---- density from the rotated orbitals (CalculateDensity_psi)
        std::vector<double> w(Ns);
        for (int n = 0; n < Ns; n++) w[n] = occfac * occ[n] / ctx->dV;
        SGPU_CUDA_TRY(cudaMemcpyAsync(d_w, w.data(), sizeof(double) * Ns, cudaMemcpyHostToDevice, st));
        if (mixed)
            SGPU_TRY(density_dev<float>(ctx, X32, N, Ns, d_w, d_rhoout, st));
        else
            SGPU_TRY(density_dev<double>(ctx, X64, N, Ns, d_w, d_rhoout, st));
        // ---- energy with the input density x_k (Calculate_Free_Energy)
        const double *xk = ctx->mix->x_k;
        double sb = 0, s2 = 0, s3 = 0, sx = 0;
        SGPU_TRY(dot_host(ctx, d_b, d_phi, N, &sb, st));
        SGPU_TRY(dot_host(ctx, xk, d_phi, N, &s2, st));
        SGPU_TRY(dot_host(ctx, xk, d_vxc, N, &s3, st));
        {   // Exc = dV * sum (rho + rho_core, clamped) * e_xc
            double *rxc = nullptr;
            SGPU_TRY(ws_get(ctx, WS_RHS, sizeof(double) * N, (void **)&rxc));
            SGPU_TRY(axpby_dev(ctx, N, 1.0, xk, 1.0, core, rxc, st));
            SGPU_TRY(dot_host(ctx, rxc, d_exc, N, &sx, st));
        }
        E1 = 0.5 * sb * ctx->dV;
        E2 = 0.5 * s2 * ctx->dV;
        E3 = s3 * ctx->dV;
        Exc = sx * ctx->dV;
        Eband = 0.0;
        Entropy = 0.0;
        for (int n = 0; n < Ns; n++) {
            Eband += occfac * occ[n] * lam[n];
            const double g = occ[n];
            if (prm->elec_T_type == 0) {
                if (g > 1e-14 && (1.0 - g) > 1e-14) Entropy += -(g * std::log(g) + (1.0 - g) * std::log(1.0 - g));
            } else {
                const double x = prm->Beta * (lam[n] - efermi);
                Entropy += 0.5 / std::sqrt(M_PI) * std::exp(-x * x);
            }
        }
        Entropy *= -occfac / prm->Beta;
        Etot = Eband + E1 - E2 - E3 + Exc + prm->Esc + Entropy;
        if (Etot != Etot) {
            set_error("sgpu_scf: total energy is NaN");
            return SGPU_ERR_NONFINITE;
        }
        // ---- SCF error, mixing, new potential
        SGPU_TRY(scf_error_dev(ctx, d_rhoout, xk, &error, st));
        if (prm->history && scf < prm->maxit_scf) {
            prm->history[3 * scf] = Etot;
            prm->history[3 * scf + 1] = error;
            prm->history[3 * scf + 2] =
                std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        }
        SGPU_TRY(mixing_step(ctx, scf, d_rhoout, st));
        SGPU_CUDA_TRY(cudaMemcpyAsync(d_rho, d_rhoout, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        SGPU_TRY(poisson_dev(ctx, d_rho, d_b, d_phi, prm->tol_poisson, prm->maxit_poisson, &pits, st));
        SGPU_TRY(lda_pw_dev(ctx, d_rho, core, prm->xc_rhotol, d_vxc, d_exc, st));
        SGPU_TRY(axpby_dev(ctx, N, 1.0, d_phi, 1.0, d_vxc, d_veff, st));
        SGPU_TRY(sgpu_set_veff(ctx, 1, d_veff));
        scf++;
        if (prm->verbose)
            printf("sgpu_scf: iter %3d  Etot/atom %.10f  error %.3e  %s\n", scf,
                   Etot / std::max(1, prm->n_atom), error,
                   mixed ? "fp32" : (graded ? "graded" : "fp64"));
        if (error < prm->tol_scf && scf >= prm->minit_scf) break;
        if (mixed) {
            // leave FP32 below the threshold, or once the FP32 error has stopped falling
            // (two iterations in a row without a 20 % gain on the best so far): the FP32
            // Rayleigh-Ritz step sets a floor on the error that depends on the system
            stall = (scf >= 4 && error > 0.8 * best_error) ? stall + 1 : 0;
            best_error = std::min(best_error, error);
            if (error < prm->fp64_switch_error || stall >= 2) {
                // widen the orbital block and continue in FP64 (or graded)
                SGPU_TRY(convert_cols<float, double>(X32, nb, X64, nb, nb, 1, st));
                ctx->launches++;
                mixed = false;
                graded = prm->graded_tail != 0;
                switch_iter = scf;
            }
        }
    }
    if (rho_out) SGPU_CUDA_TRY(cudaMemcpyAsync(rho_out, d_rho, sizeof(double) * N, cudaMemcpyDefault, st));
    SGPU_CUDA_TRY(cudaStreamSynchronize(st));
    // the SCF's wall time ends here: the optional field outputs below are not part of it
    const double t_scf = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    // what the force calculation reads: the last rotated orbitals and the potentials of the
    // final (mixed) density, as the reference leaves them when its SCF loop ends
    if (prm->psi_out) {
        if (mixed) SGPU_TRY(convert_cols<float, double>(X32, nb, X64, nb, nb, 1, st));
        SGPU_CUDA_TRY(cudaMemcpyAsync(prm->psi_out, X64, sizeof(double) * nb, cudaMemcpyDefault, st));
    }
    if (prm->phi_out)
        SGPU_CUDA_TRY(cudaMemcpyAsync(prm->phi_out, d_phi, sizeof(double) * N, cudaMemcpyDefault, st));
    if (prm->vxc_out)
        SGPU_CUDA_TRY(cudaMemcpyAsync(prm->vxc_out, d_vxc, sizeof(double) * N, cudaMemcpyDefault, st));
    if (lambda_out) std::copy(lam.begin(), lam.end(), lambda_out);
    if (occ_out) std::copy(occ.begin(), occ.end(), occ_out);
    SGPU_CUDA_TRY(cudaStreamSynchronize(st));
    res->scf_iters = scf;
    res->converged = error < prm->tol_scf ? 1 : 0;
    res->Etot = Etot; res->Eband = Eband; res->E1 = E1; res->E2 = E2; res->E3 = E3;
    res->Exc = Exc; res->Esc = prm->Esc; res->Entropy = Entropy; res->Efermi = efermi;
    res->scf_error = error;
    res->fp64_switch_iter = switch_iter;
    res->filter_ms = filter_ms;
    res->time_s = t_scf;
    return kernel_status_check(ctx);
}

}  // extern "C"
