// Hamiltonian apply and Chebyshev filter on device-resident blocks.
//
// Hamiltonian_vectors_mult (src/hamiltonianVecRoutines.c:45-121) becomes three launches on
// the context stream: nonlocal projection (alpha = dV * Gamma * Chiᵀ x), the fused stencil
// (-0.5*Lap + Veff + c, scaled, plus the optional Chebyshev term), and the owner-computes
// nonlocal apply into the same output.
//
// ChebyshevFiltering (src/eigenSolver.c:722-798) keeps the reference's scalar recurrence
// (e, c, sigma, sigma1, gamma, sigma2, vscal, vscal2) but writes each new iterate in place
// over the oldest one (its last reader is the thread that writes it), so the filter needs at
// most one scratch block and no separate scale/axpy/swap pass.
#include <utility>

#include "sgpu_internal.h"

namespace sgpu {

template <typename T>
static const T *veff_of(sgpu_ctx *ctx, int spin);
template <>
const double *veff_of<double>(sgpu_ctx *ctx, int spin)
{
    return ctx->veff64 ? ctx->veff64 + (long)spin * ctx->Nd : nullptr;
}
template <>
const float *veff_of<float>(sgpu_ctx *ctx, int spin)
{
    return ctx->veff32 ? ctx->veff32 + (long)spin * ctx->Nd : nullptr;
}

// alpha_in (optional): dV * Gamma * Chiᵀ x already formed (ld nonlocal_alpha_ld), so no
// projection is launched; alpha_out (optional, FP32 with alpha_in): receives dV * Gamma * Chiᵀ
// of the finished hx from the fused range apply, for the next filter degree.
template <typename T>
int hamiltonian_dev(sgpu_ctx *ctx, int spin, int ncol, double c, const T *x, long ldx, T *hx,
                    long ldh, double s1, double s2, const T *z, long ldz, cudaStream_t st,
                    const T *alpha_in, T *alpha_out)
{
    if (spin < 0 || spin >= ctx->nspin_veff) {
        set_error("Hamiltonian: no local potential set for this spin block");
        return SGPU_ERR_STATE;
    }
    const T *alpha = alpha_in;
    const long lda = nonlocal_alpha_ld(ncol, (int)sizeof(T));
    const size_t abytes = ctx->has_nl ? sizeof(T) * (size_t)ctx->nl.ntot * lda : 0;
    if (!alpha && ctx->has_nl && ctx->nl.ntot > 0) {
        T *a = nullptr;
        SGPU_TRY(ws_get(ctx, WS_ALPHA, abytes, (void **)&a));
        SGPU_CUDA_TRY(cudaMemsetAsync(a, 0, abytes, st));
        SGPU_TRY(launch_nonlocal_project<T>(ctx, ncol, x, ldx, a, lda, st));
        alpha = a;
    }
    SGPU_TRY(launch_stencil<T>(ctx, ncol, -0.5, 1.0, c, veff_of<T>(ctx, spin), x, ldx, hx, ldh,
                               s1, s2, z, ldz, st));
    if (!alpha) return SGPU_OK;
    if constexpr (sizeof(T) == 4) {
        if (alpha_out) {
            SGPU_CUDA_TRY(cudaMemsetAsync(alpha_out, 0, abytes, st));
            return launch_nonlocal_apply_project(ctx, ncol, alpha, lda, s1, hx, ldh, alpha_out,
                                                 st);
        }
    }
    return launch_nonlocal_apply<T>(ctx, ncol, alpha, lda, s1, hx, ldh, st);
}

bool filter_fuses_projection(sgpu_ctx *ctx)
{
    return ctx->nl_fuse && ctx->has_nl && ctx->nl.ntot > 0 && ctx->nl.nrange > 0;
}

// The FP32 filter's projection buffers when the projections are carried across degrees:
// A = dV * Gamma * Chiᵀ X (one projection launch), B the buffer the fused applies alternate
// with. Both null when the filter does not fuse.
static int carried_alpha(sgpu_ctx *ctx, int ncol, const float *X, long ldx, float **A, float **B,
                         cudaStream_t st)
{
    *A = *B = nullptr;
    if (!filter_fuses_projection(ctx)) return SGPU_OK;
    const long lda = nonlocal_alpha_ld(ncol, 4);
    const size_t bytes = sizeof(float) * (size_t)ctx->nl.ntot * lda;
    SGPU_TRY(ws_get(ctx, WS_ALPHA, bytes, (void **)A));
    SGPU_TRY(ws_get(ctx, WS_ALPHA2, bytes, (void **)B));
    SGPU_CUDA_TRY(cudaMemsetAsync(*A, 0, bytes, st));
    return launch_nonlocal_project<float>(ctx, ncol, X, ldx, *A, lda, st);
}

// On return the filtered block is in Y and the degree m-1 iterate in X, as in the reference.
// Each new iterate is written in place over the oldest one, so iterate j lands in X's buffer
// for odd j when the first output goes to Y. When m-1 is odd that would leave the result in
// X, so the first two iterates are routed through one scratch block instead (step 0 into W,
// step 1 into Y, step 2 into X) and the parities line up with no extra pass.
template <typename T>
int chebyshev_dev(sgpu_ctx *ctx, int spin, T *X, long ldx, T *Y, long ldy, int ncol, int m,
                  double a, double b, double a0, cudaStream_t st)
{
    if (m < 1) {
        set_error("ChebyshevFiltering: degree must be >= 1");
        return SGPU_ERR_ARG;
    }
    const double e = 0.5 * (b - a);
    const double c = 0.5 * (b + a);
    double sigma = e / (a0 - c);
    const double sigma1 = sigma;
    const double gamma = 2.0 / sigma1;
    const long Nd = ctx->Nd;

    T *W = nullptr;
    const bool route = ((m - 1) % 2) == 1;
    if (route) SGPU_TRY(ws_get(ctx, WS_STAGE_C, sizeof(T) * (size_t)Nd * ncol, (void **)&W));

    // FP32 with the fused range apply: each degree's apply also projects its finished output
    // for the next degree, alternating between two projection buffers
    T *acur = nullptr, *anext = nullptr;
    if constexpr (sizeof(T) == 4) SGPU_TRY(carried_alpha(ctx, ncol, X, ldx, &acur, &anext, st));

    // Y_0 = (sigma1/e) (H - c I) X
    T *y0 = route ? W : Y;
    long ly0 = route ? Nd : ldy;
    SGPU_TRY(hamiltonian_dev<T>(ctx, spin, ncol, -c, X, ldx, y0, ly0, sigma1 / e, 0.0, nullptr,
                                0, st, acur, m > 1 ? anext : nullptr));
    std::swap(acur, anext);
    // (cur, prev) = (Y_j, Y_{j-1}) with Y_{-1} = X
    T *cur = y0, *prev = X;
    long ldc = ly0, ldp = ldx;
    for (int j = 1; j < m; j++) {
        const double sigma2 = 1.0 / (gamma - sigma);
        const double vscal = 2.0 * sigma2 / e;
        const double vscal2 = sigma * sigma2;
        // Y_j = vscal (H - c I) Y_{j-1} - vscal2 Y_{j-2}
        T *dst = prev;
        long ldd = ldp;
        if (route && j == 1) { dst = Y; ldd = ldy; }
        if (route && j == 2) { dst = X; ldd = ldx; }
        SGPU_TRY(hamiltonian_dev<T>(ctx, spin, ncol, -c, cur, ldc, dst, ldd, vscal, -vscal2,
                                    prev, ldp, st, acur, j + 1 < m ? anext : nullptr));
        std::swap(acur, anext);
        prev = cur; ldp = ldc;
        cur = dst; ldc = ldd;
        sigma = sigma2;
    }
    if (route && m == 2) {  // the degree-1 iterate is still in the scratch block
        SGPU_CUDA_TRY(cudaMemcpy2DAsync(X, sizeof(T) * ldx, W, sizeof(T) * Nd, sizeof(T) * Nd,
                                        ncol, cudaMemcpyDeviceToDevice, st));
    }
    return SGPU_OK;
}

// Precision-graded filter: degrees 0 .. m-k64-1 in FP32 on (X32, Y32), the last k64 degrees
// in FP64, the filtered block landing in Y64 (X64 gets the previous iterate). A rounding error
// made at degree j is multiplied by the remaining m-1-j degrees of the filter like any other
// component: its part outside the wanted subspace is damped and its part inside is harmless
// to the Rayleigh-Ritz step, so only the last degrees need FP64 for an FP64-quality subspace.
// k64 == 0 gives a pure FP32 filter whose result is widened into Y64. All blocks have ld Nd.
int chebyshev_graded(sgpu_ctx *ctx, int spin, float *X32, float *Y32, double *X64,
                     double *Y64, int ncol, int m, int k64, double a, double b, double a0,
                     cudaStream_t st)
{
    if (m < 1 || k64 < 0 || k64 >= m) {
        set_error("ChebyshevFiltering (graded): need 0 <= FP64 degrees < m");
        return SGPU_ERR_ARG;
    }
    const long Nd = ctx->Nd;
    const double e = 0.5 * (b - a);
    const double c = 0.5 * (b + a);
    double sigma = e / (a0 - c);
    const double sigma1 = sigma;
    const double gamma = 2.0 / sigma1;
    const int m32 = m - k64;
    float *acur = nullptr, *anext = nullptr;  // carried projections (fused range apply)
    SGPU_TRY(carried_alpha(ctx, ncol, X32, Nd, &acur, &anext, st));
    SGPU_TRY(hamiltonian_dev<float>(ctx, spin, ncol, -c, X32, Nd, Y32, Nd, sigma1 / e, 0.0,
                                    nullptr, 0, st, acur, m32 > 1 ? anext : nullptr));
    std::swap(acur, anext);
    float *cur = Y32, *prev = X32;
    for (int j = 1; j < m32; j++) {
        const double sigma2 = 1.0 / (gamma - sigma);
        SGPU_TRY(hamiltonian_dev<float>(ctx, spin, ncol, -c, cur, Nd, prev, Nd,
                                        2.0 * sigma2 / e, -sigma * sigma2, prev, Nd, st, acur,
                                        j + 1 < m32 ? anext : nullptr));
        std::swap(acur, anext);
        std::swap(cur, prev);
        sigma = sigma2;
    }
    // widen; the first FP64 step writes over the widened previous iterate, so put that one
    // where the final iterate must end (Y64) when k64 is odd
    double *A = (k64 % 2 == 1) ? X64 : Y64, *B = (k64 % 2 == 1) ? Y64 : X64;
    SGPU_TRY(convert_cols<float, double>(cur, Nd, A, Nd, Nd, ncol, st));
    SGPU_TRY(convert_cols<float, double>(prev, Nd, B, Nd, Nd, ncol, st));
    double *cur64 = A, *prev64 = B;
    for (int j = m32; j < m; j++) {
        const double sigma2 = 1.0 / (gamma - sigma);
        SGPU_TRY(hamiltonian_dev<double>(ctx, spin, ncol, -c, cur64, Nd, prev64, Nd,
                                         2.0 * sigma2 / e, -sigma * sigma2, prev64, Nd, st));
        std::swap(cur64, prev64);
        sigma = sigma2;
    }
    return SGPU_OK;
}

template int hamiltonian_dev<double>(sgpu_ctx *, int, int, double, const double *, long,
                                     double *, long, double, double, const double *, long,
                                     cudaStream_t, const double *, double *);
template int hamiltonian_dev<float>(sgpu_ctx *, int, int, double, const float *, long, float *,
                                    long, double, double, const float *, long, cudaStream_t,
                                    const float *, float *);
template int chebyshev_dev<double>(sgpu_ctx *, int, double *, long, double *, long, int, int,
                                   double, double, double, cudaStream_t);
template int chebyshev_dev<float>(sgpu_ctx *, int, float *, long, float *, long, int, int,
                                  double, double, double, cudaStream_t);

}  // namespace sgpu
