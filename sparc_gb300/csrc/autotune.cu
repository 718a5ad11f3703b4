// Autotuner for the FP32 filter kernels: times each tile / register-blocking variant of the
// fused stencil + Chebyshev update, and each form of the nonlocal apply (per point over all
// column blocks, alpha rows staged per chunk of covered points, or per point with its Chi
// values hoisted out of the column loop), on scratch blocks of the
// context's grid and projector set, and keeps the fastest of each. The stencil variants
// compute the same IEEE operation sequence per point, and so do the two apply forms, so the
// choice changes speed only, never results.
#include <vector>

#include "sgpu_internal.h"

namespace sgpu {

constexpr int kStencilVariants = SGPU_STENCIL_VARIANTS;

// Times one degree-step launch (stencil + potential + recurrence term) of each FP32 variant
// over ncol columns; returns the fastest in *best and per-variant milliseconds in ms.
static int tune_stencil(sgpu_ctx *ctx, int ncol, int *best, double *ms)
{
    cudaStream_t st = ctx->stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    SGPU_CUDA_TRY(cudaStreamIsCapturing(st, &cap));
    if (cap != cudaStreamCaptureStatusNone) {
        set_error("autotune: cannot time kernels while the stream is being captured");
        return SGPU_ERR_STATE;
    }
    const long Nd = ctx->Nd;
    float *buf = nullptr;
    SGPU_CUDA_TRY(cudaMallocAsync(&buf, sizeof(float) * (size_t)Nd * ncol * 2, st));
    float *X = buf, *Y = buf + (size_t)Nd * ncol;
    int rc = SGPU_OK;
    if (cudaMemsetAsync(buf, 0, sizeof(float) * (size_t)Nd * ncol * 2, st) != cudaSuccess)
        rc = SGPU_ERR_CUDA;
    const int saved = ctx->stencil_variant;
    const bool prof = ctx->prof_on;
    ctx->prof_on = false;
    double best_ms = 1e300;
    *best = saved;
    for (int v = 0; v < kStencilVariants && rc == SGPU_OK; v++) {
        ctx->stencil_variant = v;
        auto step = [&]() {
            return launch_stencil<float>(ctx, ncol, -0.5, 1.0, 0.25, ctx->veff32, X, Nd, Y, Nd,
                                         0.9, -0.4, X, Nd, st);
        };
        if ((rc = step()) != SGPU_OK) break;  // warm-up
        float t = 0.f, tmin = 1e30f;
        for (int rep = 0; rep < 3 && rc == SGPU_OK; rep++) {
            if (cudaEventRecord(ctx->ev0, st) != cudaSuccess) { rc = SGPU_ERR_CUDA; break; }
            if ((rc = step()) != SGPU_OK) break;
            if (cudaEventRecord(ctx->ev1, st) != cudaSuccess ||
                cudaEventSynchronize(ctx->ev1) != cudaSuccess ||
                cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1) != cudaSuccess) {
                rc = SGPU_ERR_CUDA;
                break;
            }
            tmin = std::min(tmin, t);
        }
        if (rc != SGPU_OK) break;
        if (ms) ms[v] = tmin;
        if (tmin < best_ms) { best_ms = tmin; *best = v; }
    }
    ctx->stencil_variant = rc == SGPU_OK ? *best : saved;
    // nonlocal apply: per-point form, alpha rows staged per chunk, Chi hoisted per point
    if (rc == SGPU_OK && ctx->has_nl && ctx->nl.ntot > 0 && ctx->nl.ncov > 0) {
        const long lda = nonlocal_alpha_ld(ncol, 4);
        float *alpha = nullptr;
        if (cudaMallocAsync(&alpha, sizeof(float) * (size_t)ctx->nl.ntot * lda, st) != cudaSuccess ||
            cudaMemsetAsync(alpha, 0, sizeof(float) * (size_t)ctx->nl.ntot * lda, st) != cudaSuccess) {
            rc = SGPU_ERR_CUDA;
        } else {
            const int saved_a = ctx->nl_apply_variant;
            float tbest = 1e30f;
            int abest = saved_a;
            for (int v = 0; v < 3 && rc == SGPU_OK; v++) {
                ctx->nl_apply_variant = v;
                float t = 0.f, tmin = 1e30f;
                for (int rep = 0; rep < 3 && rc == SGPU_OK; rep++) {
                    if (cudaEventRecord(ctx->ev0, st) != cudaSuccess) { rc = SGPU_ERR_CUDA; break; }
                    if ((rc = launch_nonlocal_apply<float>(ctx, ncol, alpha, lda, 1.0, Y, Nd,
                                                           st)) != SGPU_OK)
                        break;
                    if (cudaEventRecord(ctx->ev1, st) != cudaSuccess ||
                        cudaEventSynchronize(ctx->ev1) != cudaSuccess ||
                        cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1) != cudaSuccess) {
                        rc = SGPU_ERR_CUDA;
                        break;
                    }
                    if (rep > 0) tmin = std::min(tmin, t);  // the first is a warm-up
                }
                if (rc == SGPU_OK && tmin < tbest) { tbest = tmin; abest = v; }
            }
            ctx->nl_apply_variant = rc == SGPU_OK ? abest : saved_a;
            cudaFreeAsync(alpha, st);
        }
    }
    ctx->prof_on = prof;
    cudaFreeAsync(buf, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == SGPU_OK) rc = SGPU_ERR_CUDA;
    if (rc == SGPU_ERR_CUDA) set_error("autotune: CUDA error while timing stencil variants");
    return rc;
}

}  // namespace sgpu

using namespace sgpu;

extern "C" {

int sgpu_set_stencil_variant(sgpu_ctx *ctx, int variant)
{
    if (!ctx || variant < 0 || variant >= kStencilVariants) {
        set_error("sgpu_set_stencil_variant: variant must be 0..6");
        return SGPU_ERR_ARG;
    }
    ctx->stencil_variant = variant;
    ctx->stencil_tuned = true;
    return SGPU_OK;
}

int sgpu_set_nonlocal_apply_variant(sgpu_ctx *ctx, int variant)
{
    if (!ctx || variant < 0 || variant > 2) {
        set_error("sgpu_set_nonlocal_apply_variant: variant must be 0, 1 or 2");
        return SGPU_ERR_ARG;
    }
    ctx->nl_apply_variant = variant;
    return SGPU_OK;
}

int sgpu_autotune(sgpu_ctx *ctx, int ncol, int *variant, double *ms)
{
    if (!ctx || ncol <= 0) {
        set_error("sgpu_autotune: need a context and ncol > 0");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    int best = 0;
    SGPU_TRY(tune_stencil(ctx, ncol, &best, ms));
    ctx->stencil_tuned = true;
    if (variant) *variant = best;
    return SGPU_OK;
}

}  // extern "C"
