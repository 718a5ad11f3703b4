// Autotuner for the FP32 filter kernels: times each tile / register-blocking variant of the
// fused stencil + Chebyshev update, and each form of the nonlocal apply (per point over all
// column blocks, alpha rows staged per chunk of covered points, per point with its Chi
// values hoisted out of the column loop, or, in FP32, a dense product per chunk or the range
// form with the output tile in shared memory), and each
// form of the FP32 projection (per image
// segment, or per range of consecutive covered points), on scratch blocks of the
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
        // a variant whose bounded copy waits ran out is never chosen (its time reads as 1e30)
        int kst = 0;
        if (kernel_status_check(ctx, &kst) != SGPU_OK) tmin = 1e30f;
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
            for (int v = 0; v < 5 && rc == SGPU_OK; v++) {
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
                if (rc == SGPU_OK) ctx->tune_apply_ms[v] = tmin;
                if (rc == SGPU_OK && tmin < tbest) { tbest = tmin; abest = v; }
            }
            ctx->nl_apply_variant = rc == SGPU_OK ? abest : saved_a;
            // FP32 projection: per image segment vs per range of covered points
            const int saved_p = ctx->nl_project_variant;
            float pbest = 1e30f;
            int pv = saved_p;
            for (int v = 0; v < 2 && rc == SGPU_OK; v++) {
                ctx->nl_project_variant = v;
                float t = 0.f, tmin = 1e30f;
                for (int rep = 0; rep < 3 && rc == SGPU_OK; rep++) {
                    if (cudaEventRecord(ctx->ev0, st) != cudaSuccess) { rc = SGPU_ERR_CUDA; break; }
                    if ((rc = launch_nonlocal_project<float>(ctx, ncol, X, Nd, alpha, lda, st)) !=
                        SGPU_OK)
                        break;
                    if (cudaEventRecord(ctx->ev1, st) != cudaSuccess ||
                        cudaEventSynchronize(ctx->ev1) != cudaSuccess ||
                        cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1) != cudaSuccess) {
                        rc = SGPU_ERR_CUDA;
                        break;
                    }
                    if (rep > 0) tmin = std::min(tmin, t);  // the first is a warm-up
                }
                if (rc == SGPU_OK) ctx->tune_project_ms[v] = tmin;
                if (rc == SGPU_OK && tmin < pbest) { pbest = tmin; pv = v; }
            }
            ctx->nl_project_variant = rc == SGPU_OK ? pv : saved_p;
            // the range apply with the next degree's projection fused: the FP32 filter uses it
            // when one fused launch beats the fastest apply plus the fastest projection
            ctx->nl_fuse = false;
            ctx->tune_fused_ms = 0.0;
            float *anext = nullptr;
            const size_t abytes = sizeof(float) * (size_t)ctx->nl.ntot * lda;
            if (rc == SGPU_OK && ctx->nl.nrange > 0) {
                if (cudaMallocAsync(&anext, abytes, st) != cudaSuccess) rc = SGPU_ERR_CUDA;
                float fbest = 1e30f;
                int cbest = 2;
                ctx->tune_fused_tc_ms = 0.0;
                // the CUDA-core kernel with 2 and 4 columns per lane, and the tensor-core kernel
                for (int cpl : {2, 4, 3}) {
                    if (rc != SGPU_OK) break;
                    if (cpl == 3 && !nonlocal_tc_ready(ctx)) continue;
                    ctx->nl_fuse_cpl = cpl;
                    float t = 0.f, tmin = 1e30f;
                    for (int rep = 0; rep < 3 && rc == SGPU_OK; rep++) {
                        if (cudaEventRecord(ctx->ev0, st) != cudaSuccess ||
                            cudaMemsetAsync(anext, 0, abytes, st) != cudaSuccess) {
                            rc = SGPU_ERR_CUDA;
                            break;
                        }
                        if ((rc = launch_nonlocal_apply_project(ctx, ncol, alpha, lda, 1.0, Y,
                                                                Nd, anext, st)) != SGPU_OK)
                            break;
                        if (cudaEventRecord(ctx->ev1, st) != cudaSuccess ||
                            cudaEventSynchronize(ctx->ev1) != cudaSuccess ||
                            cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1) != cudaSuccess) {
                            rc = SGPU_ERR_CUDA;
                            break;
                        }
                        if (rep > 0) tmin = std::min(tmin, t);  // the first is a warm-up
                    }
                    if (rc == SGPU_OK) {
                        if (cpl == 3)
                            ctx->tune_fused_tc_ms = tmin;
                        else
                            ctx->tune_fused_cpl_ms[cpl / 2 - 1] = tmin;
                    }
                    if (rc == SGPU_OK && tmin < fbest) { fbest = tmin; cbest = cpl; }
                }
                ctx->nl_fuse_cpl = cbest;
                if (rc == SGPU_OK) {
                    ctx->tune_fused_ms = fbest;
                    ctx->nl_fuse = fbest < ctx->tune_apply_ms[ctx->nl_apply_variant] +
                                               ctx->tune_project_ms[ctx->nl_project_variant];
                }
                if (anext) cudaFreeAsync(anext, st);
            }
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
        set_error("sgpu_set_stencil_variant: variant must be 0.." +
                  std::to_string(kStencilVariants - 1));
        return SGPU_ERR_ARG;
    }
    ctx->stencil_variant = variant;
    ctx->stencil_tuned = true;
    return SGPU_OK;
}

int sgpu_set_nonlocal_apply_variant(sgpu_ctx *ctx, int variant)
{
    if (!ctx || variant < 0 || variant > 4) {
        set_error("sgpu_set_nonlocal_apply_variant: variant must be 0 .. 4");
        return SGPU_ERR_ARG;
    }
    ctx->nl_apply_variant = variant;
    return SGPU_OK;
}

int sgpu_set_nonlocal_project_variant(sgpu_ctx *ctx, int variant)
{
    if (!ctx || variant < 0 || variant > 1) {
        set_error("sgpu_set_nonlocal_project_variant: variant must be 0 or 1");
        return SGPU_ERR_ARG;
    }
    ctx->nl_project_variant = variant;
    return SGPU_OK;
}

int sgpu_set_gemm_emulation(sgpu_ctx *ctx, int mode)
{
    if (!ctx || mode < 0 || mode > 2) {
        set_error("sgpu_set_gemm_emulation: need a context and mode 0, 1 or 2");
        return SGPU_ERR_ARG;
    }
    ctx->gemm_mode = mode;
    if (ctx->cublas &&
        cublasSetEmulationStrategy(ctx->cublas, mode == 1 ? CUBLAS_EMULATION_STRATEGY_EAGER
                                                          : CUBLAS_EMULATION_STRATEGY_PERFORMANT) !=
            CUBLAS_STATUS_SUCCESS) {
        set_error("sgpu_set_gemm_emulation: cublasSetEmulationStrategy failed");
        return SGPU_ERR_CUDA;
    }
    return SGPU_OK;
}

int sgpu_set_eig_solver(sgpu_ctx *ctx, int mode)
{
    if (!ctx || mode < 0 || mode > 2) {
        set_error("sgpu_set_eig_solver: need a context and mode 0, 1 or 2");
        return SGPU_ERR_ARG;
    }
    ctx->eig_mode = mode;
    return SGPU_OK;
}

int sgpu_set_rr_products(sgpu_ctx *ctx, int mode)
{
    if (!ctx || mode < 0 || mode > 2) {
        set_error("sgpu_set_rr_products: need a context and mode 0, 1 or 2");
        return SGPU_ERR_ARG;
    }
    ctx->rr_tc = mode;
    return SGPU_OK;
}

int sgpu_set_rr_batched(sgpu_ctx *ctx, int on)
{
    if (!ctx || (on != 0 && on != 1)) {
        set_error("sgpu_set_rr_batched: need a context and 0 or 1");
        return SGPU_ERR_ARG;
    }
    ctx->rr_batched = on;
    return SGPU_OK;
}

int sgpu_set_zstencil_pairs(sgpu_ctx *ctx, int on)
{
    if (!ctx || (on != 0 && on != 1)) {
        set_error("sgpu_set_zstencil_pairs: need a context and 0 or 1");
        return SGPU_ERR_ARG;
    }
    ctx->zpair_on = on;
    return SGPU_OK;
}

int sgpu_set_nonlocal_fuse(sgpu_ctx *ctx, int mode)
{
    if (!ctx || mode < 0 || mode > 4) {
        set_error("sgpu_set_nonlocal_fuse: need a context and mode 0, 1, 2, 3 or 4");
        return SGPU_ERR_ARG;
    }
    if (mode == 3 && !sgpu::nonlocal_tc_ready(ctx)) {
        set_error("sgpu_set_nonlocal_fuse: no tensor-core range tables for this projector set "
                  "(a covered point needs more than 64 projector rows, or none is set)");
        return SGPU_ERR_STATE;
    }
    ctx->nl_fuse = mode != 0;
    if (mode >= 2) ctx->nl_fuse_cpl = mode;
    return SGPU_OK;
}

int sgpu_get_nonlocal_fuse_tc(sgpu_ctx *ctx, int *available, double *tc_ms)
{
    if (!ctx) {
        set_error("sgpu_get_nonlocal_fuse_tc: null context");
        return SGPU_ERR_ARG;
    }
    if (available) *available = sgpu::nonlocal_tc_ready(ctx) ? 1 : 0;
    if (tc_ms) *tc_ms = ctx->tune_fused_tc_ms;
    return SGPU_OK;
}

int sgpu_get_nonlocal_fuse(sgpu_ctx *ctx, int *mode, double *fused_ms)
{
    if (!ctx) {
        set_error("sgpu_get_nonlocal_fuse: null context");
        return SGPU_ERR_ARG;
    }
    if (mode) *mode = filter_fuses_projection(ctx) ? ctx->nl_fuse_cpl : 0;
    if (fused_ms) {
        fused_ms[0] = ctx->tune_fused_cpl_ms[0];
        fused_ms[1] = ctx->tune_fused_cpl_ms[1];
    }
    return SGPU_OK;
}

int sgpu_get_tuning(sgpu_ctx *ctx, double *apply_ms, double *project_ms)
{
    if (!ctx) {
        set_error("sgpu_get_tuning: null context");
        return SGPU_ERR_ARG;
    }
    for (int v = 0; v < 5 && apply_ms; v++) apply_ms[v] = ctx->tune_apply_ms[v];
    for (int v = 0; v < 2 && project_ms; v++) project_ms[v] = ctx->tune_project_ms[v];
    return SGPU_OK;
}

int sgpu_get_variants(sgpu_ctx *ctx, int *stencil, int *nl_apply, int *nl_project)
{
    if (!ctx) {
        set_error("sgpu_get_variants: null context");
        return SGPU_ERR_ARG;
    }
    if (stencil) *stencil = ctx->stencil_variant;
    if (nl_apply) *nl_apply = ctx->nl_apply_variant;
    if (nl_project) *nl_project = ctx->nl_project_variant;
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
