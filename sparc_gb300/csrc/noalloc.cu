// Nonlocal apply for callers that cannot allocate device memory.
//
// sgpu_Vnl_vec_mult keeps its projection coefficients (alpha, n_proj x ncol) in a grow-only
// workspace that it enlarges with cudaMalloc / cudaFree on demand. Some callers cannot let the
// library do that: a host application that hands all of the GPU's memory to its own pool
// allocator up front leaves nothing for cudaMalloc to return, and a caller that overlaps this
// call with other work on other streams cannot accept cudaFree, which synchronises the whole
// device. sgpu_Vnl_vec_mult_noalloc serves them: the same kernels, with alpha in a fixed
// scratch array that lives in this library's own device image (every GPU that loads the
// library holds it until the process exits), so the call itself allocates nothing.
//
// Limits and rules:
//  * scratch holds kNoallocScratchDoubles doubles (8 MiB): n_proj * round_up(ncol, 8) must fit,
//    larger requests are rejected with SGPU_ERR_ARG before anything is launched;
//  * x and Hx must be device pointers (staging host arrays would need device buffers);
//  * the first call in a CUDA context looks up the scratch array's device address in that
//    context (cudaGetSymbolAddress, with the context's device current) and caches it under the
//    context's unique id; make that first call before any stream capture. Each context holds
//    its own copy of the array (a context loads its own copy of the library's device image),
//    and a context created after cudaDeviceReset gets a new id, so no stale address is used;
//  * all calls in one context share its array and each call clears it before use: calls whose
//    work overlaps on the GPU (different streams or threads using the same context) race on
//    it and must be serialised by the caller.
#include <mutex>

#include "sgpu_internal.h"

namespace {

constexpr long kNoallocScratchDoubles = 1L << 20;  // 8 MiB

static __device__ __align__(256) double g_noalloc_scratch[kNoallocScratchDoubles];

std::mutex g_noalloc_mutex;

// driver entry points, resolved through the runtime (the library does not link libcuda)
typedef int (*ctx_get_current_fn)(void **ctx);
typedef int (*ctx_get_id_fn)(void *ctx, unsigned long long *id);
ctx_get_current_fn g_ctx_get_current = nullptr;
ctx_get_id_fn g_ctx_get_id = nullptr;

struct ScratchEntry {
    unsigned long long ctx_id;
    double *ptr;
};
constexpr int kCacheSlots = 64;
ScratchEntry g_noalloc_cache[kCacheSlots];
int g_noalloc_cached = 0;
int g_noalloc_next = 0;  // slot replaced next once the table is full

// unique id of the CUDA context current on this thread (call with g_noalloc_mutex held)
int current_context_id(unsigned long long *id)
{
    if (!g_ctx_get_current || !g_ctx_get_id) {
        void *f1 = nullptr, *f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000,
                                                          cudaEnableDefault, &q1);
        cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000,
                                                          cudaEnableDefault, &q2);
        if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
            q2 != cudaDriverEntryPointSuccess || !f1 || !f2) {
            sgpu::set_error("Vnl_vec_mult_noalloc: cannot resolve cuCtxGetCurrent/cuCtxGetId");
            return SGPU_ERR_CUDA;
        }
        g_ctx_get_current = (ctx_get_current_fn)f1;
        g_ctx_get_id = (ctx_get_id_fn)f2;
    }
    void *cu_ctx = nullptr;
    if (g_ctx_get_current(&cu_ctx) != 0 || !cu_ctx || g_ctx_get_id(cu_ctx, id) != 0) {
        sgpu::set_error("Vnl_vec_mult_noalloc: no current CUDA context");
        return SGPU_ERR_CUDA;
    }
    return SGPU_OK;
}

// device address of the scratch array in the current context (looked up once per context)
int noalloc_scratch(double **out)
{
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    unsigned long long id = 0;
    SGPU_TRY(current_context_id(&id));
    for (int i = 0; i < g_noalloc_cached; ++i)
        if (g_noalloc_cache[i].ctx_id == id) {
            *out = g_noalloc_cache[i].ptr;
            return SGPU_OK;
        }
    double *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
        sgpu::set_error(std::string("Vnl_vec_mult_noalloc: cudaGetSymbolAddress: ") +
                        cudaGetErrorString(e));
        return SGPU_ERR_CUDA;
    }
    int slot = g_noalloc_cached < kCacheSlots ? g_noalloc_cached++ : g_noalloc_next;
    if (slot == g_noalloc_next && g_noalloc_cached == kCacheSlots)
        g_noalloc_next = (g_noalloc_next + 1) % kCacheSlots;
    g_noalloc_cache[slot] = {id, p};
    *out = p;
    return SGPU_OK;
}

}  // namespace

using namespace sgpu;

extern "C" int sgpu_Vnl_vec_mult_noalloc(sgpu_ctx *ctx, int ncol, const double *x, int ldi,
                                         double *Hx, int ldo)
{
    if (!ctx) {
        set_error("Vnl_vec_mult_noalloc: null context");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    if (ncol < 0 || ldi < ctx->Nd || ldo < ctx->Nd) {
        set_error("Vnl_vec_mult_noalloc: need ncol >= 0 and leading dimensions >= Nd");
        return SGPU_ERR_ARG;
    }
    if (ncol == 0 || !ctx->has_nl || ctx->nl.ntot == 0) return SGPU_OK;
    if (!is_device_ptr(x) || !is_device_ptr(Hx)) {
        set_error("Vnl_vec_mult_noalloc: x and Hx must be device pointers");
        return SGPU_ERR_ARG;
    }
    const long lda = nonlocal_alpha_ld(ncol, (int)sizeof(double));
    const long need = (long)ctx->nl.ntot * lda;
    if (need > kNoallocScratchDoubles) {
        set_error("Vnl_vec_mult_noalloc: n_proj * round_up(ncol, 8) = " + std::to_string(need) +
                  " exceeds the fixed scratch of " + std::to_string(kNoallocScratchDoubles) +
                  " doubles; use fewer columns per call");
        return SGPU_ERR_ARG;
    }
    double *alpha = nullptr;
    SGPU_TRY(noalloc_scratch(&alpha));
    // the array keeps the previous call's contents: clear the part this call accumulates into
    SGPU_CUDA_TRY(cudaMemsetAsync(alpha, 0, sizeof(double) * (size_t)need, ctx->stream));
    SGPU_TRY(launch_nonlocal_project<double>(ctx, ncol, x, ldi, alpha, lda, ctx->stream));
    SGPU_TRY(launch_nonlocal_apply<double>(ctx, ncol, alpha, lda, 1.0, Hx, ldo, ctx->stream));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}
