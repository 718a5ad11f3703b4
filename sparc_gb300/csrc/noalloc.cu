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
//  * the first call on a device looks up the scratch array's device address on that device
//    (cudaGetSymbolAddress, with that device current) and caches it; make that first call
//    before any stream capture;
//  * all calls share the one array and each call clears it before use: calls whose work
//    overlaps on the GPU (different streams, threads or contexts of the same device) race
//    on it and must be serialised by the caller.
#include <mutex>

#include "sgpu_internal.h"

namespace {

constexpr long kNoallocScratchDoubles = 1L << 20;  // 8 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoallocScratchDoubles];

std::mutex g_noalloc_mutex;
double *g_noalloc_ptr[kMaxDevices] = {nullptr};

// device address of the scratch array on the current device (looked up once per device)
int noalloc_scratch(int device, double **out)
{
    if (device < 0 || device >= kMaxDevices) {
        sgpu::set_error("Vnl_vec_mult_noalloc: device ordinal out of range");
        return SGPU_ERR_ARG;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
        double *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            sgpu::set_error(std::string("Vnl_vec_mult_noalloc: cudaGetSymbolAddress: ") +
                            cudaGetErrorString(e));
            return SGPU_ERR_CUDA;
        }
        g_noalloc_ptr[device] = p;
    }
    *out = g_noalloc_ptr[device];
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
    SGPU_TRY(noalloc_scratch(ctx->device, &alpha));
    // the array keeps the previous call's contents: clear the part this call accumulates into
    SGPU_CUDA_TRY(cudaMemsetAsync(alpha, 0, sizeof(double) * (size_t)need, ctx->stream));
    SGPU_TRY(launch_nonlocal_project<double>(ctx, ncol, x, ldi, alpha, lda, ctx->stream));
    SGPU_TRY(launch_nonlocal_apply<double>(ctx, ncol, alpha, lda, 1.0, Hx, ldo, ctx->stream));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}
