// C ABI entry points (include/sparc_gpu.h): context set-up and the reference-shaped hot-path
// calls, with host-array staging so that the reference's own malloc'ed buffers can be passed.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "sgpu_internal.h"

namespace sgpu {

static thread_local std::string g_err;

void set_error(const std::string &msg) { g_err = msg; }

int ws_get(sgpu_ctx *ctx, int slot, size_t bytes, void **out)
{
    Workspace &w = ctx->ws[slot];
    if (w.bytes < bytes) {
        if (w.ptr) {
            SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
            cudaFree(w.ptr);
            w.ptr = nullptr;
            w.bytes = 0;
        }
        size_t nb = bytes + bytes / 8 + 256;
        cudaError_t e = cudaMalloc(&w.ptr, nb);
        if (e != cudaSuccess) {
            set_error(std::string("device workspace allocation of ") + std::to_string(nb) +
                      " bytes failed: " + cudaGetErrorString(e));
            w.ptr = nullptr;
            return SGPU_ERR_NOMEM;
        }
        w.bytes = nb;
    }
    *out = w.ptr;
    return SGPU_OK;
}

int kernel_status_check(sgpu_ctx *ctx, int *status)
{
    int h = 0;
    SGPU_CUDA_TRY(cudaMemcpyAsync(&h, ctx->kstatus, sizeof(int), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (status) *status = h;
    if (h == 0) return SGPU_OK;
    SGPU_CUDA_TRY(cudaMemsetAsync(ctx->kstatus, 0, sizeof(int), ctx->stream));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    set_error("a kernel's bounded wait on its own copies ran out (status " +
              std::to_string(h) + "); results since the last check are invalid");
    return SGPU_ERR_KERNEL_WAIT;
}

static cudaEvent_t prof_event(sgpu_ctx *ctx)
{
    if (ctx->prof_next >= ctx->prof_pool.size()) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        ctx->prof_pool.push_back(e);
    }
    return ctx->prof_pool[ctx->prof_next++];
}

ProfScope::ProfScope(sgpu_ctx *c, int k, cudaStream_t s) : ctx(c), kind(k), st(s)
{
    ctx->launches++;
    if (ctx->prof_on) {
        b = prof_event(ctx);
        if (b) cudaEventRecord(b, st);
    }
}

ProfScope::~ProfScope()
{
    if (ctx->prof_on && b) {
        cudaEvent_t e = prof_event(ctx);
        if (e) {
            cudaEventRecord(e, st);
            ctx->prof_pending.push_back({kind, b, e});
        }
    }
}

static int prof_resolve(sgpu_ctx *ctx)
{
    if (ctx->prof_pending.empty()) return SGPU_OK;
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    for (auto &r : ctx->prof_pending) {
        float ms = 0.f;
        SGPU_CUDA_TRY(cudaEventElapsedTime(&ms, r.a, r.b));
        ctx->prof_ms[r.kind] += ms;
        ctx->prof_n[r.kind]++;
    }
    ctx->prof_pending.clear();
    ctx->prof_next = 0;
    return SGPU_OK;
}

bool is_device_ptr(const void *p)
{
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Bring a column block to the device: returns a device pointer with leading dimension *ld.
static int stage_in(sgpu_ctx *ctx, int slot, const double *x, int ldi, int ncol, bool copy,
                    double **dptr, long *ld)
{
    if (is_device_ptr(x)) {
        *dptr = const_cast<double *>(x);
        *ld = ldi;
        return SGPU_OK;
    }
    double *d = nullptr;
    SGPU_TRY(ws_get(ctx, slot, sizeof(double) * (size_t)ctx->Nd * (ncol > 0 ? ncol : 1),
                    (void **)&d));
    if (copy && ncol > 0 && x)
        SGPU_CUDA_TRY(cudaMemcpy2DAsync(d, sizeof(double) * ctx->Nd, x, sizeof(double) * ldi,
                                        sizeof(double) * ctx->Nd, ncol, cudaMemcpyHostToDevice,
                                        ctx->stream));
    *dptr = d;
    *ld = ctx->Nd;
    return SGPU_OK;
}

static int stage_out(sgpu_ctx *ctx, const double *dptr, long ld, double *y, int ldo, int ncol)
{
    if (dptr == y || ncol <= 0) return SGPU_OK;
    SGPU_CUDA_TRY(cudaMemcpy2DAsync(y, sizeof(double) * ldo, dptr, sizeof(double) * ld,
                                    sizeof(double) * ctx->Nd, ncol, cudaMemcpyDeviceToHost,
                                    ctx->stream));
    return SGPU_OK;
}

static int check_ctx(sgpu_ctx *ctx)
{
    if (!ctx) {
        set_error("null context");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    return SGPU_OK;
}

static int check_block(sgpu_ctx *ctx, int ncol, int ldi, int ldo)
{
    if (ncol < 0 || ldi < ctx->Nd || ldo < ctx->Nd) {
        set_error("column block: need ncol >= 0 and leading dimensions >= Nd");
        return SGPU_ERR_ARG;
    }
    return SGPU_OK;
}

}  // namespace sgpu

using namespace sgpu;

extern "C" {

const char *sgpu_last_error(void) { return g_err.c_str(); }

int sgpu_version(void) { return 1; }

int sgpu_create(sgpu_ctx **out, int device, int Nx, int Ny, int Nz, int FDn, const double *cx,
                const double *cy, const double *cz, double dV)
{
    if (!out || !cx || !cy || !cz) {
        set_error("sgpu_create: null argument");
        return SGPU_ERR_ARG;
    }
    *out = nullptr;
    if (FDn != kMaxFDn) {
        set_error("sgpu_create: only FD order 12 (FDn = 6) is supported");
        return SGPU_ERR_ARG;
    }
    if (Nx < FDn || Ny < FDn || Nz < FDn || dV <= 0.0) {
        set_error("sgpu_create: each grid dimension must be >= FDn and dV > 0");
        return SGPU_ERR_ARG;
    }
    int ndev = 0;
    SGPU_CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) {
        set_error("sgpu_create: no such CUDA device");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(device));
    sgpu_ctx *ctx = new sgpu_ctx();
    ctx->device = device;
    ctx->Nx = Nx; ctx->Ny = Ny; ctx->Nz = Nz; ctx->FDn = FDn;
    ctx->Nd = (long)Nx * Ny * Nz;
    ctx->dV = dV;
    for (int p = 0; p <= FDn; p++) { ctx->cx[p] = cx[p]; ctx->cy[p] = cy[p]; ctx->cz[p] = cz[p]; }
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->kstatus, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(ctx->kstatus, 0, sizeof(int));
    if (e != cudaSuccess) {
        set_error(std::string("sgpu_create: ") + cudaGetErrorString(e));
        if (ctx->kstatus) cudaFree(ctx->kstatus);
        delete ctx;
        return SGPU_ERR_CUDA;
    }
    *out = ctx;
    return SGPU_OK;
}

int sgpu_set_grid_coeffs(sgpu_ctx *ctx, const double *cx, const double *cy, const double *cz,
                         double dV)
{
    SGPU_TRY(check_ctx(ctx));
    if (!cx || !cy || !cz || !(dV > 0.0)) {
        set_error("sgpu_set_grid_coeffs: null weights or dV <= 0");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    for (int p = 0; p <= ctx->FDn; p++) { ctx->cx[p] = cx[p]; ctx->cy[p] = cy[p]; ctx->cz[p] = cz[p]; }
    ctx->dV = dV;
    return SGPU_OK;
}

int sgpu_destroy(sgpu_ctx *ctx)
{
    if (!ctx) return SGPU_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    nonlocal_free(ctx->nl);
    if (ctx->veff64) cudaFree(ctx->veff64);
    if (ctx->veff32) cudaFree(ctx->veff32);
    for (auto &w : ctx->ws)
        if (w.ptr) cudaFree(w.ptr);
    if (ctx->cublas) cublasDestroy(ctx->cublas);
    if (ctx->cusolver) cusolverDnDestroy(ctx->cusolver);
    if (ctx->xparams) cusolverDnDestroyParams(ctx->xparams);
    free(ctx->xhost);
    for (auto e : ctx->prof_pool) cudaEventDestroy(e);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->kstatus) cudaFree(ctx->kstatus);
    if (ctx->copy_in) cudaStreamSynchronize(ctx->copy_in);
    if (ctx->copy_out) cudaStreamSynchronize(ctx->copy_out);
    for (auto &slot : ctx->pipe_ev)
        for (auto &e : slot)
            if (e) cudaEventDestroy(e);
    if (ctx->copy_in) cudaStreamDestroy(ctx->copy_in);
    if (ctx->copy_out) cudaStreamDestroy(ctx->copy_out);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx->mix;
    kpoint_free(ctx);
    setup_free(ctx);
    delete ctx;
    return SGPU_OK;
}

int sgpu_set_veff(sgpu_ctx *ctx, int nspin, const double *veff)
{
    SGPU_TRY(check_ctx(ctx));
    if (nspin < 1 || !veff) {
        set_error("sgpu_set_veff: need nspin >= 1 and a non-null array");
        return SGPU_ERR_ARG;
    }
    const size_t n = (size_t)ctx->Nd * nspin;
    if (ctx->nspin_veff != nspin) {
        if (ctx->veff64) cudaFree(ctx->veff64);
        if (ctx->veff32) cudaFree(ctx->veff32);
        ctx->veff64 = nullptr;
        ctx->veff32 = nullptr;
        ctx->nspin_veff = 0;
        SGPU_CUDA_TRY(cudaMalloc(&ctx->veff64, n * sizeof(double)));
        SGPU_CUDA_TRY(cudaMalloc(&ctx->veff32, n * sizeof(float)));
        ctx->nspin_veff = nspin;
    }
    SGPU_CUDA_TRY(cudaMemcpyAsync(ctx->veff64, veff, n * sizeof(double), cudaMemcpyDefault,
                                  ctx->stream));
    SGPU_TRY(convert_cols<double, float>(ctx->veff64, (long)n, ctx->veff32, (long)n, (long)n, 1,
                                         ctx->stream));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_set_nonlocal(sgpu_ctx *ctx, int n_atom, const int *IP_displ, const double *Gamma,
                      int n_img, const int *img_atom, const int *img_ndc, const int *grid_pos,
                      const double *Chi)
{
    SGPU_TRY(check_ctx(ctx));
    if (n_atom < 0 || n_img < 0 || (n_atom > 0 && !IP_displ) ||
        (n_img > 0 && (!img_atom || !img_ndc))) {
        set_error("sgpu_set_nonlocal: bad sizes or null arrays");
        return SGPU_ERR_ARG;
    }
    if (n_atom == 0 || n_img == 0) {
        nonlocal_free(ctx->nl);
        ctx->has_nl = false;
        return SGPU_OK;
    }
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return nonlocal_upload(ctx, n_atom, IP_displ, Gamma, n_img, img_atom, img_ndc, grid_pos,
                           Chi);
}

int sgpu_Lap_plus_diag_vec_mult_orth(sgpu_ctx *ctx, int ncol, double a, double b, double c,
                                     const double *v, const double *x, int ldi, double *y,
                                     int ldo)
{
    SGPU_TRY(check_ctx(ctx));
    SGPU_TRY(check_block(ctx, ncol, ldi, ldo));
    if (ncol == 0) return SGPU_OK;
    double *dx, *dy, *dv = nullptr;
    long lx, ly, lv;
    SGPU_TRY(stage_in(ctx, WS_STAGE_A, x, ldi, ncol, true, &dx, &lx));
    SGPU_TRY(stage_in(ctx, WS_STAGE_B, y, ldo, ncol, false, &dy, &ly));
    if (v && !(fabs(b) < 1e-14)) SGPU_TRY(stage_in(ctx, WS_STAGE_C, v, (int)ctx->Nd, 1, true, &dv, &lv));
    SGPU_TRY(launch_stencil<double>(ctx, ncol, a, b, c, dv, dx, lx, dy, ly, 1.0, 0.0, nullptr,
                                    0, ctx->stream));
    SGPU_TRY(stage_out(ctx, dy, ly, y, ldo, ncol));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_Lap_vec_mult(sgpu_ctx *ctx, int ncol, double c, const double *x, int ldi,
                      double *Lapx, int ldo)
{
    return sgpu_Lap_plus_diag_vec_mult_orth(ctx, ncol, 1.0, 0.0, c, nullptr, x, ldi, Lapx, ldo);
}

int sgpu_Vnl_vec_mult(sgpu_ctx *ctx, int ncol, const double *x, int ldi, double *Hx, int ldo)
{
    SGPU_TRY(check_ctx(ctx));
    SGPU_TRY(check_block(ctx, ncol, ldi, ldo));
    if (ncol == 0 || !ctx->has_nl) return SGPU_OK;
    double *dx, *dh, *alpha;
    long lx, lh;
    SGPU_TRY(stage_in(ctx, WS_STAGE_A, x, ldi, ncol, true, &dx, &lx));
    SGPU_TRY(stage_in(ctx, WS_STAGE_B, Hx, ldo, ncol, true, &dh, &lh));
    const long lda = nonlocal_alpha_ld(ncol, (int)sizeof(double));
    const size_t bytes = sizeof(double) * (size_t)ctx->nl.ntot * lda;
    SGPU_TRY(ws_get(ctx, WS_ALPHA, bytes, (void **)&alpha));
    SGPU_CUDA_TRY(cudaMemsetAsync(alpha, 0, bytes, ctx->stream));
    SGPU_TRY(launch_nonlocal_project<double>(ctx, ncol, dx, lx, alpha, lda, ctx->stream));
    SGPU_TRY(launch_nonlocal_apply<double>(ctx, ncol, alpha, lda, 1.0, dh, lh, ctx->stream));
    SGPU_TRY(stage_out(ctx, dh, lh, Hx, ldo, ncol));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_Hamiltonian_vectors_mult(sgpu_ctx *ctx, int spin, int ncol, double c, const double *x,
                                  int ldi, double *Hx, int ldo)
{
    SGPU_TRY(check_ctx(ctx));
    SGPU_TRY(check_block(ctx, ncol, ldi, ldo));
    if (ncol == 0) return SGPU_OK;
    double *dx, *dh;
    long lx, lh;
    SGPU_TRY(stage_in(ctx, WS_STAGE_A, x, ldi, ncol, true, &dx, &lx));
    SGPU_TRY(stage_in(ctx, WS_STAGE_B, Hx, ldo, ncol, false, &dh, &lh));
    SGPU_TRY(hamiltonian_dev<double>(ctx, spin, ncol, c, dx, lx, dh, lh, 1.0, 0.0, nullptr, 0,
                                     ctx->stream));
    SGPU_TRY(stage_out(ctx, dh, lh, Hx, ldo, ncol));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

// Host-array filter, pipelined over column chunks. The filter acts on every column on its own,
// so the block is cut into chunks that move through three device slots: while chunk i is
// filtered on the context stream, chunk i+1 is copied in on one copy stream and chunk i-1
// copied out on another. The host-device copies then hide behind the filter instead of
// adding to it. Each column's arithmetic is the one of the unchunked call.
// return_x false: X is input only (its chunks are not copied back).
static int filter_pipelined(sgpu_ctx *ctx, int spin, double *X, int ldi, double *Y, int ldo,
                            int ncol, int nc, int m, double a, double b, double a0, bool f32,
                            bool return_x)
{
    const long Nd = ctx->Nd;
    if (!ctx->copy_in) {
        SGPU_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->copy_in, cudaStreamNonBlocking));
        SGPU_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->copy_out, cudaStreamNonBlocking));
        for (auto &slot : ctx->pipe_ev)
            for (auto &e : slot) SGPU_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    // per slot: FP64 X and Y of nc columns, and (FP32) their FP32 images
    const size_t n64 = (size_t)Nd * nc, per = n64 * (2 * sizeof(double) + (f32 ? 2 * sizeof(float) : 0));
    char *base = nullptr;
    SGPU_TRY(ws_get(ctx, WS_STAGE_A, 3 * per, (void **)&base));
    // the previous call's copies out of these buffers are complete: every call ends synchronised
    cudaStream_t cs = ctx->stream;
    // chunk widths: the first and last chunks, whose copies nothing overlaps, are small
    // (nc/4, then 3nc/4 to get back in step), the ones between nc wide
    std::vector<int> widths;
    if (ncol >= 4 * nc && nc >= 16) {
        const int q = nc / 4;
        widths = {q, nc - q};
        int left = ncol - nc;
        while (left > nc) {
            const int w = std::min(nc, left - nc);
            if (w <= 0) break;
            widths.push_back(w);
            left -= w;
        }
        widths.push_back(left - q);
        widths.push_back(q);
    } else {
        for (int c = 0; c < ncol; c += nc) widths.push_back(std::min(nc, ncol - c));
    }
    const int nchunk = (int)widths.size();
    int c0 = 0;
    for (int i = 0; i < nchunk; c0 += widths[i], i++) {
        const int s = i % 3, w = widths[i];
        double *dX = reinterpret_cast<double *>(base + s * per), *dY = dX + n64;
        float *fX = reinterpret_cast<float *>(dY + n64), *fY = fX + n64;
        cudaEvent_t in_done = ctx->pipe_ev[s][0], filtered = ctx->pipe_ev[s][1],
                    freed = ctx->pipe_ev[s][2];
        if (i >= 3) SGPU_CUDA_TRY(cudaStreamWaitEvent(ctx->copy_in, freed, 0));
        SGPU_CUDA_TRY(cudaMemcpy2DAsync(dX, sizeof(double) * Nd, X + (long)c0 * ldi,
                                        sizeof(double) * ldi, sizeof(double) * Nd, w,
                                        cudaMemcpyHostToDevice, ctx->copy_in));
        SGPU_CUDA_TRY(cudaEventRecord(in_done, ctx->copy_in));
        SGPU_CUDA_TRY(cudaStreamWaitEvent(cs, in_done, 0));
        if (i == 0) SGPU_CUDA_TRY(cudaEventRecord(ctx->ev0, cs));
        if (f32) {
            {
                ProfScope ps(ctx, SGPU_KERNEL_OTHER, cs);
                SGPU_TRY(convert_cols<double, float>(dX, Nd, fX, Nd, Nd, w, cs));
            }
            SGPU_TRY(chebyshev_dev<float>(ctx, spin, fX, Nd, fY, Nd, w, m, a, b, a0, cs));
            ProfScope ps(ctx, SGPU_KERNEL_OTHER, cs);
            if (return_x) SGPU_TRY(convert_cols<float, double>(fX, Nd, dX, Nd, Nd, w, cs));
            SGPU_TRY(convert_cols<float, double>(fY, Nd, dY, Nd, Nd, w, cs));
            ctx->launches++;
        } else {
            SGPU_TRY(chebyshev_dev<double>(ctx, spin, dX, Nd, dY, Nd, w, m, a, b, a0, cs));
        }
        if (i == nchunk - 1) SGPU_CUDA_TRY(cudaEventRecord(ctx->ev1, cs));
        SGPU_CUDA_TRY(cudaEventRecord(filtered, cs));
        SGPU_CUDA_TRY(cudaStreamWaitEvent(ctx->copy_out, filtered, 0));
        if (return_x)
            SGPU_CUDA_TRY(cudaMemcpy2DAsync(X + (long)c0 * ldi, sizeof(double) * ldi, dX,
                                            sizeof(double) * Nd, sizeof(double) * Nd, w,
                                            cudaMemcpyDeviceToHost, ctx->copy_out));
        SGPU_CUDA_TRY(cudaMemcpy2DAsync(Y + (long)c0 * ldo, sizeof(double) * ldo, dY,
                                        sizeof(double) * Nd, sizeof(double) * Nd, w,
                                        cudaMemcpyDeviceToHost, ctx->copy_out));
        SGPU_CUDA_TRY(cudaEventRecord(freed, ctx->copy_out));
    }
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->copy_out));
    SGPU_CUDA_TRY(cudaStreamSynchronize(cs));
    SGPU_CUDA_TRY(cudaEventElapsedTime(&ctx->last_filter_ms, ctx->ev0, ctx->ev1));
    return kernel_status_check(ctx);
}

static int filter_host_or_device(sgpu_ctx *ctx, int spin, double *X, int ldi, double *Y,
                                 int ldo, int ncol, int m, double a, double b, double a0,
                                 int precision, bool return_x);

int sgpu_ChebyshevFiltering(sgpu_ctx *ctx, int spin, double *X, int ldi, double *Y, int ldo,
                            int ncol, int m, double a, double b, double a0, int precision)
{
    return filter_host_or_device(ctx, spin, X, ldi, Y, ldo, ncol, m, a, b, a0, precision, true);
}

int sgpu_ChebyshevFiltering_y(sgpu_ctx *ctx, int spin, const double *X, int ldi, double *Y,
                              int ldo, int ncol, int m, double a, double b, double a0,
                              int precision)
{
    if (X && is_device_ptr(X)) {
        set_error("sgpu_ChebyshevFiltering_y: X must be a host array (device blocks: use "
                  "sgpu_ChebyshevFiltering, which works in place)");
        return SGPU_ERR_ARG;
    }
    return filter_host_or_device(ctx, spin, const_cast<double *>(X), ldi, Y, ldo, ncol, m, a, b,
                                 a0, precision, false);
}

static int filter_host_or_device(sgpu_ctx *ctx, int spin, double *X, int ldi, double *Y,
                                 int ldo, int ncol, int m, double a, double b, double a0,
                                 int precision, bool return_x)
{
    SGPU_TRY(check_ctx(ctx));
    SGPU_TRY(check_block(ctx, ncol, ldi, ldo));
    if (precision != SGPU_PREC_FP64 && precision != SGPU_PREC_FP32) {
        set_error("ChebyshevFiltering: precision must be SGPU_PREC_FP64 or SGPU_PREC_FP32");
        return SGPU_ERR_ARG;
    }
    if (!(b > a) || !(a > a0) || m < 1) {
        set_error("ChebyshevFiltering: need a0 < a < b and m >= 1");
        return SGPU_ERR_ARG;
    }
    if (ncol == 0) return SGPU_OK;
    // host arrays: stream column chunks (a quarter of the block, at least 64 columns) through
    // the device so the copies overlap the filter
    if (ncol >= 128 && !is_device_ptr(X) && !is_device_ptr(Y)) {
        const int nc = std::max(64, (ncol + 3) / 4);
        return filter_pipelined(ctx, spin, X, ldi, Y, ldo, ncol, nc, m, a, b, a0,
                                precision == SGPU_PREC_FP32, return_x);
    }
    double *dX, *dY;
    long lX, lY;
    SGPU_TRY(stage_in(ctx, WS_STAGE_A, X, ldi, ncol, true, &dX, &lX));
    SGPU_TRY(stage_in(ctx, WS_STAGE_B, Y, ldo, ncol, false, &dY, &lY));
    if (precision == SGPU_PREC_FP64) {
        SGPU_CUDA_TRY(cudaEventRecord(ctx->ev0, ctx->stream));
        SGPU_TRY(chebyshev_dev<double>(ctx, spin, dX, lX, dY, lY, ncol, m, a, b, a0,
                                       ctx->stream));
        SGPU_CUDA_TRY(cudaEventRecord(ctx->ev1, ctx->stream));
    } else {
        float *fX, *fY;
        const size_t fb = sizeof(float) * (size_t)ctx->Nd * ncol;
        SGPU_TRY(ws_get(ctx, WS_MISC, 2 * fb, (void **)&fX));
        fY = fX + (size_t)ctx->Nd * ncol;
        {
            ProfScope ps(ctx, SGPU_KERNEL_OTHER, ctx->stream);
            SGPU_TRY(convert_cols<double, float>(dX, lX, fX, ctx->Nd, ctx->Nd, ncol, ctx->stream));
        }
        SGPU_CUDA_TRY(cudaEventRecord(ctx->ev0, ctx->stream));
        SGPU_TRY(chebyshev_dev<float>(ctx, spin, fX, ctx->Nd, fY, ctx->Nd, ncol, m, a, b, a0,
                                      ctx->stream));
        SGPU_CUDA_TRY(cudaEventRecord(ctx->ev1, ctx->stream));
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, ctx->stream);
        if (return_x)
            SGPU_TRY(convert_cols<float, double>(fX, ctx->Nd, dX, lX, ctx->Nd, ncol, ctx->stream));
        SGPU_TRY(convert_cols<float, double>(fY, ctx->Nd, dY, lY, ctx->Nd, ncol, ctx->stream));
        ctx->launches++;
    }
    if (return_x) SGPU_TRY(stage_out(ctx, dX, lX, X, ldi, ncol));
    SGPU_TRY(stage_out(ctx, dY, lY, Y, ldo, ncol));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    SGPU_CUDA_TRY(cudaEventElapsedTime(&ctx->last_filter_ms, ctx->ev0, ctx->ev1));
    return SGPU_OK;
}

int sgpu_ChebyshevFiltering_f32(sgpu_ctx *ctx, int spin, float *X, int ldi, float *Y, int ldo,
                                int ncol, int m, double a, double b, double a0)
{
    SGPU_TRY(check_ctx(ctx));
    SGPU_TRY(check_block(ctx, ncol, ldi, ldo));
    if (!(b > a) || !(a > a0) || m < 1) {
        set_error("ChebyshevFiltering: need a0 < a < b and m >= 1");
        return SGPU_ERR_ARG;
    }
    if (ncol == 0) return SGPU_OK;
    const size_t pitch = sizeof(float) * ctx->Nd;
    float *dX = X, *dY = Y;
    long lX = ldi, lY = ldo;
    const bool hx = !is_device_ptr(X), hy = !is_device_ptr(Y);
    if (hx) {
        SGPU_TRY(ws_get(ctx, WS_STAGE_A, pitch * ncol, (void **)&dX));
        SGPU_CUDA_TRY(cudaMemcpy2DAsync(dX, pitch, X, sizeof(float) * ldi, pitch, ncol,
                                        cudaMemcpyHostToDevice, ctx->stream));
        lX = ctx->Nd;
    }
    if (hy) {
        SGPU_TRY(ws_get(ctx, WS_STAGE_B, pitch * ncol, (void **)&dY));
        lY = ctx->Nd;
    }
    SGPU_CUDA_TRY(cudaEventRecord(ctx->ev0, ctx->stream));
    SGPU_TRY(chebyshev_dev<float>(ctx, spin, dX, lX, dY, lY, ncol, m, a, b, a0, ctx->stream));
    SGPU_CUDA_TRY(cudaEventRecord(ctx->ev1, ctx->stream));
    if (hx)
        SGPU_CUDA_TRY(cudaMemcpy2DAsync(X, sizeof(float) * ldi, dX, pitch, pitch, ncol,
                                        cudaMemcpyDeviceToHost, ctx->stream));
    if (hy)
        SGPU_CUDA_TRY(cudaMemcpy2DAsync(Y, sizeof(float) * ldo, dY, pitch, pitch, ncol,
                                        cudaMemcpyDeviceToHost, ctx->stream));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    SGPU_CUDA_TRY(cudaEventElapsedTime(&ctx->last_filter_ms, ctx->ev0, ctx->ev1));
    return kernel_status_check(ctx);
}

int sgpu_get_stream(sgpu_ctx *ctx, void **stream)
{
    if (!ctx || !stream) {
        set_error("sgpu_get_stream: null argument");
        return SGPU_ERR_ARG;
    }
    *stream = (void *)ctx->stream;
    return SGPU_OK;
}

int sgpu_poisson_residual(sgpu_ctx *ctx, double c, const double *x, const double *b, double *r)
{
    SGPU_TRY(check_ctx(ctx));
    double *dx, *db, *dr;
    long lx, lb, lr;
    SGPU_TRY(stage_in(ctx, WS_STAGE_A, x, (int)ctx->Nd, 1, true, &dx, &lx));
    SGPU_TRY(stage_in(ctx, WS_STAGE_C, b, (int)ctx->Nd, 1, true, &db, &lb));
    SGPU_TRY(stage_in(ctx, WS_STAGE_B, r, (int)ctx->Nd, 1, false, &dr, &lr));
    // r = 1 * (Lap + c) x + 1 * b
    SGPU_TRY(launch_stencil<double>(ctx, 1, 1.0, 0.0, c, nullptr, dx, lx, dr, lr, 1.0, 1.0, db,
                                    lb, ctx->stream));
    SGPU_TRY(stage_out(ctx, dr, lr, r, (int)ctx->Nd, 1));
    SGPU_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return SGPU_OK;
}

int sgpu_profile_enable(sgpu_ctx *ctx, int on)
{
    SGPU_TRY(check_ctx(ctx));
    SGPU_TRY(prof_resolve(ctx));
    ctx->prof_on = on != 0;
    for (int k = 0; k < SGPU_KERNEL_KINDS; k++) {
        ctx->prof_ms[k] = 0.0;
        ctx->prof_n[k] = 0;
    }
    ctx->launches = 0;
    return SGPU_OK;
}

int sgpu_profile_read(sgpu_ctx *ctx, int kind, double *total_ms, long *launches)
{
    SGPU_TRY(check_ctx(ctx));
    if (kind < 0 || kind > SGPU_KERNEL_KINDS || !total_ms || !launches) {
        set_error("sgpu_profile_read: bad kind or null output");
        return SGPU_ERR_ARG;
    }
    SGPU_TRY(prof_resolve(ctx));
    if (kind == SGPU_KERNEL_KINDS) {
        *total_ms = 0.0;
        *launches = ctx->launches;
    } else {
        *total_ms = ctx->prof_ms[kind];
        *launches = ctx->prof_n[kind];
    }
    return SGPU_OK;
}

int sgpu_kernel_status(sgpu_ctx *ctx, int *status)
{
    SGPU_TRY(check_ctx(ctx));
    if (!status) {
        set_error("sgpu_kernel_status: null argument");
        return SGPU_ERR_ARG;
    }
    return kernel_status_check(ctx, status);
}

int sgpu_check_wait_bound(sgpu_ctx *ctx, int *status)
{
    SGPU_TRY(check_ctx(ctx));
    if (!status) {
        set_error("sgpu_check_wait_bound: null argument");
        return SGPU_ERR_ARG;
    }
    SGPU_TRY(kernel_status_check(ctx));  // start from a clear word
    SGPU_TRY(wait_bound_check(ctx));
    int st = 0;
    const int rc = kernel_status_check(ctx, &st);
    *status = st;
    if (st == 2) return SGPU_OK;  // the bound ran out as it should and the word is clear again
    if (rc != SGPU_OK) return rc;
    set_error("sgpu_check_wait_bound: the bounded wait did not report running out");
    return SGPU_ERR_STATE;
}

int sgpu_measure_fp64_rate(sgpu_ctx *ctx, double *tflops)
{
    SGPU_TRY(check_ctx(ctx));
    if (!tflops) {
        set_error("sgpu_measure_fp64_rate: null argument");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    return fp64_fma_rate(ctx, tflops);
}

int sgpu_last_filter_ms(sgpu_ctx *ctx, float *ms)
{
    if (!ctx || !ms) {
        set_error("sgpu_last_filter_ms: null argument");
        return SGPU_ERR_ARG;
    }
    *ms = ctx->last_filter_ms;
    return SGPU_OK;
}

}  // extern "C"
