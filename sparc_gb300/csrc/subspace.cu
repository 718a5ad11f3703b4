// Rayleigh-Ritz step of CheFSI: projection, generalized eigensolve, rotation.
//
// Reference (USE_DP_SUBEIG path, one process):
//   DP_Project_Hamiltonian            src/eigenSolver.c:939-1082
//       HY = H Y (one more Hamiltonian apply, :960), Mp = Yᵀ Y, Hp = Yᵀ HY (cblas_dgemm :1022-1033)
//   DP_Solve_Generalized_EigenProblem src/eigenSolver.c:1262-1375
//       LAPACKE_dsygvd(COL_MAJOR, 1, 'V', 'U', Ns, Hp, Ns, Mp, Ns, lambda) (:1318); Q = Hp
//   DP_Subspace_Rotation              src/eigenSolver.c:1386-1439
//       X = Y Q (cblas_dgemm :1415)
//
// GPU form: with rr_tc set (sgpu_set_rr_products), FP32 blocks (the mixed-precision filter)
// and the mixed-precision SCF's FP64 phase use the library's own tcgen05 kernels (rr_tc.cu:
// split-slice BF16 products with exact chunk accumulation, FP32- or FP64-accurate); the plain
// FP64 drop-in keeps cuBLAS DSYRK/DGEMM, and with rr_tc = 0 FP32 blocks go to cuBLAS FP32
// GEMMs (BF16x9 emulation requested; on this GB300 cuBLAS keeps its FP32 SIMT GEMM, 56
// TFLOP/s at the Si216 shapes). The Ns x Ns generalized eigenproblem stays FP64 on cuSOLVER
// (dsygvd).
#include <algorithm>

#include <cuda_bf16.h>

#include "sgpu_internal.h"

namespace sgpu {

int ensure_solver_handles(sgpu_ctx *ctx);
static int ensure_handles(sgpu_ctx *ctx) { return ensure_solver_handles(ctx); }

// cuBLAS / cuSOLVER handles of the context, on its stream (created on first use)
int ensure_solver_handles(sgpu_ctx *ctx)
{
    if (!ctx->cublas) {
        SGPU_CUBLAS_TRY(cublasCreate(&ctx->cublas));
        SGPU_CUBLAS_TRY(cublasSetStream(ctx->cublas, ctx->stream));
        SGPU_CUBLAS_TRY(cublasSetEmulationStrategy(
            ctx->cublas, ctx->gemm_mode == 1 ? CUBLAS_EMULATION_STRATEGY_EAGER
                                             : CUBLAS_EMULATION_STRATEGY_PERFORMANT));
    }
    if (!ctx->cusolver) {
        if (cusolverDnCreate(&ctx->cusolver) != CUSOLVER_STATUS_SUCCESS) {
            set_error("cusolverDnCreate failed");
            return SGPU_ERR_CUDA;
        }
        cusolverDnSetStream(ctx->cusolver, ctx->stream);
    }
    return SGPU_OK;
}

namespace {
// symmetrise an Ns x Ns column-major matrix from its upper triangle
template <typename T>
__global__ void k_sym_from_upper(T *A, int n, int lda)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i < n && j < n && i > j) A[(long)j * lda + i] = A[(long)i * lda + j];
}

__global__ void k_f32_to_f64(const float *__restrict__ a, double *__restrict__ b, long n)
{
    for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < n;
         t += (long)gridDim.x * blockDim.x)
        b[t] = (double)a[t];
}
}  // namespace

// Hp = Yᵀ HY and Mp = Yᵀ Y (full symmetric Ns x Ns, column-major, ld = Ns), FP64 blocks.
int project_f64(sgpu_ctx *ctx, int ncol, const double *Y, long ldy, const double *HY,
                long ldh, double *Hp, double *Mp, cudaStream_t st)
{
    if (ctx->rr_tc == 2) return tc_project<double>(ctx, ncol, Y, ldy, HY, ldh, Hp, Mp, true, st);
    SGPU_TRY(ensure_handles(ctx));
    SGPU_CUBLAS_TRY(cublasSetStream(ctx->cublas, st));
    const double one = 1.0, zero = 0.0;
    {
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        SGPU_CUBLAS_TRY(cublasDsyrk(ctx->cublas, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_T, ncol,
                                    (int)ctx->Nd, &one, Y, (int)ldy, &zero, Mp, ncol));
    }
    {
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        SGPU_CUBLAS_TRY(cublasDgemm(ctx->cublas, CUBLAS_OP_T, CUBLAS_OP_N, ncol, ncol,
                                    (int)ctx->Nd, &one, Y, (int)ldy, HY, (int)ldh, &zero, Hp,
                                    ncol));
    }
    dim3 b(16, 16), g((ncol + 15) / 16, (ncol + 15) / 16);
    k_sym_from_upper<double><<<g, b, 0, st>>>(Mp, ncol, ncol);
    ctx->launches++;
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

// FP32-accurate products on the BF16 tensor cores (gemm_mode 2). Each FP32 operand x becomes
// three BF16 parts, hi = bf16(x), mid = bf16(x - hi), lo = bf16(x - hi - mid) (both
// differences are exact in FP32), which carry its 24-bit significand 8 bits at a time; a
// product is then the sum of the six part products whose orders add up to at most 2 (the
// dropped ones are below FP32 rounding), each a BF16 GEMM with FP32 accumulation, smallest
// first. x: rows x cols, leading dimension ldx; parts: leading dimension rows.
__global__ void k_split3_bf16(const float *__restrict__ x, long ldx, long rows,
                              __nv_bfloat16 *__restrict__ p0, __nv_bfloat16 *__restrict__ p1,
                              __nv_bfloat16 *__restrict__ p2)
{
    const long c = blockIdx.y;
    const float *xc = x + c * ldx;
    const long o = c * rows;
    for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < rows;
         r += (long)gridDim.x * blockDim.x) {
        const float v = xc[r];
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        const float r1 = v - __bfloat162float(h);
        const __nv_bfloat16 m = __float2bfloat16_rn(r1);
        const float r2 = r1 - __bfloat162float(m);
        p0[o + r] = h;
        p1[o + r] = m;
        p2[o + r] = __float2bfloat16_rn(r2);
    }
}

static int split3(sgpu_ctx *ctx, const float *x, long ldx, long rows, int cols, int slot,
                  __nv_bfloat16 **parts, cudaStream_t st)
{
    __nv_bfloat16 *base = nullptr;
    SGPU_TRY(ws_get(ctx, slot, sizeof(__nv_bfloat16) * 3 * (size_t)rows * cols, (void **)&base));
    for (int i = 0; i < 3; i++) parts[i] = base + (size_t)i * rows * cols;
    const dim3 grid((unsigned)std::max<long>(1, std::min<long>((rows + 1023) / 1024, 64)), cols);
    ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
    k_split3_bf16<<<grid, 256, 0, st>>>(x, ldx, rows, parts[0], parts[1], parts[2]);
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

// C (m x n, FP32) = op(A) op(B) from the three parts of each operand
static int gemm_split3(sgpu_ctx *ctx, cublasOperation_t ta, cublasOperation_t tb, int m, int n,
                       int k, __nv_bfloat16 *const *A, int lda, __nv_bfloat16 *const *B, int ldb,
                       float *C, int ldc, cudaStream_t st)
{
    static const int terms[6][2] = {{2, 0}, {0, 2}, {1, 1}, {1, 0}, {0, 1}, {0, 0}};
    const float one = 1.f, zero = 0.f;
    for (int t = 0; t < 6; t++) {
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        SGPU_CUBLAS_TRY(cublasGemmEx(ctx->cublas, ta, tb, m, n, k, &one, A[terms[t][0]],
                                     CUDA_R_16BF, lda, B[terms[t][1]], CUDA_R_16BF, ldb,
                                     t == 0 ? &zero : &one, C, CUDA_R_32F, ldc,
                                     CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT));
    }
    return SGPU_OK;
}

// The same for FP32 blocks: FP32-accurate products, accumulated in FP32, then widened to FP64
// for the eigensolver. gemm_mode 0 / 1: cuBLAS FP32 GEMM with the BF16x9 emulation requested
// (performant / eager strategy); 2: the three-part BF16 split above on the tensor cores.
int project_f32(sgpu_ctx *ctx, int ncol, const float *Y, long ldy, const float *HY, long ldh,
                double *Hp, double *Mp, cudaStream_t st)
{
    if (ctx->rr_tc) return tc_project<float>(ctx, ncol, Y, ldy, HY, ldh, Hp, Mp, false, st);
    SGPU_TRY(ensure_handles(ctx));
    SGPU_CUBLAS_TRY(cublasSetStream(ctx->cublas, st));
    float *tmp = nullptr;
    SGPU_TRY(ws_get(ctx, WS_EIG, sizeof(float) * 2 * (size_t)ncol * ncol, (void **)&tmp));
    const float one = 1.f, zero = 0.f;
    if (ctx->gemm_mode == 2) {
        __nv_bfloat16 *ys[3], *hs[3];
        SGPU_TRY(split3(ctx, Y, ldy, ctx->Nd, ncol, WS_SPLIT_A, ys, st));
        SGPU_TRY(split3(ctx, HY, ldh, ctx->Nd, ncol, WS_SPLIT_B, hs, st));
        SGPU_TRY(gemm_split3(ctx, CUBLAS_OP_T, CUBLAS_OP_N, ncol, ncol, (int)ctx->Nd, ys,
                             (int)ctx->Nd, ys, (int)ctx->Nd, tmp, ncol, st));
        SGPU_TRY(gemm_split3(ctx, CUBLAS_OP_T, CUBLAS_OP_N, ncol, ncol, (int)ctx->Nd, ys,
                             (int)ctx->Nd, hs, (int)ctx->Nd, tmp + (size_t)ncol * ncol, ncol, st));
    }
    for (int w = 0; w < 2 && ctx->gemm_mode != 2; w++) {
        const float *B = w == 0 ? Y : HY;
        const long ldb = w == 0 ? ldy : ldh;
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        SGPU_CUBLAS_TRY(cublasGemmEx(ctx->cublas, CUBLAS_OP_T, CUBLAS_OP_N, ncol, ncol,
                                     (int)ctx->Nd, &one, Y, CUDA_R_32F, (int)ldy, B, CUDA_R_32F,
                                     (int)ldb, &zero, tmp + (size_t)w * ncol * ncol, CUDA_R_32F,
                                     ncol, CUBLAS_COMPUTE_32F_EMULATED_16BFX9,
                                     CUBLAS_GEMM_DEFAULT));
    }
    const long n2 = (long)ncol * ncol;
    k_f32_to_f64<<<std::max<long>(1, std::min<long>((n2 + 255) / 256, 4096)), 256, 0, st>>>(
        tmp, Mp, n2);
    k_f32_to_f64<<<std::max<long>(1, std::min<long>((n2 + 255) / 256, 4096)), 256, 0, st>>>(
        tmp + n2, Hp, n2);
    ctx->launches += 2;
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

static int potrf_upper(sgpu_ctx *ctx, int n, double *M, cudaStream_t st);
static int standard_eig_j(sgpu_ctx *ctx, int n, double *A, double *lambda_dev, bool jacobi,
                          cudaStream_t st);

// The same pencil reduced by hand: Mp = Uᵀ U (dpotrf), C = U^-T Hp U^-1 (two dtrsm), C = V Λ Vᵀ
// (dsyevd, or Jacobi dsyevj), Q = U^-1 V (dtrsm); the steps LAPACK's dsygvd takes, as
// separate library calls (eig_mode 1 and 2: timed against dsygvd by bench.py --rr-gemm)
static int generalized_eig_reduced(sgpu_ctx *ctx, int n, double *Hp, double *Mp,
                                   double *lambda_dev, bool jacobi, cudaStream_t st)
{
    SGPU_TRY(potrf_upper(ctx, n, Mp, st));
    SGPU_CUBLAS_TRY(cublasSetStream(ctx->cublas, st));
    const double one = 1.0;
    {
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        SGPU_CUBLAS_TRY(cublasDtrsm(ctx->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER,
                                    CUBLAS_OP_T, CUBLAS_DIAG_NON_UNIT, n, n, &one, Mp, n, Hp, n));
        SGPU_CUBLAS_TRY(cublasDtrsm(ctx->cublas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_UPPER,
                                    CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, n, &one, Mp, n, Hp, n));
    }
    SGPU_TRY(standard_eig_j(ctx, n, Hp, lambda_dev, jacobi, st));
    ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
    SGPU_CUBLAS_TRY(cublasDtrsm(ctx->cublas, CUBLAS_SIDE_LEFT, CUBLAS_FILL_MODE_UPPER,
                                CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, n, n, &one, Mp, n, Hp, n));
    return SGPU_OK;
}

// Hp q = lambda Mp q (upper triangles referenced); on return Hp holds Q, lambda ascending.
// Mp is overwritten by its Cholesky factor. ctx->eig_mode: 0 cuSOLVER dsygvd (the reference's
// LAPACKE_dsygvd, src/eigenSolver.c:1318), 1 Cholesky reduction + dsyevd, 2 Cholesky
// reduction + Jacobi dsyevj.
int generalized_eig(sgpu_ctx *ctx, int n, double *Hp, double *Mp, double *lambda_dev,
                    cudaStream_t st)
{
    SGPU_TRY(ensure_handles(ctx));
    cusolverDnSetStream(ctx->cusolver, st);
    if (ctx->eig_mode == 1 || ctx->eig_mode == 2)
        return generalized_eig_reduced(ctx, n, Hp, Mp, lambda_dev, ctx->eig_mode == 2, st);
    int lwork = 0;
    if (cusolverDnDsygvd_bufferSize(ctx->cusolver, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR,
                                    CUBLAS_FILL_MODE_UPPER, n, Hp, n, Mp, n, lambda_dev,
                                    &lwork) != CUSOLVER_STATUS_SUCCESS) {
        set_error("cusolverDnDsygvd_bufferSize failed");
        return SGPU_ERR_CUDA;
    }
    char *wsp = nullptr;
    SGPU_TRY(ws_get(ctx, WS_MISC, sizeof(double) * ((size_t)lwork + 1) + 64, (void **)&wsp));
    double *work = reinterpret_cast<double *>(wsp);
    int *info = reinterpret_cast<int *>(wsp + sizeof(double) * ((size_t)lwork + 1));
    ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
    if (cusolverDnDsygvd(ctx->cusolver, CUSOLVER_EIG_TYPE_1, CUSOLVER_EIG_MODE_VECTOR,
                         CUBLAS_FILL_MODE_UPPER, n, Hp, n, Mp, n, lambda_dev, work, lwork,
                         info) != CUSOLVER_STATUS_SUCCESS) {
        set_error("cusolverDnDsygvd failed to launch");
        return SGPU_ERR_CUDA;
    }
    int hinfo = 0;
    SGPU_CUDA_TRY(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, st));
    SGPU_CUDA_TRY(cudaStreamSynchronize(st));
    if (hinfo != 0) {
        set_error("dsygvd: info = " + std::to_string(hinfo) +
                  (hinfo > n ? " (Mp is not positive definite)" : " (no convergence)"));
        return SGPU_ERR_LINALG;
    }
    return SGPU_OK;
}

// M = Rᵀ R in place (upper triangle, cuSOLVER dpotrf)
static int potrf_upper(sgpu_ctx *ctx, int n, double *M, cudaStream_t st)
{
    int lwork = 0;
    if (cusolverDnDpotrf_bufferSize(ctx->cusolver, CUBLAS_FILL_MODE_UPPER, n, M, n, &lwork) !=
        CUSOLVER_STATUS_SUCCESS) {
        set_error("cusolverDnDpotrf_bufferSize failed");
        return SGPU_ERR_CUDA;
    }
    char *wsp = nullptr;
    SGPU_TRY(ws_get(ctx, WS_MISC, sizeof(double) * ((size_t)lwork + 1) + 64, (void **)&wsp));
    double *work = reinterpret_cast<double *>(wsp);
    int *info = reinterpret_cast<int *>(wsp + sizeof(double) * ((size_t)lwork + 1));
    {
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        if (cusolverDnDpotrf(ctx->cusolver, CUBLAS_FILL_MODE_UPPER, n, M, n, work, lwork,
                             info) != CUSOLVER_STATUS_SUCCESS) {
            set_error("cusolverDnDpotrf failed to launch");
            return SGPU_ERR_CUDA;
        }
    }
    int hinfo = 0;
    SGPU_CUDA_TRY(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, st));
    SGPU_CUDA_TRY(cudaStreamSynchronize(st));
    if (hinfo != 0) {
        set_error("dpotrf: the Gram matrix is not positive definite (info = " +
                  std::to_string(hinfo) + ")");
        return SGPU_ERR_LINALG;
    }
    return SGPU_OK;
}

// Cholesky orthonormalisation of an FP64 block, as DP_Project_Hamiltonian_std does it
// (src/eigenSolver.c:1130-1163): Mp = Yᵀ Y, Mp = Rᵀ R (dpotrf, upper), Y <- Y R^{-1} (dtrsm).
int cholqr_f64(sgpu_ctx *ctx, int ncol, double *Y, long ldy, cudaStream_t st)
{
    SGPU_TRY(ensure_handles(ctx));
    SGPU_CUBLAS_TRY(cublasSetStream(ctx->cublas, st));
    cusolverDnSetStream(ctx->cusolver, st);
    double *M = nullptr;
    SGPU_TRY(ws_get(ctx, WS_EIG, sizeof(double) * (size_t)ncol * ncol, (void **)&M));
    const double one = 1.0, zero = 0.0;
    {
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        SGPU_CUBLAS_TRY(cublasDsyrk(ctx->cublas, CUBLAS_FILL_MODE_UPPER, CUBLAS_OP_T, ncol,
                                    (int)ctx->Nd, &one, Y, (int)ldy, &zero, M, ncol));
    }
    SGPU_TRY(potrf_upper(ctx, ncol, M, st));
    ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
    SGPU_CUBLAS_TRY(cublasDtrsm(ctx->cublas, CUBLAS_SIDE_RIGHT, CUBLAS_FILL_MODE_UPPER,
                                CUBLAS_OP_N, CUBLAS_DIAG_NON_UNIT, (int)ctx->Nd, ncol, &one, M,
                                ncol, Y, (int)ldy));
    return SGPU_OK;
}

// A = V Λ Vᵀ with Jacobi sweeps (cuSOLVER dsyevj, tolerance 1e-15, up to 100 sweeps); A
// becomes V, lambda ascending
static int syevj(sgpu_ctx *ctx, int n, double *A, double *lambda_dev, cudaStream_t st)
{
    syevjInfo_t params = nullptr;
    if (cusolverDnCreateSyevjInfo(&params) != CUSOLVER_STATUS_SUCCESS) {
        set_error("cusolverDnCreateSyevjInfo failed");
        return SGPU_ERR_CUDA;
    }
    cusolverDnXsyevjSetTolerance(params, 1e-15);
    cusolverDnXsyevjSetMaxSweeps(params, 100);
    int lwork = 0, rc = SGPU_OK;
    if (cusolverDnDsyevj_bufferSize(ctx->cusolver, CUSOLVER_EIG_MODE_VECTOR,
                                    CUBLAS_FILL_MODE_UPPER, n, A, n, lambda_dev, &lwork,
                                    params) != CUSOLVER_STATUS_SUCCESS) {
        cusolverDnDestroySyevjInfo(params);
        set_error("cusolverDnDsyevj_bufferSize failed");
        return SGPU_ERR_CUDA;
    }
    char *wsp = nullptr;
    rc = ws_get(ctx, WS_MISC, sizeof(double) * ((size_t)lwork + 1) + 64, (void **)&wsp);
    if (rc == SGPU_OK) {
        double *work = reinterpret_cast<double *>(wsp);
        int *info = reinterpret_cast<int *>(wsp + sizeof(double) * ((size_t)lwork + 1));
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        if (cusolverDnDsyevj(ctx->cusolver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n,
                             A, n, lambda_dev, work, lwork, info,
                             params) != CUSOLVER_STATUS_SUCCESS) {
            set_error("cusolverDnDsyevj failed to launch");
            rc = SGPU_ERR_CUDA;
        } else {
            int hinfo = 0;
            if (cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, st) !=
                    cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess) {
                set_error("dsyevj: reading info failed");
                rc = SGPU_ERR_CUDA;
            } else if (hinfo != 0) {
                set_error("dsyevj: info = " + std::to_string(hinfo));
                rc = SGPU_ERR_LINALG;
            }
        }
    }
    cusolverDnDestroySyevjInfo(params);
    return rc;
}

static int standard_eig_j(sgpu_ctx *ctx, int n, double *A, double *lambda_dev, bool jacobi,
                          cudaStream_t st)
{
    return jacobi ? syevj(ctx, n, A, lambda_dev, st) : standard_eig(ctx, n, A, lambda_dev, st);
}

// Hp q = lambda q (upper triangle; dsyevd, the STANDARD_EIGEN branch of
// DP_Solve_Generalized_EigenProblem, src/eigenSolver.c:1318-1321); Hp becomes Q.
int standard_eig(sgpu_ctx *ctx, int n, double *Hp, double *lambda_dev, cudaStream_t st)
{
    SGPU_TRY(ensure_handles(ctx));
    cusolverDnSetStream(ctx->cusolver, st);
    int lwork = 0;
    if (cusolverDnDsyevd_bufferSize(ctx->cusolver, CUSOLVER_EIG_MODE_VECTOR,
                                    CUBLAS_FILL_MODE_UPPER, n, Hp, n, lambda_dev,
                                    &lwork) != CUSOLVER_STATUS_SUCCESS) {
        set_error("cusolverDnDsyevd_bufferSize failed");
        return SGPU_ERR_CUDA;
    }
    char *wsp = nullptr;
    SGPU_TRY(ws_get(ctx, WS_MISC, sizeof(double) * ((size_t)lwork + 1) + 64, (void **)&wsp));
    double *work = reinterpret_cast<double *>(wsp);
    int *info = reinterpret_cast<int *>(wsp + sizeof(double) * ((size_t)lwork + 1));
    ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
    if (cusolverDnDsyevd(ctx->cusolver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, n, Hp,
                         n, lambda_dev, work, lwork, info) != CUSOLVER_STATUS_SUCCESS) {
        set_error("cusolverDnDsyevd failed to launch");
        return SGPU_ERR_CUDA;
    }
    int hinfo = 0;
    SGPU_CUDA_TRY(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, st));
    SGPU_CUDA_TRY(cudaStreamSynchronize(st));
    if (hinfo != 0) {
        set_error("dsyevd: info = " + std::to_string(hinfo));
        return SGPU_ERR_LINALG;
    }
    return SGPU_OK;
}

// X = Y Q (FP64)
int rotate_f64(sgpu_ctx *ctx, int ncol, const double *Y, long ldy, const double *Q, double *X,
               long ldx, cudaStream_t st)
{
    if (ctx->rr_tc == 2) return tc_rotate<double>(ctx, ncol, Y, ldy, Q, ncol, X, ldx, true, st);
    SGPU_TRY(ensure_handles(ctx));
    SGPU_CUBLAS_TRY(cublasSetStream(ctx->cublas, st));
    const double one = 1.0, zero = 0.0;
    ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
    SGPU_CUBLAS_TRY(cublasDgemm(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, (int)ctx->Nd, ncol, ncol,
                                &one, Y, (int)ldy, Q, ncol, &zero, X, (int)ldx));
    return SGPU_OK;
}

// X = Y Q with FP32 blocks: Q is narrowed to FP32, FP32 product (BF16x9 emulation requested)
int rotate_f32(sgpu_ctx *ctx, int ncol, const float *Y, long ldy, const double *Q, float *X,
               long ldx, cudaStream_t st)
{
    if (ctx->rr_tc) return tc_rotate<float>(ctx, ncol, Y, ldy, Q, ncol, X, ldx, false, st);
    SGPU_TRY(ensure_handles(ctx));
    SGPU_CUBLAS_TRY(cublasSetStream(ctx->cublas, st));
    float *q32 = nullptr;
    SGPU_TRY(ws_get(ctx, WS_EIG, sizeof(float) * (size_t)ncol * ncol, (void **)&q32));
    {
        ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
        SGPU_TRY(convert_cols<double, float>(Q, ncol, q32, ncol, ncol, ncol, st));
    }
    if (ctx->gemm_mode == 2) {
        __nv_bfloat16 *ys[3], *qs[3];
        SGPU_TRY(split3(ctx, Y, ldy, ctx->Nd, ncol, WS_SPLIT_A, ys, st));
        SGPU_TRY(split3(ctx, q32, ncol, ncol, ncol, WS_SPLIT_B, qs, st));
        return gemm_split3(ctx, CUBLAS_OP_N, CUBLAS_OP_N, (int)ctx->Nd, ncol, ncol, ys,
                           (int)ctx->Nd, qs, ncol, X, (int)ldx, st);
    }
    const float one = 1.f, zero = 0.f;
    ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
    SGPU_CUBLAS_TRY(cublasGemmEx(ctx->cublas, CUBLAS_OP_N, CUBLAS_OP_N, (int)ctx->Nd, ncol, ncol,
                                 &one, Y, CUDA_R_32F, (int)ldy, q32, CUDA_R_32F, ncol, &zero, X,
                                 CUDA_R_32F, (int)ldx, CUBLAS_COMPUTE_32F_EMULATED_16BFX9,
                                 CUBLAS_GEMM_DEFAULT));
    return SGPU_OK;
}

}  // namespace sgpu
