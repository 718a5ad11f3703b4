// Internal declarations of the GB300 CheFSI library (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <cstddef>
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "../../include/sparc_gpu.h"

namespace sgpu {

constexpr int kMaxFDn = 6;  // the library is specialised for FD order 12 (radius 6)
constexpr int kApplyChunkPts = 128;  // covered points per chunk of the staged nonlocal apply
constexpr int kRangePts = 128;       // covered points per range of the range projection
constexpr int kRangeMaxEnt = 320;    // entries per range at most (bounds its staged Chi)
constexpr int kRangeItemEnt = 96;    // entries per work item of the range projection at most
constexpr int kRangeWarps = 8;       // warps per range block
static_assert(kRangePts % kRangeWarps == 0, "whole tile rows per warp");

// thread-local error text, returned by sgpu_last_error()
void set_error(const std::string &msg);

#define SGPU_CUDA_TRY(...)                                                                   \
    do {                                                                                     \
        cudaError_t err_ = (__VA_ARGS__);                                                    \
        if (err_ != cudaSuccess) {                                                           \
            ::sgpu::set_error(std::string(#__VA_ARGS__) + ": " + cudaGetErrorString(err_));  \
            return SGPU_ERR_CUDA;                                                            \
        }                                                                                    \
    } while (0)

#define SGPU_CUBLAS_TRY(call)                                                                \
    do {                                                                                     \
        cublasStatus_t st_ = (call);                                                         \
        if (st_ != CUBLAS_STATUS_SUCCESS) {                                                  \
            ::sgpu::set_error(std::string(#call) + ": cuBLAS status " + std::to_string(st_)); \
            return SGPU_ERR_CUDA;                                                            \
        }                                                                                    \
    } while (0)

#define SGPU_TRY(...)                                                                        \
    do {                                                                                     \
        int rc_ = (__VA_ARGS__);                                                                    \
        if (rc_ != SGPU_OK) return rc_;                                                      \
    } while (0)

// Device copy of the nonlocal projector set, in two index orders:
//  * image order (as the reference's Atom_Influence_nloc / nlocProj): for the projection
//    alpha = Chiᵀ x, parallel over (image, point chunk);
//  * point order (a CSR over covered grid points): for the owner-computes apply
//    Hx[p] += sum over entries (image, i) of Chi_img[i, :] alpha_atom.
struct Nonlocal {
    int natom = 0, nimg = 0, ntot = 0, max_np = 0;
    long nchi = 0, npos = 0;
    int *ip_displ = nullptr;    // natom + 1
    int *img_atom = nullptr;    // nimg
    int *img_ndc = nullptr;     // nimg
    long *img_off = nullptr;    // nimg, offset of the image's grid positions
    long *img_chi_off = nullptr;// nimg, offset of the image's Chi block
    int *grid_pos = nullptr;    // npos
    double *chi64 = nullptr;    // nchi, per image ndc x np column-major
    float *chi32 = nullptr;
    double *gamma64 = nullptr;  // ntot, per projector
    float *gamma32 = nullptr;
    // point CSR for the apply
    int ncov = 0;
    long nent = 0;
    int *cov_pt = nullptr;      // ncov covered grid points, ascending
    int *cov_ptr = nullptr;     // ncov + 1
    long *ent_chi = nullptr;    // nent: offset of the entry's Chi row (image block + index)
    int4 *ent_meta = nullptr;   // nent: (first projector row, projector count, ndc, image)
    // projection work items: (image, first point) segments
    int nseg = 0;
    int *seg_img = nullptr;
    int *seg_start = nullptr;
    // staged apply: chunks of consecutive covered points with the alpha rows they use
    int nchunk = 0, max_chunk_rows = 0;
    int *ent_slot = nullptr;       // nent: staged row of the entry's atom within its chunk
    int *chunk_row_ptr = nullptr;  // nchunk + 1
    int *chunk_rows = nullptr;     // alpha rows staged per chunk
    // range projection (FP32): ranges of consecutive covered points, each with its entries
    // regrouped by image into work items of at most kRangeItemEnt entries
    int nrange = 0, nitem = 0, max_range_ent = 0, range_jp = 0, max_range_items = 0;
    int *rng_pt0 = nullptr;     // nrange + 1: first covered point of each range
    int *rng_ent0 = nullptr;    // nrange + 1: first entry (range order) of each range
    int *rng_item0 = nullptr;   // nrange + 1: first work item of each range
    int *item_e0 = nullptr;     // nitem + 1: first entry (range order) of each item
    int *item_wsplit = nullptr; // nitem x (kRangeWarps + 1): an item's entries split by the
                                // warp that owns their point (range apply)
    int2 *item_row = nullptr;   // nitem: (first projector row, projector count)
    int *pe_lp = nullptr;       // entries in range order: point index within the range
    float *pe_chi32 = nullptr;  // entries in range order: Chi values, range_jp per entry
    // fused apply + projection on the tensor cores (nonlocal_tc.cu): ranges of at most 128
    // covered points (taken in compact-block order) whose atoms own at most 64 projector rows,
    // one merged entry per (point, atom); tc_nrange 0 when a covered point alone needs more
    int tc_nrange = 0;
    int *tc_pt0 = nullptr;      // tc_nrange + 1: first point of each range in tc_pts
    int *tc_pts = nullptr;      // grid point of every range point (ranges back to back)
    int *tc_row0 = nullptr;     // tc_nrange + 1: first row-list entry of each range
    int *tc_rows = nullptr;     // alpha row of every range row
    int *tc_ent0 = nullptr;     // tc_nrange + 1: first merged entry of each range
    int *tc_ent = nullptr;      // point | row offset << 7 | projector count << 14
    float *tc_chi = nullptr;    // Chi values of the merged entries, range_jp per entry
};

struct Workspace {
    void *ptr = nullptr;
    size_t bytes = 0;
};

struct KpointState;  // kpoint.cu
void kpoint_free(sgpu_ctx *ctx);
struct SetupState;   // setup.cu
void setup_free(sgpu_ctx *ctx);

// periodic-Pulay density mixing parameters (SPARC_OBJ fields of the same meaning)
struct MixParams {
    int m = 7;                 // MixingHistory
    int pulay_freq = 1;        // PulayFrequency
    int restart = 0;           // PulayRestartFlag
    double beta = 0.3;         // MixingParameter
    double omega = 0.3;        // MixingParameterSimple
    int kerker = 1;            // MixingPrecond == 1
    double kTF = 1.0;          // precond_kerker_kTF
    double idiemac = 0.1;      // precond_kerker_thresh
    double precond_tol = 1e-4; // TOL_PRECOND
    double neg_charge = 0.0;   // NegCharge (minus the electron count)
    int nspden = 1;            // Nspden: 1, or 2 for collinear spin (mixed vector [rho, magz])
    double beta_mag = 0.3;     // MixingParameterMag
    double omega_mag = 0.3;    // MixingParameterSimpleMag
};

// device-resident mixing history (mixing_hist_* of SPARC_OBJ)
struct MixState {
    int m = 0;
    MixParams prm;
    double *buf = nullptr;
    double *x_k = nullptr, *x_km1 = nullptr, *f_k = nullptr, *f_km1 = nullptr;
    double *Pf = nullptr, *x_wavg = nullptr, *f_wavg = nullptr, *tmp = nullptr;
    double *R = nullptr, *F = nullptr;
    ~MixState();
};

}  // namespace sgpu

struct sgpu_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int Nx = 0, Ny = 0, Nz = 0, FDn = 0;
    long Nd = 0;
    double cx[sgpu::kMaxFDn + 1] = {0}, cy[sgpu::kMaxFDn + 1] = {0}, cz[sgpu::kMaxFDn + 1] = {0};
    double dV = 0.0;
    int nspin_veff = 0;
    double *veff64 = nullptr;  // Nd * nspin
    float *veff32 = nullptr;
    sgpu::Nonlocal nl;
    bool has_nl = false;
    cublasHandle_t cublas = nullptr;
    cusolverDnHandle_t cusolver = nullptr;
    cusolverDnParams_t xparams = nullptr;   // 64-bit cuSOLVER API parameters (batched syev)
    void *xhost = nullptr;                  // its host workspace
    size_t xhost_bytes = 0;
    int rr_batched = 1;                     // k-point CheFSI pass: batched Rayleigh-Ritz step
                                            // for blocks of one width (sgpu_set_rr_batched)
    sgpu::Workspace ws[16];    // grow-only scratch slots (see enum WsSlot)
    sgpu::MixState *mix = nullptr;
    sgpu::KpointState *kp = nullptr;  // cell lengths and image coordinates (k-point calls)
    sgpu::SetupState *setup = nullptr;  // pseudopotential tables (set-up calls)
    int stencil_variant = 0;   // FP32 stencil kernel variant (autotune.cu)
    bool stencil_tuned = false;
    int nl_apply_variant = 0;  // real nonlocal apply: 0 per point over all columns, 1 staged,
                               // 2 per point with the Chi values hoisted, 3 dense per chunk,
                               // 4 per range with the output tile in shared memory
    int nl_project_variant = 0;  // FP32 projection: 0 per image segment, 1 per point range
    bool nl_fuse = false;  // FP32 filter: project each new iterate inside the range apply that
                           // finishes it (one projection launch per filter, not per degree)
    int nl_fuse_cpl = 2;   // fused apply form, chosen by the tuner: columns per lane of the
                           // CUDA-core kernel (2 or 4), or 3 for the tensor-core kernel
    int gemm_mode = 0;  // FP32-block products: 0 cuBLAS FP32 GEMM (BF16x9 emulation where
                        // cuBLAS expects a gain), 1 the same with eager emulation, 2 the
                        // library's three-part BF16 split on the tensor cores (cuBLAS GEMMs)
    int eig_mode = 0;   // subspace eigensolver: 0 dsygvd, 1 Cholesky reduction + dsyevd,
                        // 2 Cholesky reduction + Jacobi dsyevj (sgpu_set_eig_solver)
    int rr_tc = 1;      // Rayleigh-Ritz products on the library's own tcgen05 split-slice
                        // kernels (rr_tc.cu): 1 (default) for FP32 blocks (FP32-accurate) and
                        // the mixed SCF's FP64 phase (FP64-accurate), 2 also for plain FP64
                        // calls; 0 cuBLAS
    int zpair_on = 1;   // complex64 stencil: the two-points-per-thread kernel (1) or the
                        // one-point kernel (0) (sgpu_set_zstencil_pairs)
    double tune_fused_ms = 0.0;  // last timing of the fused apply + projection (chosen form)
    double tune_fused_cpl_ms[2] = {0, 0};  // last timings of the 2- and 4-column forms
    double tune_fused_tc_ms = 0.0;         // last timing of the tensor-core form
    double tune_apply_ms[5] = {0, 0, 0, 0, 0}, tune_project_ms[2] = {0, 0};  // last timings
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int *kstatus = nullptr;    // device word: bits set by kernel waits that ran out
    // host-array filter pipeline (capi.cu): copy-in and copy-out streams, and per buffer slot
    // the events "input landed", "filtered", "slot free again"
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    cudaEvent_t pipe_ev[3][3] = {};
    float last_filter_ms = 0.f;
    // optional per-kernel timing (sgpu_profile_enable): events recorded around launches on
    // the context stream, resolved by sgpu_profile_read
    bool prof_on = false;
    std::vector<cudaEvent_t> prof_pool;
    size_t prof_next = 0;
    struct ProfRec { int kind; cudaEvent_t a, b; };
    std::vector<ProfRec> prof_pending;
    double prof_ms[SGPU_KERNEL_KINDS] = {0};
    long prof_n[SGPU_KERNEL_KINDS] = {0};
    long launches = 0;  // kernels launched by this context since the last profile reset
};

namespace sgpu {

enum WsSlot {
    WS_STAGE_A = 0, WS_STAGE_B, WS_STAGE_C, WS_ALPHA, WS_MISC, WS_EIG, WS_POIS, WS_MIX,
    WS_RED, WS_RHS, WS_SCF, WS_SCF2, WS_ALPHA2, WS_SPLIT_A, WS_SPLIT_B, WS_TC_PART,
    WS_COUNT
};

// grow-only device scratch
int ws_get(sgpu_ctx *ctx, int slot, size_t bytes, void **out);
int fp64_fma_rate(sgpu_ctx *ctx, double *tflops);

// profiling: returns an event pair recorded around a launch of `kind` (or nulls when off)
struct ProfScope {
    sgpu_ctx *ctx;
    int kind;
    cudaStream_t st;
    cudaEvent_t b = nullptr;
    ProfScope(sgpu_ctx *c, int k, cudaStream_t s);
    ~ProfScope();
};

// read and clear ctx->kstatus (synchronises the stream); SGPU_ERR_KERNEL_WAIT when set
int kernel_status_check(sgpu_ctx *ctx, int *status = nullptr);
// one block waiting (bounded, about a millisecond) on a barrier phase nothing completes; the
// wait runs out and sets bit 2 of ctx->kstatus (stencil.cu)
int wait_bound_check(sgpu_ctx *ctx);

// memory-kind query: true when p is device (or managed) memory this context can use directly
bool is_device_ptr(const void *p);

// ---- stencil (stencil.cu)
// out[:, n] = s1 * ( a*Lap + bv*diag(v) + c*I ) x[:, n]  +  s2 * z[:, n]
// (z may be null; v may be null). All arrays column-major with the given leading dims.
template <typename T>
int launch_stencil(sgpu_ctx *ctx, int ncol, double a, double bv, double c, const T *v,
                   const T *x, long ldx, T *out, long ldo, double s1, double s2, const T *z,
                   long ldz, cudaStream_t st);

// ---- nonlocal (nonlocal.cu)
// alpha is (ntot x lda) projector-major: alpha[row * lda + n]; lda from nonlocal_alpha_ld
long nonlocal_alpha_ld(int ncol, int elem_bytes);
template <typename T>
int launch_nonlocal_project(sgpu_ctx *ctx, int ncol, const T *x, long ldx, T *alpha, long lda,
                            cudaStream_t st);
// alpha += Chi^T x (no dV, no Gamma: ones holds ntot ones), the segment kernel in FP64
int launch_nonlocal_project_plain(sgpu_ctx *ctx, int ncol, const double *x, long ldx,
                                  double *alpha, long lda, const double *ones, cudaStream_t st);

// ---- forces (forces.cu)
// out[:, n] = D1 derivative of x[:, n] along dir (0 x, 1 y, 2 z), periodic; w[1..FDn] are the
// first-derivative weights of that direction (w[0] unused)
int launch_gradient(sgpu_ctx *ctx, int ncol, const double *x, long ldx, double *out, long ldo,
                    int dir, const double *w, cudaStream_t st);
template <typename T>
int launch_nonlocal_apply(sgpu_ctx *ctx, int ncol, const T *alpha, long lda, double scale,
                          T *out, long ldo, cudaStream_t st);
// the range apply of alpha into out with the projection of the finished out fused:
// alpha_next (zeroed by the caller; may be null) += dV * Gamma * Chi^T out
int launch_nonlocal_apply_project(sgpu_ctx *ctx, int ncol, const float *alpha, long lda,
                                  double scale, float *out, long ldo, float *alpha_next,
                                  cudaStream_t st);
// the same with the tensor-core kernel (nonlocal_tc.cu); needs the tensor-core range tables
int launch_nonlocal_apply_project_tc(sgpu_ctx *ctx, int ncol, const float *alpha, long lda,
                                     double scale, float *out, long ldo, float *alpha_next,
                                     cudaStream_t st);
bool nonlocal_tc_ready(const sgpu_ctx *ctx);
// builds the tensor-core range tables from the point CSR of nonlocal_upload
int nonlocal_tc_build(Nonlocal &nl, int Nx, int Ny, const std::vector<int> &covpts,
                      const std::vector<int> &covptr, const std::vector<long> &ent_chi,
                      const std::vector<int4> &ent_meta, const double *chi);
int nonlocal_upload(sgpu_ctx *ctx, int natom, const int *ip_displ, const double *gamma,
                    int nimg, const int *img_atom, const int *img_ndc, const int *grid_pos,
                    const double *chi);
void nonlocal_free(Nonlocal &nl);

// ---- Hamiltonian and filter (chefsi.cu)
template <typename T>
int hamiltonian_dev(sgpu_ctx *ctx, int spin, int ncol, double c, const T *x, long ldx, T *hx,
                    long ldh, double s1, double s2, const T *z, long ldz, cudaStream_t st,
                    const T *alpha_in = nullptr, T *alpha_out = nullptr);
// whether the FP32 filter carries the projections across degrees (fused range apply)
bool filter_fuses_projection(sgpu_ctx *ctx);
template <typename T>
int chebyshev_dev(sgpu_ctx *ctx, int spin, T *X, long ldx, T *Y, long ldy, int ncol, int m,
                  double a, double b, double a0, cudaStream_t st);
// first m-k64 degrees in FP32 on (X32, Y32), last k64 in FP64; result in Y64 (ld = Nd)
int chebyshev_graded(sgpu_ctx *ctx, int spin, float *X32, float *Y32, double *X64,
                     double *Y64, int ncol, int m, int k64, double a, double b, double a0,
                     cudaStream_t st);

// ---- Rayleigh-Ritz (subspace.cu)
int project_f64(sgpu_ctx *ctx, int ncol, const double *Y, long ldy, const double *HY,
                long ldh, double *Hp, double *Mp, cudaStream_t st);
int project_f32(sgpu_ctx *ctx, int ncol, const float *Y, long ldy, const float *HY, long ldh,
                double *Hp, double *Mp, cudaStream_t st);
int generalized_eig(sgpu_ctx *ctx, int n, double *Hp, double *Mp, double *lambda_dev,
                    cudaStream_t st);
int ensure_solver_handles(sgpu_ctx *ctx);
template <typename T>
int tc_project(sgpu_ctx *ctx, int ncol, const T *Y, long ldy, const T *HY, long ldh, double *Hp,
               double *Mp, bool fp64_accurate, cudaStream_t st);
template <typename T>
int tc_rotate(sgpu_ctx *ctx, int ncol, const T *Y, long ldy, const double *Q, int ldq, T *X,
              long ldx, bool fp64_accurate, cudaStream_t st);
int rotate_f64(sgpu_ctx *ctx, int ncol, const double *Y, long ldy, const double *Q, double *X,
               long ldx, cudaStream_t st);
int cholqr_f64(sgpu_ctx *ctx, int ncol, double *Y, long ldy, cudaStream_t st);
int standard_eig(sgpu_ctx *ctx, int n, double *Hp, double *lambda_dev, cudaStream_t st);
int rotate_f32(sgpu_ctx *ctx, int ncol, const float *Y, long ldy, const double *Q, float *X,
               long ldx, cudaStream_t st);

// ---- SCF-side operations (scf_ops.cu), all FP64 vectors of Nd
int dot_dev(sgpu_ctx *ctx, const double *a, const double *b, long n, double *d_out,
            cudaStream_t st);  // b == nullptr: plain sum
int dot_host(sgpu_ctx *ctx, const double *a, const double *b, long n, double *out,
             cudaStream_t st);
template <typename T>
int density_dev(sgpu_ctx *ctx, const T *psi, long ld, int ncol, const double *w_dev,
                double *rho, cudaStream_t st);
int lda_pw_dev(sgpu_ctx *ctx, const double *rho, const double *rho_core, double rhotol,
               double *vxc, double *exc, cudaStream_t st);
int axpby_dev(sgpu_ctx *ctx, long n, double a, const double *x, double b, const double *y,
              double *z, cudaStream_t st);
int remove_mean_dev(sgpu_ctx *ctx, double *x, cudaStream_t st);
// ||out - in|| / ||out|| over n values (n <= 0: Nd)
int scf_error_dev(sgpu_ctx *ctx, const double *out, const double *in, double *err,
                  cudaStream_t st, long n = 0);
// spin-polarised LDA (PW92) on the spin densities; rho_core may be null
int lsda_pw_dev(sgpu_ctx *ctx, const double *up, const double *dn, const double *rho_core,
                double rhotol, double *vxc_up, double *vxc_dn, double *exc, cudaStream_t st);
int aar_dev(sgpu_ctx *ctx, double c, double *x, const double *b, double omega, double beta,
            int m, int p, double tol, int max_iter, int *iters, cudaStream_t st);
int poisson_dev(sgpu_ctx *ctx, const double *rho, const double *b, double *phi, double tol,
                int max_iter, int *iters, cudaStream_t st);
int kerker_dev(sgpu_ctx *ctx, const double *f, double a, double kTF, double idiemac,
               double tol, double *Pf, cudaStream_t st);
int mixing_init(sgpu_ctx *ctx, const MixParams &prm, const double *x0);
int mixing_step(sgpu_ctx *ctx, int iter_count, double *g, cudaStream_t st);
// rho (+)= sum_n w_n |psi_n|^2 over ncol complex columns (CT = double2 or float2)
template <typename CT>
int density_z_dev(sgpu_ctx *ctx, const CT *psi, long ld, int ncol, const double *w_dev,
                  double *rho, bool accumulate, cudaStream_t st);

// ---- SCF pieces shared by the Gamma-point and k-point drivers (scf.cu)
// uniform [-0.5, 0.5) values from (seed, index)
void init_orbitals(sgpu_ctx *ctx, double *X, long n, unsigned long long seed, int blocks,
                   cudaStream_t st);
double smearing(double beta, double lam, double ef, int type);
// Fermi level: sum_i w_i f(lam_i) = nelec; *status = 1 when no bracket is found
double fermi_level(const std::vector<double> &lam, const std::vector<double> &w, double nelec,
                   double beta, int type, double x1, double x2, double tol, int max_iter,
                   int *status);
int lanczos_run(sgpu_ctx *ctx, long len, const std::function<int(const double *, double *)> &apply,
                const double *x0, double tol, int maxit, double *eigmin, double *eigmax,
                cudaStream_t st);
// complex (k-point) Rayleigh-Ritz pieces (kpoint.cu)
template <typename CT>
int hamiltonian_z(sgpu_ctx *ctx, int spin, const double *k, int ncol, double c, const CT *x,
                  long ldx, CT *hx, long ldh, double s1, double s2, const CT *z, long ldz,
                  cudaStream_t st);
int kpoint_set_phases(sgpu_ctx *ctx, const double *k, cudaStream_t st);
template <typename CT>
int chefsi_batched(sgpu_ctx *ctx, int nblk, const sgpu_filter_block *blk, int m,
                   double *lambda, cudaStream_t st);
// complex64 filter of b32, complex128 Rayleigh-Ritz step on b64 (the same blocks in complex128
// storage), Ritz vectors narrowed back into b32's X
int chefsi_batched_graded(sgpu_ctx *ctx, int nblk, const sgpu_filter_block *b32,
                          const sgpu_filter_block *b64, int m, double *lambda, cudaStream_t st);

// ---- elementwise helpers (util.cu)
template <typename T>
int swap_blocks(T *a, long lda, T *b, long ldb, long rows, int ncol, cudaStream_t st);
// dst[:, n] = (Tout) src[:, n] for column blocks of `rows` rows
template <typename Tin, typename Tout>
int convert_cols(const Tin *src, long lds, Tout *dst, long ldd, long rows, int ncol,
                 cudaStream_t st);

}  // namespace sgpu
