// Kleinman-Bylander nonlocal projector apply, split in two device passes.
//
// Reference: Vnl_vec_mult (src/nlocVecRoutines.c:798-886), per atom J:
//   alpha_J = dV * Chi_Jᵀ x[grid_pos_J]          (gather + dgemm, :806-833)
//   alpha_J[j, n] *= Gamma_J[j]                   (:843-866)
//   Hx[grid_pos_J] += Chi_J alpha_J               (dgemm + scatter, :869-884)
//
// GPU form:
//   * project: one thread block per (atom image, projector group, column group); threads
//     stride over the image's grid points, gather x, accumulate in registers, then one
//     block-level reduction and one atomic add per output into alpha (ntot x ncol,
//     projector index fastest). dV and Gamma are folded into that add.
//   * apply: owner-computes over a CSR of covered grid points, so each output element is
//     written by exactly one thread (no atomics on the orbital block, overlapping spheres
//     are summed in registers).
#include <algorithm>
#include <numeric>

#include "sgpu_internal.h"

namespace sgpu {
namespace {

constexpr int kProjThreads = 256;

template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// alpha layout: alpha[row * lda + n], row = IP_displ[atom] + j (projector), n = column;
// lda is a multiple of the apply's column block so rows can be read as vectors.
//
// Projection as a gathered GEMM: block = (atom image g, group of NC columns). The image's
// points are walked in chunks of PCH: the block gathers x[grid_pos[chunk], n0:n0+NC] into
// shared memory (coalesced along points for each column) together with the chunk's Chi rows,
// then thread (n, jg) accumulates alpha[j, n] for j = jg, jg + 8, ... over the chunk. One
// atomic add per (projector, column) output at the end, with dV * Gamma folded in.
template <typename T, int PCH, int NC, int MAXJ>
__global__ void __launch_bounds__(kProjThreads)
    k_nl_project(const int *__restrict__ img_atom, const int *__restrict__ img_ndc,
                 const long *__restrict__ img_off, const long *__restrict__ img_chi_off,
                 const int *__restrict__ grid_pos, const T *__restrict__ chi,
                 const int *__restrict__ ip_displ, const T *__restrict__ gamma, int ncol,
                 const T *__restrict__ x, long ldx, T *__restrict__ alpha, long lda, T dV)
{
    static_assert(kProjThreads == 8 * NC, "thread (n, jg) layout: NC columns x 8 groups");
    constexpr int JG = 8;
    constexpr int NJ = (MAXJ + JG - 1) / JG;
    __shared__ T xs[NC][PCH + 1];     // +1: conflict-free reads across columns
    __shared__ T cs[MAXJ][PCH];
    const int g = blockIdx.x;
    const int n0 = blockIdx.y * NC;
    const int a = img_atom[g];
    const int np = ip_displ[a + 1] - ip_displ[a];
    const int ndc = img_ndc[g];
    const int *__restrict__ gp = grid_pos + img_off[g];
    const T *__restrict__ ch = chi + img_chi_off[g];
    const int t = threadIdx.x;
    const int n = t % NC, jg = t / NC;
    T acc[NJ];
#pragma unroll
    for (int u = 0; u < NJ; u++) acc[u] = T(0);

    for (int i0 = 0; i0 < ndc; i0 += PCH) {
        const int cnt = min(PCH, ndc - i0);
        __syncthreads();  // previous chunk consumed
        // gather: PCH points x NC columns, kProjThreads threads
        for (int e = t; e < PCH * NC; e += kProjThreads) {
            const int i = e % PCH, c = e / PCH;
            T v = T(0);
            if (i < cnt && n0 + c < ncol) v = __ldg(x + (long)(n0 + c) * ldx + gp[i0 + i]);
            xs[c][i] = v;
        }
        for (int e = t; e < PCH * MAXJ; e += kProjThreads) {
            const int i = e % PCH, j = e / PCH;
            cs[j][i] = (i < cnt && j < np) ? __ldg(ch + (long)j * ndc + i0 + i) : T(0);
        }
        __syncthreads();
#pragma unroll 4
        for (int i = 0; i < PCH; i++) {
            const T xv = xs[n][i];
#pragma unroll
            for (int u = 0; u < NJ; u++)
                if (jg + u * JG < MAXJ) acc[u] += cs[jg + u * JG][i] * xv;
        }
    }
    if (n0 + n < ncol) {
#pragma unroll
        for (int u = 0; u < NJ; u++) {
            const int j = jg + u * JG;
            if (j < np) {
                const int row = ip_displ[a] + j;
                atomicAdd(alpha + (long)row * lda + n0 + n, dV * gamma[row] * acc[u]);
            }
        }
    }
}

template <typename T, int CB>
struct VecOf;
template <> struct VecOf<float, 4> { using type = float4; };
template <> struct VecOf<double, 2> { using type = double2; };

// Apply: one thread per covered grid point and CB columns; alpha rows are read as vectors
// (VW elements per load, broadcast across the warp when neighbouring points share an atom).
template <typename T, int CB, int VW>
__global__ void __launch_bounds__(256)
    k_nl_apply(int ncov, const int *__restrict__ cov_pt, const int *__restrict__ cov_ptr,
               const long *__restrict__ ent_chi, const int4 *__restrict__ ent_meta,
               const T *__restrict__ chi, int ncol, const T *__restrict__ alpha, long lda,
               T scale, T *__restrict__ out, long ldo)
{
    using V = typename VecOf<T, VW>::type;
    const int cidx = blockIdx.x * blockDim.x + threadIdx.x;
    if (cidx >= ncov) return;
    const int n0 = blockIdx.y * CB;
    T acc[CB];
#pragma unroll
    for (int c = 0; c < CB; c++) acc[c] = T(0);
    const int e1 = cov_ptr[cidx + 1];
    for (int e = cov_ptr[cidx]; e < e1; e++) {
        const int4 meta = ent_meta[e];  // (first projector row, projector count, image size)
        const int ip = meta.x, np = meta.y, ndc = meta.z;
        const T *__restrict__ ch = chi + ent_chi[e];
        for (int j = 0; j < np; j++) {
            const T cv = __ldg(ch + (long)j * ndc);
            const V *__restrict__ al = reinterpret_cast<const V *>(alpha + (long)(ip + j) * lda + n0);
#pragma unroll
            for (int c = 0; c < CB / VW; c++) {
                const V av = __ldg(al + c);
                const T *ae = reinterpret_cast<const T *>(&av);
#pragma unroll
                for (int w = 0; w < VW; w++) acc[c * VW + w] += cv * ae[w];
            }
        }
    }
    const long p = cov_pt[cidx];
#pragma unroll
    for (int c = 0; c < CB; c++)
        if (n0 + c < ncol) out[(long)(n0 + c) * ldo + p] += scale * acc[c];
}

template <typename T>
const T *chi_of(const Nonlocal &nl);
template <>
const double *chi_of<double>(const Nonlocal &nl) { return nl.chi64; }
template <>
const float *chi_of<float>(const Nonlocal &nl) { return nl.chi32; }
template <typename T>
const T *gamma_of(const Nonlocal &nl);
template <>
const double *gamma_of<double>(const Nonlocal &nl) { return nl.gamma64; }
template <>
const float *gamma_of<float>(const Nonlocal &nl) { return nl.gamma32; }

}  // namespace

template <typename T>
static constexpr int apply_cb() { return sizeof(T) == 4 ? 16 : 8; }

long nonlocal_alpha_ld(int ncol, int elem_bytes)
{
    const int cb = elem_bytes == 4 ? 16 : 8;
    return ((long)ncol + cb - 1) / cb * cb;
}

template <typename T, int MAXJ>
static void project_launch(sgpu_ctx *ctx, int ncol, const T *x, long ldx, T *alpha, long lda,
                           cudaStream_t st)
{
    constexpr int NC = kProjThreads / 8, PCH = sizeof(T) == 4 ? 128 : 64;
    const Nonlocal &nl = ctx->nl;
    const int ncb = (ncol + NC - 1) / NC;
    for (int cb0 = 0; cb0 < ncb; cb0 += 65535) {
        int nb = std::min(65535, ncb - cb0);
        dim3 grid(nl.nimg, nb);
        ProfScope ps(ctx, SGPU_KERNEL_NL_PROJECT, st);
        k_nl_project<T, PCH, NC, MAXJ><<<grid, kProjThreads, 0, st>>>(
            nl.img_atom, nl.img_ndc, nl.img_off, nl.img_chi_off, nl.grid_pos, chi_of<T>(nl),
            nl.ip_displ, gamma_of<T>(nl), ncol - cb0 * NC, x + (long)cb0 * NC * ldx, ldx,
            alpha + (long)cb0 * NC, lda, (T)ctx->dV);
    }
}

template <typename T>
int launch_nonlocal_project(sgpu_ctx *ctx, int ncol, const T *x, long ldx, T *alpha, long lda,
                            cudaStream_t st)
{
    const Nonlocal &nl = ctx->nl;
    if (!ctx->has_nl || nl.nimg == 0 || ncol <= 0) return SGPU_OK;
    if (nl.max_np <= 9)
        project_launch<T, 9>(ctx, ncol, x, ldx, alpha, lda, st);
    else if (nl.max_np <= 18)
        project_launch<T, 18>(ctx, ncol, x, ldx, alpha, lda, st);
    else if (nl.max_np <= 32)
        project_launch<T, 32>(ctx, ncol, x, ldx, alpha, lda, st);
    else {
        set_error("nonlocal: more than 32 projectors per atom is not built");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

template <typename T>
int launch_nonlocal_apply(sgpu_ctx *ctx, int ncol, const T *alpha, long lda, double scale,
                          T *out, long ldo, cudaStream_t st)
{
    const Nonlocal &nl = ctx->nl;
    if (!ctx->has_nl || nl.ncov == 0 || ncol <= 0) return SGPU_OK;
    constexpr int CB = apply_cb<T>();
    constexpr int VW = sizeof(T) == 4 ? 4 : 2;
    const int ncb = (ncol + CB - 1) / CB;
    for (int cb0 = 0; cb0 < ncb; cb0 += 65535) {
        int nb = std::min(65535, ncb - cb0);
        dim3 grid((nl.ncov + 255) / 256, nb);
        ProfScope ps(ctx, SGPU_KERNEL_NL_APPLY, st);
        k_nl_apply<T, CB, VW><<<grid, 256, 0, st>>>(
            nl.ncov, nl.cov_pt, nl.cov_ptr, nl.ent_chi, nl.ent_meta, chi_of<T>(nl),
            ncol - cb0 * CB, alpha + (long)cb0 * CB, lda, (T)scale,
            out + (long)cb0 * CB * ldo, ldo);
    }
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

template int launch_nonlocal_project<double>(sgpu_ctx *, int, const double *, long, double *,
                                             long, cudaStream_t);
template int launch_nonlocal_project<float>(sgpu_ctx *, int, const float *, long, float *, long,
                                            cudaStream_t);
template int launch_nonlocal_apply<double>(sgpu_ctx *, int, const double *, long, double,
                                           double *, long, cudaStream_t);
template int launch_nonlocal_apply<float>(sgpu_ctx *, int, const float *, long, double, float *,
                                          long, cudaStream_t);

void nonlocal_free(Nonlocal &nl)
{
    void *ptrs[] = {nl.ip_displ, nl.img_atom, nl.img_ndc, nl.img_off, nl.img_chi_off,
                    nl.grid_pos, nl.chi64,    nl.chi32,   nl.gamma64, nl.gamma32,
                    nl.cov_pt,   nl.cov_ptr,  nl.ent_chi, nl.ent_meta};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    nl = Nonlocal();
}

namespace {
template <typename T>
int upload(T **dst, const T *src, size_t n)
{
    SGPU_CUDA_TRY(cudaMalloc((void **)dst, sizeof(T) * (n > 0 ? n : 1)));
    if (n > 0) SGPU_CUDA_TRY(cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice));
    return SGPU_OK;
}
}  // namespace

int nonlocal_upload(sgpu_ctx *ctx, int natom, const int *ip_displ, const double *gamma,
                    int nimg, const int *img_atom, const int *img_ndc, const int *grid_pos,
                    const double *chi)
{
    Nonlocal nl;
    nl.natom = natom;
    nl.nimg = nimg;
    nl.ntot = ip_displ[natom];
    for (int a = 0; a < natom; a++) {
        const int np = ip_displ[a + 1] - ip_displ[a];
        if (np < 0) {
            set_error("set_nonlocal: ip_displ must be non-decreasing");
            return SGPU_ERR_ARG;
        }
        nl.max_np = std::max(nl.max_np, np);
    }
    std::vector<long> off(nimg), chioff(nimg);
    long npos = 0, nchi = 0;
    for (int g = 0; g < nimg; g++) {
        if (img_atom[g] < 0 || img_atom[g] >= natom || img_ndc[g] < 0) {
            set_error("set_nonlocal: image " + std::to_string(g) + " has a bad atom or size");
            return SGPU_ERR_ARG;
        }
        off[g] = npos;
        chioff[g] = nchi;
        npos += img_ndc[g];
        nchi += (long)img_ndc[g] * (ip_displ[img_atom[g] + 1] - ip_displ[img_atom[g]]);
    }
    for (long i = 0; i < npos; i++) {
        if (grid_pos[i] < 0 || grid_pos[i] >= ctx->Nd) {
            set_error("set_nonlocal: grid position out of range");
            return SGPU_ERR_ARG;
        }
    }
    nl.npos = npos;
    nl.nchi = nchi;

    // point CSR: entries (image, local index) bucketed by grid point
    std::vector<int> count(ctx->Nd + 1, 0);
    for (long i = 0; i < npos; i++) count[grid_pos[i] + 1]++;
    std::vector<int> covpts;
    std::vector<int> covptr(1, 0);
    for (long p = 0; p < ctx->Nd; p++) {
        if (count[p + 1] > 0) {
            covpts.push_back((int)p);
            covptr.push_back(covptr.back() + count[p + 1]);
        }
    }
    std::vector<int> slot(ctx->Nd, -1);
    for (size_t c = 0; c < covpts.size(); c++) slot[covpts[c]] = covptr[c];
    std::vector<long> ent_chi(npos);
    std::vector<int4> ent_meta(npos);
    for (int g = 0; g < nimg; g++) {
        const int a = img_atom[g];
        const int ip = ip_displ[a], np = ip_displ[a + 1] - ip_displ[a];
        for (int ii = 0; ii < img_ndc[g]; ii++) {
            const int p = grid_pos[off[g] + ii];
            const int e = slot[p]++;
            ent_chi[e] = chioff[g] + ii;
            ent_meta[e] = make_int4(ip, np, img_ndc[g], g);
        }
    }
    nl.ncov = (int)covpts.size();
    nl.nent = npos;

    std::vector<float> chi32(nchi), gamma32(nl.ntot);
    for (long i = 0; i < nchi; i++) chi32[i] = (float)chi[i];
    for (int i = 0; i < nl.ntot; i++) gamma32[i] = (float)gamma[i];

    int rc = SGPU_OK;
#define UP(dst, src, n)                                                                      \
    if (rc == SGPU_OK) rc = upload(&nl.dst, src, n)
    UP(ip_displ, ip_displ, (size_t)natom + 1);
    UP(img_atom, img_atom, (size_t)nimg);
    UP(img_ndc, img_ndc, (size_t)nimg);
    UP(img_off, off.data(), (size_t)nimg);
    UP(img_chi_off, chioff.data(), (size_t)nimg);
    UP(grid_pos, grid_pos, (size_t)npos);
    UP(chi64, chi, (size_t)nchi);
    UP(chi32, chi32.data(), (size_t)nchi);
    UP(gamma64, gamma, (size_t)nl.ntot);
    UP(gamma32, gamma32.data(), (size_t)nl.ntot);
    UP(cov_pt, covpts.data(), covpts.size());
    UP(cov_ptr, covptr.data(), covptr.size());
    UP(ent_chi, ent_chi.data(), ent_chi.size());
    UP(ent_meta, ent_meta.data(), ent_meta.size());
#undef UP
    if (rc != SGPU_OK) {
        nonlocal_free(nl);
        return rc;
    }
    nonlocal_free(ctx->nl);
    ctx->nl = nl;
    ctx->has_nl = true;
    return SGPU_OK;
}

}  // namespace sgpu
