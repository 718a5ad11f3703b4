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
constexpr int kProjNPB = 8;  // projectors per block
constexpr int kProjCB = 4;   // columns per block
constexpr int kApplyCB = 4;  // columns per thread in the apply

template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
__global__ void __launch_bounds__(kProjThreads)
    k_nl_project(const int *__restrict__ img_atom, const int *__restrict__ img_ndc,
                 const long *__restrict__ img_off, const long *__restrict__ img_chi_off,
                 const int *__restrict__ grid_pos, const T *__restrict__ chi,
                 const int *__restrict__ ip_displ, const T *__restrict__ gamma, int ntot,
                 int ncol, const T *__restrict__ x, long ldx, T *__restrict__ alpha, T dV)
{
    const int g = blockIdx.x;
    const int jg = blockIdx.y * kProjNPB;
    const int n0 = blockIdx.z * kProjCB;
    const int a = img_atom[g];
    const int np = ip_displ[a + 1] - ip_displ[a];
    if (jg >= np) return;
    const int ndc = img_ndc[g];
    const int *__restrict__ gp = grid_pos + img_off[g];
    const T *__restrict__ ch = chi + img_chi_off[g];

    T acc[kProjNPB][kProjCB];
#pragma unroll
    for (int j = 0; j < kProjNPB; j++)
#pragma unroll
        for (int c = 0; c < kProjCB; c++) acc[j][c] = T(0);

    for (int ii = threadIdx.x; ii < ndc; ii += kProjThreads) {
        const long p = gp[ii];
        T xv[kProjCB];
#pragma unroll
        for (int c = 0; c < kProjCB; c++)
            xv[c] = (n0 + c < ncol) ? __ldg(x + (long)(n0 + c) * ldx + p) : T(0);
#pragma unroll
        for (int j = 0; j < kProjNPB; j++) {
            if (jg + j < np) {
                const T cv = __ldg(ch + (long)(jg + j) * ndc + ii);
#pragma unroll
                for (int c = 0; c < kProjCB; c++) acc[j][c] += cv * xv[c];
            }
        }
    }

    __shared__ T red[kProjThreads / 32][kProjNPB * kProjCB];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < kProjNPB; j++)
#pragma unroll
        for (int c = 0; c < kProjCB; c++) {
            T v = warp_sum(acc[j][c]);
            if (lane == 0) red[warp][j * kProjCB + c] = v;
        }
    __syncthreads();
    if (threadIdx.x < kProjNPB * kProjCB) {
        const int j = threadIdx.x / kProjCB, c = threadIdx.x % kProjCB;
        if (jg + j < np && n0 + c < ncol) {
            T s = T(0);
#pragma unroll
            for (int w = 0; w < kProjThreads / 32; w++) s += red[w][threadIdx.x];
            const int row = ip_displ[a] + jg + j;
            atomicAdd(alpha + (long)(n0 + c) * ntot + row, dV * gamma[row] * s);
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(256)
    k_nl_apply(int ncov, const int *__restrict__ cov_pt, const int *__restrict__ cov_ptr,
               const int *__restrict__ ent_img, const int *__restrict__ ent_i,
               const int *__restrict__ img_atom, const int *__restrict__ img_ndc,
               const long *__restrict__ img_chi_off, const T *__restrict__ chi,
               const int *__restrict__ ip_displ, int ntot, int ncol,
               const T *__restrict__ alpha, T scale, T *__restrict__ out, long ldo)
{
    const int cidx = blockIdx.x * blockDim.x + threadIdx.x;
    if (cidx >= ncov) return;
    const int n0 = blockIdx.y * kApplyCB;
    T acc[kApplyCB];
#pragma unroll
    for (int c = 0; c < kApplyCB; c++) acc[c] = T(0);
    const int e1 = cov_ptr[cidx + 1];
    for (int e = cov_ptr[cidx]; e < e1; e++) {
        const int g = ent_img[e], ii = ent_i[e];
        const int a = img_atom[g];
        const int ip = ip_displ[a], np = ip_displ[a + 1] - ip;
        const int ndc = img_ndc[g];
        const T *__restrict__ ch = chi + img_chi_off[g] + ii;
        for (int j = 0; j < np; j++) {
            const T cv = __ldg(ch + (long)j * ndc);
#pragma unroll
            for (int c = 0; c < kApplyCB; c++)
                if (n0 + c < ncol) acc[c] += cv * __ldg(alpha + (long)(n0 + c) * ntot + ip + j);
        }
    }
    const long p = cov_pt[cidx];
#pragma unroll
    for (int c = 0; c < kApplyCB; c++)
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
int launch_nonlocal_project(sgpu_ctx *ctx, int ncol, const T *x, long ldx, T *alpha,
                            cudaStream_t st)
{
    const Nonlocal &nl = ctx->nl;
    if (!ctx->has_nl || nl.nimg == 0 || ncol <= 0) return SGPU_OK;
    const int njg = (nl.max_np + kProjNPB - 1) / kProjNPB;
    const int ncb = (ncol + kProjCB - 1) / kProjCB;
    for (int cb0 = 0; cb0 < ncb; cb0 += 65535) {
        int nb = std::min(65535, ncb - cb0);
        dim3 grid(nl.nimg, njg, nb);
        ProfScope ps(ctx, SGPU_KERNEL_NL_PROJECT, st);
        k_nl_project<T><<<grid, kProjThreads, 0, st>>>(
            nl.img_atom, nl.img_ndc, nl.img_off, nl.img_chi_off, nl.grid_pos, chi_of<T>(nl),
            nl.ip_displ, gamma_of<T>(nl), nl.ntot, ncol - cb0 * kProjCB,
            x + (long)cb0 * kProjCB * ldx, ldx, alpha + (long)cb0 * kProjCB * nl.ntot,
            (T)ctx->dV);
    }
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

template <typename T>
int launch_nonlocal_apply(sgpu_ctx *ctx, int ncol, const T *alpha, double scale, T *out,
                          long ldo, cudaStream_t st)
{
    const Nonlocal &nl = ctx->nl;
    if (!ctx->has_nl || nl.ncov == 0 || ncol <= 0) return SGPU_OK;
    const int ncb = (ncol + kApplyCB - 1) / kApplyCB;
    for (int cb0 = 0; cb0 < ncb; cb0 += 65535) {
        int nb = std::min(65535, ncb - cb0);
        dim3 grid((nl.ncov + 255) / 256, nb);
        ProfScope ps(ctx, SGPU_KERNEL_NL_APPLY, st);
        k_nl_apply<T><<<grid, 256, 0, st>>>(
            nl.ncov, nl.cov_pt, nl.cov_ptr, nl.ent_img, nl.ent_i, nl.img_atom, nl.img_ndc,
            nl.img_chi_off, chi_of<T>(nl), nl.ip_displ, nl.ntot, ncol - cb0 * kApplyCB,
            alpha + (long)cb0 * kApplyCB * nl.ntot, (T)scale, out + (long)cb0 * kApplyCB * ldo,
            ldo);
    }
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

template int launch_nonlocal_project<double>(sgpu_ctx *, int, const double *, long, double *,
                                             cudaStream_t);
template int launch_nonlocal_project<float>(sgpu_ctx *, int, const float *, long, float *,
                                            cudaStream_t);
template int launch_nonlocal_apply<double>(sgpu_ctx *, int, const double *, double, double *,
                                           long, cudaStream_t);
template int launch_nonlocal_apply<float>(sgpu_ctx *, int, const float *, double, float *, long,
                                          cudaStream_t);

void nonlocal_free(Nonlocal &nl)
{
    void *ptrs[] = {nl.ip_displ, nl.img_atom, nl.img_ndc, nl.img_off, nl.img_chi_off,
                    nl.grid_pos, nl.chi64,    nl.chi32,   nl.gamma64, nl.gamma32,
                    nl.work_img, nl.work_start, nl.cov_pt, nl.cov_ptr, nl.ent_img, nl.ent_i};
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
    std::vector<int> ent_img(npos), ent_i(npos);
    for (int g = 0; g < nimg; g++) {
        for (int ii = 0; ii < img_ndc[g]; ii++) {
            const int p = grid_pos[off[g] + ii];
            const int e = slot[p]++;
            ent_img[e] = g;
            ent_i[e] = ii;
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
    UP(ent_img, ent_img.data(), ent_img.size());
    UP(ent_i, ent_i.data(), ent_i.size());
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
