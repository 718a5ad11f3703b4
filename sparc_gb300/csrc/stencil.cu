// Radius-6 finite-difference stencil for an orthogonal periodic grid, fused with the diagonal
// (local potential), the shift and the Chebyshev three-term update:
//
//   out[:, n] = s1 * ( a*Lap + bv*diag(v) + c*I ) x[:, n]  +  s2 * z[:, n]
//
// This one kernel serves Lap_plus_diag_vec_mult_orth (src/lapVecRoutines.c:306, with
// s1 = 1, s2 = 0), the local part of Hamiltonian_vectors_mult
// (src/hamiltonianVecRoutines.c:45, a = -0.5, bv = 1) and each degree of ChebyshevFiltering
// (src/eigenSolver.c:722-798, s1 = 2*sigma2/e, s2 = -sigma*sigma2, z = X), so the recurrence
// costs no extra pass over HBM.
//
// Layout: column-major blocks with leading dimension ld, grid index i + j*Nx + k*Nx*Ny.
// Each thread block owns a tile of an xy-plane for one column and marches along z: the
// z-neighbours of a thread's point live in a register queue of 2R+1 values, the current plane
// plus its x/y halo lives in shared memory (two buffers, one barrier per plane), and periodic
// images are resolved by wrapping indices while loading (no ghost-extended copy, unlike the
// reference's x_ex). Values for the next plane (halo, potential, Chebyshev term) are
// prefetched into registers one plane ahead.
#include "sgpu_internal.h"
#include "mbarrier.cuh"
#include "cpasync.cuh"

namespace sgpu {
namespace {

template <typename T>
struct StencilParams {
    const T *__restrict__ x;
    T *__restrict__ out;
    const T *__restrict__ z;
    const T *__restrict__ v;
    long ldx, ldo, ldz;
    int Nx, Ny, Nz, nslab, zlen;
    T wx[kMaxFDn + 1], wy[kMaxFDn + 1], wz[kMaxFDn + 1];
    T c0, bv, s1, s2;
    int *status;  // kernel status word (bounded waits that ran out set bits here)
};

__device__ __forceinline__ int wrapi(int i, int n)
{
    i %= n;
    return i < 0 ? i + n : i;
}

// FP64 (and generic) kernel: one point per thread. On GB300 the FP64 pipe, not HBM, bounds it.
template <typename T, int R, int BX, int BY>
__global__ void __launch_bounds__(BX *BY)
    k_stencil_orth(const StencilParams<T> p)
{
    __shared__ T s[2][BY + 2 * R][BX + 2 * R];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    const int col = blockIdx.z / p.nslab;
    const int slab = blockIdx.z - col * p.nslab;
    const int zs = slab * p.zlen;
    const int ze = min(zs + p.zlen, p.Nz);
    if (zs >= ze) return;

    const int i = x0 + tx, j = y0 + ty;
    const bool active = (i < p.Nx) && (j < p.Ny);
    const int gi = wrapi(i, p.Nx), gj = wrapi(j, p.Ny);
    const long NxNy = (long)p.Nx * p.Ny;

    const T *__restrict__ xc = p.x + (long)col * p.ldx;
    const T *__restrict__ zc = p.z ? p.z + (long)col * p.ldz : nullptr;
    T *__restrict__ oc = p.out + (long)col * p.ldo;
    const long own = gi + (long)gj * p.Nx;

    const bool hx = tx < R, hy = ty < R;
    long hxl = 0, hxr = 0, hyl = 0, hyr = 0;
    if (hx) {
        hxl = wrapi(x0 - R + tx, p.Nx) + (long)gj * p.Nx;
        hxr = wrapi(x0 + BX + tx, p.Nx) + (long)gj * p.Nx;
    }
    if (hy) {
        hyl = gi + (long)wrapi(y0 - R + ty, p.Ny) * p.Nx;
        hyr = gi + (long)wrapi(y0 + BY + ty, p.Ny) * p.Nx;
    }

    T q[2 * R + 2];  // q[m] = x at plane k - R + m; q[2R+1], plane k+R+1, is in flight
#pragma unroll
    for (int m = 0; m <= 2 * R; m++)
        q[m] = __ldg(xc + own + (long)wrapi(zs - R + m, p.Nz) * NxNy);

    T h0 = T(0), h1 = T(0), h2 = T(0), h3 = T(0), vv = T(0), zz = T(0);
    {
        const long pk = (long)zs * NxNy;
        if (hx) { h0 = __ldg(xc + pk + hxl); h1 = __ldg(xc + pk + hxr); }
        if (hy) { h2 = __ldg(xc + pk + hyl); h3 = __ldg(xc + pk + hyr); }
        if (p.v) vv = __ldg(p.v + own + pk);
        if (zc) zz = zc[own + pk];
    }

    for (int k = zs; k < ze; k++) {
        const int b = k & 1;
        q[2 * R + 1] = __ldg(xc + own + (long)wrapi(k + R + 1, p.Nz) * NxNy);
        s[b][ty + R][tx + R] = q[R];
        if (hx) { s[b][ty + R][tx] = h0; s[b][ty + R][tx + BX + R] = h1; }
        if (hy) { s[b][ty][tx + R] = h2; s[b][ty + BY + R][tx + R] = h3; }
        const T vcur = vv, zcur = zz;
        if (k + 1 < ze) {
            const long pn = (long)(k + 1) * NxNy;
            if (hx) { h0 = __ldg(xc + pn + hxl); h1 = __ldg(xc + pn + hxr); }
            if (hy) { h2 = __ldg(xc + pn + hyl); h3 = __ldg(xc + pn + hyr); }
            if (p.v) vv = __ldg(p.v + own + pn);
            if (zc) zz = zc[own + pn];
        }
        __syncthreads();
        if (active) {
            // three independent FMA chains (x, y, z): on GB300 the FP64 pipe bounds this
            // kernel, and chained FMAs need 6 FP64 instructions per offset instead of 9
            T rx = p.c0 * q[R], ry = T(0), rz = T(0);
#pragma unroll
            for (int r = 1; r <= R; r++) {
                rx = fma(s[b][ty + R][tx + R - r] + s[b][ty + R][tx + R + r], p.wx[r], rx);
                ry = fma(s[b][ty + R - r][tx + R] + s[b][ty + R + r][tx + R], p.wy[r], ry);
                rz = fma(q[R - r] + q[R + r], p.wz[r], rz);
            }
            T res = rx + (ry + rz);
            if (p.v) res += p.bv * (vcur * q[R]);
            T o = p.s1 * res;
            if (zc) o += p.s2 * zcur;
            oc[own + (long)k * NxNy] = o;
        }
#pragma unroll
        for (int m = 0; m <= 2 * R; m++) q[m] = q[m + 1];
    }
}

// FP32 kernel: each thread owns two neighbouring x-points. Shared-memory reads are paired
// (8-byte), the neighbour pair sums use Blackwell's packed f32x2 add, and the weighted sums
// run as three independent FMA chains (x, y, z) whose weights come straight from the kernel
// parameter bank. The z-loop is unrolled by the queue length 2R+1, so the register queue
// rotates by renaming instead of moves. In-column offsets are 32-bit.
template <int R, int BXP, int BY, int MINB>
__global__ void __launch_bounds__(BXP / 2 * BY, MINB)
    k_stencil_f32x2(const StencilParams<float> p)
{
    constexpr int Q = 2 * R + 1;
    constexpr int W = BXP + 2 * R;
    static_assert(R % 2 == 0 && BXP % 2 == 0, "paired layout needs even radius and tile");
    static_assert(Q == 13, "the unrolled z-loop below is written for radius 6");
    __shared__ __align__(16) float s[2][BY + 2 * R][W];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x0 = blockIdx.x * BXP, y0 = blockIdx.y * BY;
    const int col = blockIdx.z / p.nslab;
    const int slab = blockIdx.z - col * p.nslab;
    const int zs = slab * p.zlen;
    const int ze = min(zs + p.zlen, p.Nz);
    if (zs >= ze) return;

    const int i0 = x0 + 2 * tx, j = y0 + ty;
    const bool act0 = (i0 < p.Nx) && (j < p.Ny), act1 = (i0 + 1 < p.Nx) && (j < p.Ny);
    const int gj = wrapi(j, p.Ny);
    const int row = gj * p.Nx;
    const int own0 = wrapi(i0, p.Nx) + row;
    const int own1 = wrapi(i0 + 1, p.Nx) + row;
    const int NxNy = p.Nx * p.Ny;
    const float *__restrict__ xc = p.x + (long)col * p.ldx;
    const float *__restrict__ zc = p.z ? p.z + (long)col * p.ldz : nullptr;
    float *__restrict__ oc = p.out + (long)col * p.ldo;

    const bool hx = tx < R / 2, hy = ty < R;
    int hA0 = 0, hA1 = 0, hB0 = 0, hB1 = 0;  // x-halo (left, right) or y-halo (top, bottom)
    if (hx) {
        hA0 = wrapi(x0 - R + 2 * tx, p.Nx) + row;
        hA1 = wrapi(x0 - R + 2 * tx + 1, p.Nx) + row;
        hB0 = wrapi(x0 + BXP + 2 * tx, p.Nx) + row;
        hB1 = wrapi(x0 + BXP + 2 * tx + 1, p.Nx) + row;
    }
    int hT0 = 0, hT1 = 0, hD0 = 0, hD1 = 0;
    if (hy) {
        const int rt = wrapi(y0 - R + ty, p.Ny) * p.Nx;
        const int rb = wrapi(y0 + BY + ty, p.Ny) * p.Nx;
        hT0 = own0 - row + rt; hT1 = own1 - row + rt;
        hD0 = own0 - row + rb; hD1 = own1 - row + rb;
    }

    float2 q[Q];
#pragma unroll
    for (int m = 0; m < 2 * R; m++) {
        const int pl = wrapi(zs - R + m, p.Nz) * NxNy;
        q[m] = make_float2(__ldg(xc + own0 + pl), __ldg(xc + own1 + pl));
    }
    float2 hL = make_float2(0.f, 0.f), hR = hL, hT = hL, hB = hL, vv = hL, zz = hL;
    {
        const int pk = zs * NxNy;
        if (hx) {
            hL = make_float2(__ldg(xc + pk + hA0), __ldg(xc + pk + hA1));
            hR = make_float2(__ldg(xc + pk + hB0), __ldg(xc + pk + hB1));
        }
        if (hy) {
            hT = make_float2(__ldg(xc + pk + hT0), __ldg(xc + pk + hT1));
            hB = make_float2(__ldg(xc + pk + hD0), __ldg(xc + pk + hD1));
        }
        if (p.v) vv = make_float2(__ldg(p.v + own0 + pk), __ldg(p.v + own1 + pk));
        if (zc) zz = make_float2(zc[own0 + pk], zc[own1 + pk]);
    }

    // one plane: U is the unroll slot; the queue slot of plane k-R+m is (U+m) % Q
#define SGPU_F2_STEP(U)                                                                          \
    {                                                                                            \
        const int k = kb + (U);                                                                  \
        if (k < ze) {                                                                            \
            const int b = k & 1;                                                                 \
            {                                                                                    \
                const int pl = wrapi(k + R, p.Nz) * NxNy;                                        \
                q[((U) + 2 * R) % Q] = make_float2(__ldg(xc + own0 + pl), __ldg(xc + own1 + pl)); \
            }                                                                                    \
            const float2 cen = q[((U) + R) % Q];                                                 \
            *reinterpret_cast<float2 *>(&s[b][ty + R][R + 2 * tx]) = cen;                        \
            if (hx) {                                                                            \
                *reinterpret_cast<float2 *>(&s[b][ty + R][2 * tx]) = hL;                         \
                *reinterpret_cast<float2 *>(&s[b][ty + R][R + BXP + 2 * tx]) = hR;               \
            }                                                                                    \
            if (hy) {                                                                            \
                *reinterpret_cast<float2 *>(&s[b][ty][R + 2 * tx]) = hT;                         \
                *reinterpret_cast<float2 *>(&s[b][ty + BY + R][R + 2 * tx]) = hB;                \
            }                                                                                    \
            const float2 vcur = vv, zcur = zz;                                                   \
            if (k + 1 < ze) {                                                                    \
                const int pn = (k + 1) * NxNy;                                                   \
                if (hx) {                                                                        \
                    hL = make_float2(__ldg(xc + pn + hA0), __ldg(xc + pn + hA1));                \
                    hR = make_float2(__ldg(xc + pn + hB0), __ldg(xc + pn + hB1));                \
                }                                                                                \
                if (hy) {                                                                        \
                    hT = make_float2(__ldg(xc + pn + hT0), __ldg(xc + pn + hT1));                \
                    hB = make_float2(__ldg(xc + pn + hD0), __ldg(xc + pn + hD1));                \
                }                                                                                \
                if (p.v) vv = make_float2(__ldg(p.v + own0 + pn), __ldg(p.v + own1 + pn));       \
                if (zc) zz = make_float2(zc[own0 + pn], zc[own1 + pn]);                          \
            }                                                                                    \
            __syncthreads();                                                                     \
            if (act0 || act1) {                                                                  \
                const float *srow = &s[b][ty + R][2 * tx];                                       \
                float2 L[R + 1];                                                                 \
                _Pragma("unroll") for (int m = 0; m <= R; m++)                                   \
                    L[m] = *reinterpret_cast<const float2 *>(srow + 2 * m);                      \
                float ax0 = p.c0 * cen.x, ax1 = p.c0 * cen.y;                                    \
                float ay0 = 0.f, ay1 = 0.f, az0 = 0.f, az1 = 0.f;                                \
                _Pragma("unroll") for (int r = 1; r <= R; r++) {                                 \
                    float2 lo, hi;                                                               \
                    if (r % 2 == 0) {                                                            \
                        lo = L[(R - r) / 2];                                                     \
                        hi = L[(R + r) / 2];                                                     \
                    } else {                                                                     \
                        lo = make_float2(L[(R - r) / 2].y, L[(R - r + 1) / 2].x);                \
                        hi = make_float2(L[(R + r) / 2].y, L[(R + r + 1) / 2].x);                \
                    }                                                                            \
                    const float2 xs = __fadd2_rn(lo, hi);                                        \
                    const float2 ys = __fadd2_rn(                                                \
                        *reinterpret_cast<const float2 *>(&s[b][ty + R - r][R + 2 * tx]),       \
                        *reinterpret_cast<const float2 *>(&s[b][ty + R + r][R + 2 * tx]));      \
                    const float2 zsum = __fadd2_rn(q[((U) + R - r) % Q], q[((U) + R + r) % Q]);  \
                    ax0 = fmaf(xs.x, p.wx[r], ax0); ax1 = fmaf(xs.y, p.wx[r], ax1);              \
                    ay0 = fmaf(ys.x, p.wy[r], ay0); ay1 = fmaf(ys.y, p.wy[r], ay1);              \
                    az0 = fmaf(zsum.x, p.wz[r], az0); az1 = fmaf(zsum.y, p.wz[r], az1);          \
                }                                                                                \
                float r0 = ax0 + (ay0 + az0), r1 = ax1 + (ay1 + az1);                            \
                if (p.v) {                                                                       \
                    r0 = fmaf(p.bv, vcur.x * cen.x, r0);                                         \
                    r1 = fmaf(p.bv, vcur.y * cen.y, r1);                                         \
                }                                                                                \
                r0 *= p.s1;                                                                      \
                r1 *= p.s1;                                                                      \
                if (zc) {                                                                        \
                    r0 = fmaf(p.s2, zcur.x, r0);                                                 \
                    r1 = fmaf(p.s2, zcur.y, r1);                                                 \
                }                                                                                \
                const int pk = k * NxNy;                                                         \
                if (act0) oc[own0 + pk] = r0;                                                    \
                if (act1) oc[own1 + pk] = r1;                                                    \
            }                                                                                    \
        }                                                                                        \
    }

    for (int kb = zs; kb < ze; kb += Q) {
        SGPU_F2_STEP(0) SGPU_F2_STEP(1) SGPU_F2_STEP(2) SGPU_F2_STEP(3) SGPU_F2_STEP(4)
        SGPU_F2_STEP(5) SGPU_F2_STEP(6) SGPU_F2_STEP(7) SGPU_F2_STEP(8) SGPU_F2_STEP(9)
        SGPU_F2_STEP(10) SGPU_F2_STEP(11) SGPU_F2_STEP(12)
    }
#undef SGPU_F2_STEP
}

// ---------------------------------------------------------------------------------------------
// FP32 kernel with 2x2 register blocking: each thread owns points (i0, i0+1) x (j0, j0+1), so
// one column of 14 shared-memory pairs serves the y-neighbours of both rows and the z-queue
// holds two pairs per plane. Halo values reach shared memory by cp.async (no staging
// registers), one plane ahead, into the buffer the previous plane has finished with. VEC
// selects 8-byte global accesses (even Nx, even leading dimensions, 8-byte aligned bases);
// without it every access is a 4-byte one. Per point the arithmetic is the same sequence of
// IEEE operations as k_stencil_f32x2, so the two kernels give identical results.

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}

template <bool VEC>
__device__ __forceinline__ float2 ld_pair(const float *__restrict__ base, int o0, int o1)
{
    if constexpr (VEC)
        return __ldg(reinterpret_cast<const float2 *>(base + o0));
    else
        return make_float2(__ldg(base + o0), __ldg(base + o1));
}

// Arithmetic of one 2x2 block at plane k (queue slot (U+R) % Q holds plane k): x-neighbours
// from the shared-memory rows srow0 and srow0 + W (each starting R points left of the
// block's first column), y-neighbours from the column yv (rows j0-R .. j0+1+R), z-neighbours
// from the register queues qa (row j0) and qb (row j0+1). Per point this is the operation
// sequence of k_stencil_f32x2: three FMA chains (x, y, z) over the symmetric pair sums, the
// potential term, the s1 scale and the recurrence term.
template <int R, int Q, int U>
__device__ __forceinline__ void b22_block(const StencilParams<float> &p,
                                          const float *__restrict__ srow0, int W,
                                          const float2 (&yv)[2 * R + 2], const float2 (&qa)[Q],
                                          const float2 (&qb)[Q], const float2 (&vc)[2],
                                          const float2 (&zc)[2], bool hasv, bool hasz,
                                          float2 (&o)[2])
{
#pragma unroll
    for (int rr = 0; rr < 2; rr++) {
        const float2 cen = rr ? qb[(U + R) % Q] : qa[(U + R) % Q];
        const float *srow = srow0 + rr * W;
        float2 L[R + 1];
#pragma unroll
        for (int m = 0; m <= R; m++) L[m] = *reinterpret_cast<const float2 *>(srow + 2 * m);
        // packed (f32x2) forms of the scalar sequence: each lane rounds exactly as fmaf / * / +
        float2 ax = __fmul2_rn(cen, make_float2(p.c0, p.c0));
        float2 ay = make_float2(0.f, 0.f), az = ay;
#pragma unroll
        for (int r = 1; r <= R; r++) {
            float2 lo, hi;
            if (r % 2 == 0) {
                lo = L[(R - r) / 2];
                hi = L[(R + r) / 2];
            } else {
                lo = make_float2(L[(R - r) / 2].y, L[(R - r + 1) / 2].x);
                hi = make_float2(L[(R + r) / 2].y, L[(R + r + 1) / 2].x);
            }
            const float2 xs = __fadd2_rn(lo, hi);
            const float2 ys = __fadd2_rn(yv[R + rr - r], yv[R + rr + r]);
            const float2 zsum = rr ? __fadd2_rn(qb[(U + R - r) % Q], qb[(U + R + r) % Q])
                                   : __fadd2_rn(qa[(U + R - r) % Q], qa[(U + R + r) % Q]);
            ax = __ffma2_rn(xs, make_float2(p.wx[r], p.wx[r]), ax);
            ay = __ffma2_rn(ys, make_float2(p.wy[r], p.wy[r]), ay);
            az = __ffma2_rn(zsum, make_float2(p.wz[r], p.wz[r]), az);
        }
        float2 ov = __fadd2_rn(ax, __fadd2_rn(ay, az));
        if (hasv) ov = __ffma2_rn(make_float2(p.bv, p.bv), __fmul2_rn(vc[rr], cen), ov);
        ov = __fmul2_rn(ov, make_float2(p.s1, p.s1));
        if (hasz) ov = __ffma2_rn(make_float2(p.s2, p.s2), zc[rr], ov);
        o[rr] = ov;
    }
}

// Stores one 2x2 block (rows beyond Ny and points beyond Nx are skipped).
template <bool VEC>
__device__ __forceinline__ void b22_store(float *__restrict__ oc, int kpl, int row0, int row1,
                                          int gx0, int gx1, bool r0ok, bool r1ok, bool in0,
                                          bool in1, const float2 (&o)[2])
{
#pragma unroll
    for (int rr = 0; rr < 2; rr++) {
        const bool rok = rr ? r1ok : r0ok;
        const int orow = (rr ? row1 : row0) + kpl;
        if (VEC && rok && in1) {
            *reinterpret_cast<float2 *>(oc + orow + gx0) = o[rr];
        } else if (rok) {
            if (in0) oc[orow + gx0] = o[rr].x;
            if (in1) oc[orow + gx1] = o[rr].y;
        }
    }
}

template <int R, int BX, int BY, int MINB, bool VEC>
__global__ void __launch_bounds__(BX / 2 * (BY / 2), MINB)
    k_stencil_f32_b22(const StencilParams<float> p)
{
    // z-queue of Q = 2R+1 slots (planes k-R .. k+R). A 2R+2 ring that keeps plane k+R+1 in
    // flight was measured slower: its extra registers cost a resident block per SM.
    constexpr int Q = 2 * R + 1;
    constexpr int W = BX + 2 * R;
    static_assert(Q == 13 && R % 2 == 0, "the unrolled z-loop below is written for radius 6");
    __shared__ __align__(16) float s[2][BY + 2 * R][W];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    const int col = blockIdx.z / p.nslab;
    const int slab = blockIdx.z - col * p.nslab;
    const int zs = slab * p.zlen;
    const int ze = min(zs + p.zlen, p.Nz);
    if (zs >= ze) return;

    const int i0 = x0 + 2 * tx, j0 = y0 + 2 * ty;
    const bool in0 = i0 < p.Nx, in1 = i0 + 1 < p.Nx;
    const bool r0ok = j0 < p.Ny, r1ok = j0 + 1 < p.Ny;
    const int gx0 = wrapi(i0, p.Nx), gx1 = wrapi(i0 + 1, p.Nx);
    const int row0 = wrapi(j0, p.Ny) * p.Nx, row1 = wrapi(j0 + 1, p.Ny) * p.Nx;
    const int NxNy = p.Nx * p.Ny;
    const float *__restrict__ xc = p.x + (long)col * p.ldx;
    const float *__restrict__ zc = p.z ? p.z + (long)col * p.ldz : nullptr;
    float *__restrict__ oc = p.out + (long)col * p.ldo;

    // halo sources (offsets within a plane) and shared-memory slots
    const bool hx = tx < R / 2, hy = ty < R / 2;
    int hxo[4][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};  // (left, right) x (row 0, row 1)
    int hyo[4][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};  // top rows 0,1 then bottom rows 0,1
    if (hx) {
        const int lx = x0 - R + 2 * tx, rx = x0 + BX + 2 * tx;
        const int rows[2] = {row0, row1};
        for (int r = 0; r < 2; r++) {
            hxo[r][0] = wrapi(lx, p.Nx) + rows[r];
            hxo[r][1] = wrapi(lx + 1, p.Nx) + rows[r];
            hxo[2 + r][0] = wrapi(rx, p.Nx) + rows[r];
            hxo[2 + r][1] = wrapi(rx + 1, p.Nx) + rows[r];
        }
    }
    if (hy) {
        const int ty0 = y0 - R + 2 * ty, by0 = y0 + BY + 2 * ty;
        const int rr[4] = {wrapi(ty0, p.Ny) * p.Nx, wrapi(ty0 + 1, p.Ny) * p.Nx,
                           wrapi(by0, p.Ny) * p.Nx, wrapi(by0 + 1, p.Ny) * p.Nx};
        for (int r = 0; r < 4; r++) {
            hyo[r][0] = gx0 + rr[r];
            hyo[r][1] = gx1 + rr[r];
        }
    }
    auto issue_halo = [&](int k, int b) {
        const float *pl = xc + k * NxNy;
        if (hx) {
            for (int r = 0; r < 2; r++) {
                float *dl = &s[b][2 * ty + R + r][2 * tx];
                float *dr = &s[b][2 * ty + R + r][R + BX + 2 * tx];
                if constexpr (VEC) {
                    cp_async8(dl, pl + hxo[r][0]);
                    cp_async8(dr, pl + hxo[2 + r][0]);
                } else {
                    cp_async4(dl, pl + hxo[r][0]); cp_async4(dl + 1, pl + hxo[r][1]);
                    cp_async4(dr, pl + hxo[2 + r][0]); cp_async4(dr + 1, pl + hxo[2 + r][1]);
                }
            }
        }
        if (hy) {
            const int srow[4] = {2 * ty, 2 * ty + 1, BY + R + 2 * ty, BY + R + 2 * ty + 1};
            for (int r = 0; r < 4; r++) {
                float *d = &s[b][srow[r]][R + 2 * tx];
                if constexpr (VEC) {
                    cp_async8(d, pl + hyo[r][0]);
                } else {
                    cp_async4(d, pl + hyo[r][0]); cp_async4(d + 1, pl + hyo[r][1]);
                }
            }
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };

    float2 qa[Q], qb[Q];  // z-queues of rows j0 and j0+1: slot of plane k-R+m is (U+m) % Q
#pragma unroll
    for (int m = 0; m < 2 * R; m++) {
        const int pl = wrapi(zs - R + m, p.Nz) * NxNy;
        qa[m] = ld_pair<VEC>(xc, pl + gx0 + row0, pl + gx1 + row0);
        qb[m] = ld_pair<VEC>(xc, pl + gx0 + row1, pl + gx1 + row1);
    }
    float2 va = make_float2(0.f, 0.f), vb = va, za = va, zb = va;
    {
        const int pk = zs * NxNy;
        if (p.v) {
            va = ld_pair<VEC>(p.v, pk + gx0 + row0, pk + gx1 + row0);
            vb = ld_pair<VEC>(p.v, pk + gx0 + row1, pk + gx1 + row1);
        }
        if (zc) {
            za = ld_pair<VEC>(zc, pk + gx0 + row0, pk + gx1 + row0);
            zb = ld_pair<VEC>(zc, pk + gx0 + row1, pk + gx1 + row1);
        }
    }
    issue_halo(zs, zs & 1);

#define SGPU_B22_STEP(U)                                                                         \
    {                                                                                            \
        const int k = kb + (U);                                                                  \
        if (k < ze) {                                                                            \
            const int b = k & 1;                                                                 \
            {                                                                                    \
                const int pl = wrapi(k + R, p.Nz) * NxNy;                                        \
                qa[((U) + 2 * R) % Q] = ld_pair<VEC>(xc, pl + gx0 + row0, pl + gx1 + row0);      \
                qb[((U) + 2 * R) % Q] = ld_pair<VEC>(xc, pl + gx0 + row1, pl + gx1 + row1);      \
            }                                                                                    \
            const float2 ca = qa[((U) + R) % Q], cb = qb[((U) + R) % Q];                         \
            *reinterpret_cast<float2 *>(&s[b][2 * ty + R][R + 2 * tx]) = ca;                     \
            *reinterpret_cast<float2 *>(&s[b][2 * ty + R + 1][R + 2 * tx]) = cb;                 \
            const float2 vca = va, vcb = vb, zca = za, zcb = zb;                                 \
            cp_async_wait_all();                                                                 \
            __syncthreads();                                                                     \
            if (k + 1 < ze) {                                                                    \
                issue_halo(k + 1, b ^ 1);                                                        \
                const int pn = (k + 1) * NxNy;                                                   \
                if (p.v) {                                                                       \
                    va = ld_pair<VEC>(p.v, pn + gx0 + row0, pn + gx1 + row0);                    \
                    vb = ld_pair<VEC>(p.v, pn + gx0 + row1, pn + gx1 + row1);                    \
                }                                                                                \
                if (zc) {                                                                        \
                    za = ld_pair<VEC>(zc, pn + gx0 + row0, pn + gx1 + row0);                     \
                    zb = ld_pair<VEC>(zc, pn + gx0 + row1, pn + gx1 + row1);                     \
                }                                                                                \
            }                                                                                    \
            float2 yv[2 * R + 2];                                                                \
            _Pragma("unroll") for (int t = 0; t < 2 * R + 2; t++)                                \
                yv[t] = *reinterpret_cast<const float2 *>(&s[b][2 * ty + t][R + 2 * tx]);        \
            const float2 vcs[2] = {vca, vcb}, zcs[2] = {zca, zcb};                               \
            float2 o[2];                                                                         \
            b22_block<R, Q, (U)>(p, &s[b][2 * ty + R][2 * tx], W, yv, qa, qb, vcs, zcs,          \
                                 p.v != nullptr, zc != nullptr, o);                              \
            b22_store<VEC>(oc, k * NxNy, row0, row1, gx0, gx1, r0ok, r1ok, in0, in1, o);         \
        }                                                                                        \
    }

    for (int kb = zs; kb < ze; kb += Q) {
        SGPU_B22_STEP(0) SGPU_B22_STEP(1) SGPU_B22_STEP(2) SGPU_B22_STEP(3) SGPU_B22_STEP(4)
        SGPU_B22_STEP(5) SGPU_B22_STEP(6) SGPU_B22_STEP(7) SGPU_B22_STEP(8) SGPU_B22_STEP(9)
        SGPU_B22_STEP(10) SGPU_B22_STEP(11) SGPU_B22_STEP(12)
    }
#undef SGPU_B22_STEP
    cp_async_wait_all();
}

// ---------------------------------------------------------------------------------------------
// FP32 kernel with 2x2 register blocking fed from a shared-memory plane ring. Every plane
// (centre tile plus its x/y halo) reaches shared memory by cp.async R+D planes before the
// block computes it, and the potential / recurrence-term planes D planes before; the register
// z-queue is topped up from the ring (plane k+R, in shared memory since step k-D) instead of
// from global memory, so no step waits on a global load issued in the same step. One barrier
// per plane: after it the slot of plane k-1 is free and receives plane k+R+D. Same arithmetic
// (b22_block) as k_stencil_f32_b22, so the results are identical.
// EW = floats per copy: 4 (16-byte copies that bypass L1; needs Nx % 4 == 0 and 16-byte
// aligned columns, and the x-halo is widened to 8 points so every copy is aligned), 2 (8-byte)
// or 1. XO = shared-memory column of the tile's first point.
template <int R, int BX, int BY, int D, int EW_, bool VG = false>
struct RingShape {
    static constexpr int NA = VG ? 1 : 2;  // staged arrays per potential slot (VG: z only)
    static constexpr int EW = EW_;
    static constexpr int XO = EW == 4 ? (R + 3) / 4 * 4 : R;
    static constexpr int W = BX + 2 * XO, H = BY + 2 * R;
    static constexpr int SLOT = H * W;     // one plane with its halo (the corners stay unused)
    static constexpr int NR = R + D + 1;   // ring slots: planes k .. k+R+D
    static constexpr int NV = D + 1;       // potential / recurrence-term slots: planes k .. k+D
    static constexpr int NT = BX / 2 * (BY / 2);
    static constexpr int CROW = W / EW, HROW = BX / EW;
    static constexpr int NCOPY = BY * CROW + 2 * R * HROW;  // copies per plane
    static constexpr int NU = (NCOPY + NT - 1) / NT;        // copies per thread and plane
    static constexpr size_t smem_bytes = sizeof(float) * ((size_t)NR * SLOT + (size_t)NV * NA * BX * BY);
};

template <int R, int BX, int BY, int MINB, int EW, int D, bool VG>
__global__ void __launch_bounds__(BX / 2 * (BY / 2), MINB)
    k_stencil_f32_ring(const StencilParams<float> p)
{
    using S = RingShape<R, BX, BY, D, EW, VG>;
    constexpr bool VEC = EW >= 2;
    constexpr int Q = 2 * R + 1;
    constexpr int W = S::W, XO = S::XO;
    static_assert(Q == 13 && R % 2 == 0 && D >= 1, "the unrolled z-loop is written for radius 6");
    extern __shared__ __align__(16) float ring[];
    float *const vzs = ring + S::NR * S::SLOT;  // [NV][2][BY][BX]: potential, recurrence term
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * (BX / 2) + tx;
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    const int col = blockIdx.z / p.nslab;
    const int slab = blockIdx.z - col * p.nslab;
    const int zs = slab * p.zlen;
    const int ze = min(zs + p.zlen, p.Nz);
    if (zs >= ze) return;

    const int i0 = x0 + 2 * tx, j0 = y0 + 2 * ty;
    const bool in0 = i0 < p.Nx, in1 = i0 + 1 < p.Nx;
    const bool r0ok = j0 < p.Ny, r1ok = j0 + 1 < p.Ny;
    const int gx0 = wrapi(i0, p.Nx), gx1 = wrapi(i0 + 1, p.Nx);
    const int row0 = wrapi(j0, p.Ny) * p.Nx, row1 = wrapi(j0 + 1, p.Ny) * p.Nx;
    const int NxNy = p.Nx * p.Ny;
    const float *__restrict__ xc = p.x + (long)col * p.ldx;
    const float *__restrict__ zc = p.z ? p.z + (long)col * p.ldz : nullptr;
    float *__restrict__ oc = p.out + (long)col * p.ldo;

    // this thread's copies of a plane: in-plane source offset and ring-slot destination
    // (shared-space byte address within slot 0; -1: no copy)
    int gofs[S::NU];
    int sofs[S::NU];
    const unsigned sring = (unsigned)__cvta_generic_to_shared(ring);
#pragma unroll
    for (int u = 0; u < S::NU; u++) {
        const int e = tid + u * S::NT;
        gofs[u] = 0;
        sofs[u] = -1;
        if (e < S::NCOPY) {
            int r, c;
            if (e < BY * S::CROW) {
                r = R + e / S::CROW;
                c = (e % S::CROW) * EW;
            } else {
                const int e2 = e - BY * S::CROW, hr = e2 / S::HROW;
                r = hr < R ? hr : hr + BY;
                c = XO + (e2 % S::HROW) * EW;
            }
            gofs[u] = wrapi(y0 - R + r, p.Ny) * p.Nx + wrapi(x0 - XO + c, p.Nx);
            sofs[u] = (int)sizeof(float) * (r * W + c);
        }
    }
    const unsigned svz = (unsigned)__cvta_generic_to_shared(vzs + 2 * ty * BX + 2 * tx);
    const float *vsrc = p.v ? p.v + gx0 + row0 : nullptr;
    const float *zsrc = zc ? zc + gx0 + row0 : nullptr;
    const int drow = row1 - row0, dx = gx1 - gx0;
    const int NzNxNy = p.Nz * NxNy;

    // Copy groups, one committed per step (possibly empty): ring plane number kp (offset pw,
    // slot rs) and, when vzon, the potential / recurrence term of plane offset vo (slot vs).
    int pw = zs * NxNy, rs = zs % S::NR;  // next ring plane to copy: zs
    int vo = zs * NxNy, vs = zs % S::NV;  // next potential plane to copy: zs
    auto issue = [&](bool ringon, bool vzon) {
        if (ringon) {
            const float *pl = xc + pw;
            const unsigned dst = sring + (unsigned)(rs * S::SLOT * (int)sizeof(float));
#pragma unroll
            for (int u = 0; u < S::NU; u++) {
                if (sofs[u] >= 0) {
                    if constexpr (EW == 4) cp_async16s(dst + sofs[u], pl + gofs[u]);
                    else if constexpr (EW == 2) cp_async8s(dst + sofs[u], pl + gofs[u]);
                    else cp_async4s(dst + sofs[u], pl + gofs[u]);
                }
            }
            pw += NxNy;
            if (pw == NzNxNy) pw = 0;
            rs = rs + 1 == S::NR ? 0 : rs + 1;
        }
        if (vzon) {
            const unsigned d = svz + (unsigned)(vs * S::NA * BX * BY * (int)sizeof(float));
            const float *srcs[2] = {VG ? nullptr : vsrc, zsrc};
#pragma unroll
            for (int a = 0; a < 2; a++) {
                if (!srcs[a]) continue;
                const float *g = srcs[a] + vo;
                const int ai = VG ? 0 : a;  // array index within the slot
                const unsigned da = d + (unsigned)(ai * BX * BY * (int)sizeof(float));
                if constexpr (VEC) {
                    cp_async8s(da, g);
                    cp_async8s(da + BX * sizeof(float), g + drow);
                } else {
                    cp_async4s(da, g);
                    cp_async4s(da + sizeof(float), g + dx);
                    cp_async4s(da + BX * sizeof(float), g + drow);
                    cp_async4s(da + (BX + 1) * sizeof(float), g + drow + dx);
                }
            }
            vo += NxNy;
            vs = vs + 1 == S::NV ? 0 : vs + 1;
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };

    // prologue: the register queue holds planes zs-R .. zs+R-1; the ring receives planes
    // zs .. zs+R+D-1 and the potential planes zs .. zs+D-1 (the groups of steps
    // zs-R-D .. zs-1: group j copies ring plane zs+j and potential plane zs+j-R)
    float2 qa[Q], qb[Q];
#pragma unroll
    for (int m = 0; m < 2 * R; m++) {
        const int pl = wrapi(zs - R + m, p.Nz) * NxNy;
        qa[m] = ld_pair<VEC>(xc, pl + gx0 + row0, pl + gx1 + row0);
        qb[m] = ld_pair<VEC>(xc, pl + gx0 + row1, pl + gx1 + row1);
    }
    for (int j = 0; j < R + D; j++) {
        const int kstep = zs - R - D + j;  // the step this group belongs to
        issue(kstep + D < ze, j >= R && kstep + D < ze);
    }
    int sk = zs % S::NR;      // ring slot of plane k
    int svk = zs % S::NV;     // potential slot of plane k
    int ko = zs * NxNy;       // offset of plane k

#define SGPU_RING_STEP(U)                                                                        \
    {                                                                                            \
        const int k = kb + (U);                                                                  \
        if (k < ze) {                                                                            \
            cp_async_wait_group<D - 1>();                                                        \
            __syncthreads();                                                                     \
            issue(k + D < ze, k + D < ze);                                                       \
            const float *sl = ring + sk * S::SLOT;                                               \
            const int skr = sk + R >= S::NR ? sk + R - S::NR : sk + R;                           \
            const float *sq = ring + skr * S::SLOT + (2 * ty + R) * W + XO + 2 * tx;             \
            qa[((U) + 2 * R) % Q] = *reinterpret_cast<const float2 *>(sq);                       \
            qb[((U) + 2 * R) % Q] = *reinterpret_cast<const float2 *>(sq + W);                   \
            const float *vz = vzs + svk * S::NA * BX * BY + 2 * ty * BX + 2 * tx;                \
            float2 vcs[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};                      \
            float2 zcs[2] = {vcs[0], vcs[1]};                                                    \
            if (vsrc) {                                                                          \
                if constexpr (VG) { /* shared by all columns: from L2 */                         \
                    vcs[0] = ld_pair<VEC>(vsrc, ko, ko + dx);                                    \
                    vcs[1] = ld_pair<VEC>(vsrc, ko + drow, ko + drow + dx);                      \
                } else {                                                                         \
                    vcs[0] = *reinterpret_cast<const float2 *>(vz);                              \
                    vcs[1] = *reinterpret_cast<const float2 *>(vz + BX);                         \
                }                                                                                \
            }                                                                                    \
            if (zsrc) {                                                                          \
                const float *zz = vz + (VG ? 0 : BX * BY);                                       \
                zcs[0] = *reinterpret_cast<const float2 *>(zz);                                  \
                zcs[1] = *reinterpret_cast<const float2 *>(zz + BX);                             \
            }                                                                                    \
            float2 yv[2 * R + 2];                                                                \
            _Pragma("unroll") for (int t = 0; t < 2 * R + 2; t++)                                \
                yv[t] = *reinterpret_cast<const float2 *>(sl + (2 * ty + t) * W + XO + 2 * tx);  \
            float2 o[2];                                                                         \
            b22_block<R, Q, (U)>(p, sl + (2 * ty + R) * W + XO - R + 2 * tx, W, yv, qa, qb,     \
                                 vcs, zcs, vsrc != nullptr, zsrc != nullptr, o);                 \
            b22_store<VEC>(oc, ko, row0, row1, gx0, gx1, r0ok, r1ok, in0, in1, o);               \
            sk = sk + 1 == S::NR ? 0 : sk + 1;                                                   \
            svk = svk + 1 == S::NV ? 0 : svk + 1;                                                \
            ko += NxNy;                                                                          \
        }                                                                                        \
    }

    for (int kb = zs; kb < ze; kb += Q) {
        SGPU_RING_STEP(0) SGPU_RING_STEP(1) SGPU_RING_STEP(2) SGPU_RING_STEP(3)
        SGPU_RING_STEP(4) SGPU_RING_STEP(5) SGPU_RING_STEP(6) SGPU_RING_STEP(7)
        SGPU_RING_STEP(8) SGPU_RING_STEP(9) SGPU_RING_STEP(10) SGPU_RING_STEP(11)
        SGPU_RING_STEP(12)
    }
#undef SGPU_RING_STEP
    cp_async_wait_all();
}

template <int R, int BX, int BY, int MINB, int EW, int D, bool VG>
int launch_ring(const StencilParams<float> &q, dim3 grid, cudaStream_t st)
{
    constexpr size_t smem = RingShape<R, BX, BY, D, EW, VG>::smem_bytes;
    auto kern = k_stencil_f32_ring<R, BX, BY, MINB, EW, D, VG>;
    SGPU_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    kern<<<grid, dim3(BX / 2, BY / 2), smem, st>>>(q);
    return SGPU_OK;
}

// ---------------------------------------------------------------------------------------------
// Plane ring fed by bulk copies of the tensor memory accelerator, with no block-wide barrier in
// the plane loop. Each row of a plane's tile (48 floats for the BY centre rows, x-halo
// included; 32 for the 2R y-halo rows) and each row of the recurrence term's tile (32 floats)
// moves by one cp.async.bulk (two where the row wraps periodically in x), issued by one lane
// of warp 0 (ring) or warp 1 (recurrence term); the potential is read from L2 as in the
// two-planes-ahead cp.async ring. Three sets of mbarriers order the pipeline:
//   full[s]   one arrival (expect_tx of the plane's bytes) per fill of ring slot s; the bulk
//             copies complete its transaction count;
//   zfull[s]  the same for recurrence-term slot s;
//   empty[s]  each warp arrives (once its lanes have met at __syncwarp) when it has finished
//             the step of the plane in ring slot s.
// Step k reuses the ring slot and the recurrence-term slot of plane k-1, so the issuing warps
// wait on empty for step k-1 and every other warp runs on as soon as its own planes are full:
// warps drift apart by up to D steps instead of meeting at a barrier each plane.
// Every wait is bounded (2e9 SM cycles, about one second): a wait that runs out sets bit 1 of the status
// word, the thread stops waiting and finishes its loop, and thread 0 waits (bounded) for the
// last fill of every slot before the block exits, so no copy lands after the block is gone.
// Needs Nx % 4 == 0 and 16-byte aligned rows of x and z (every copy's address and size are
// then multiples of 16 bytes). Same arithmetic (b22_block) as the other 2x2 kernels.
// A barrier phase that nothing completes, waited on with a bound of `limit` cycles: the wait
// runs out and sets bit 2 of the status word; one thread then arrives so the phase completes
// and the barrier is left balanced. Shows the bound and the status path work on the device.
__global__ void k_wait_bound_check(int *status, long long limit)
{
    __shared__ __align__(8) unsigned long long bar;
    const unsigned a = (unsigned)__cvta_generic_to_shared(&bar);
    if (threadIdx.x == 0) {
        mbar_init(a, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    __syncthreads();
    const bool ok = mbar_wait_bounded(a, 0, limit);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (!ok) atomicOr(status, 2);
        mbar_arrive(a);
    }
}
// one tile row: n floats of global row `grow` from column xs (wrapped periodically, split
// wherever it wraps) into shared memory at byte address dst; Nx % 4 == 0 and xs % 4 == 0.
// The general form, for grids narrower than a tile row; wider grids use the precomputed
// one- or two-piece split of the row descriptors.
__device__ __noinline__ void bulk_row_general(unsigned dst, const float *grow, int xs, int n,
                                              int Nx, unsigned mbar)
{
    int gx = xs % Nx;
    if (gx < 0) gx += Nx;
#pragma unroll 1
    while (n > 0) {
        const int len = min(n, Nx - gx);
        bulk_g2s(dst, grow + gx, (unsigned)len * 4u, mbar);
        dst += (unsigned)len * 4u;
        n -= len;
        gx = 0;
    }
}

template <int R, int BX, int BY, int D>
struct BulkShape {
    static constexpr int XO = (R + 3) / 4 * 4;  // x-halo widened to a 16-byte boundary
    static constexpr int W = BX + 2 * XO, H = BY + 2 * R;
    static constexpr int SLOT = H * W;
    static constexpr int NR = R + D + 1;        // ring slots: planes k .. k+R+D
    static constexpr int NV = D + 1;            // recurrence-term slots: planes k .. k+D
    static constexpr int NT = BX / 2 * (BY / 2);
    static constexpr unsigned plane_bytes = sizeof(float) * (BY * W + 2 * R * BX);
    static constexpr unsigned zplane_bytes = sizeof(float) * BX * BY;
    static constexpr size_t data_bytes = sizeof(float) * ((size_t)NR * SLOT + (size_t)NV * BX * BY);
    static constexpr size_t bar_bytes = (8 * (2 * NR + NV) + 15) / 16 * 16;
    static constexpr int NDESC = 32 + BY;       // row descriptors: ring rows 0.., z rows 32..
    // + one 16-byte word after the descriptors: the block's abort flag
    static constexpr size_t smem_bytes = data_bytes + bar_bytes + 16 * (NDESC + 1);
    static_assert(H <= 32 && BY <= 32 && NR + NV <= 32 && NT >= 64, "one lane per tile row");
    static_assert(data_bytes % 16 == 0 && (SLOT * sizeof(float)) % 16 == 0, "16-byte slots");
};

template <int R, int BX, int BY, int MINB, int D>
__global__ void __launch_bounds__(BX / 2 * (BY / 2), MINB)
    k_stencil_f32_bulk(const StencilParams<float> p)
{
    using S = BulkShape<R, BX, BY, D>;
    constexpr int Q = 2 * R + 1;
    constexpr int W = S::W, XO = S::XO, NR = S::NR, NV = S::NV;
    static_assert(Q == 13 && R % 2 == 0 && D >= 1, "the unrolled z-loop is written for radius 6");
    extern __shared__ __align__(16) float ring[];
    const float *const zsl = ring + NR * S::SLOT;  // [NV][BY][BX] recurrence term
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * (BX / 2) + tx;
    const int warp = tid >> 5, lane = tid & 31;
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    const int col = blockIdx.z / p.nslab;
    const int slab = blockIdx.z - col * p.nslab;
    const int zs = slab * p.zlen;
    const int ze = min(zs + p.zlen, p.Nz);
    if (zs >= ze) return;

    const unsigned sring = (unsigned)__cvta_generic_to_shared(ring);
    const unsigned bfull = sring + (unsigned)S::data_bytes;  // full[NR]
    const unsigned bzfull = bfull + 8u * NR;                 // zfull[NV]
    const unsigned bempty = bzfull + 8u * NV;                // empty[NR]
    // row descriptors {plane offset of the first piece, of the second piece (column 0),
    // shared byte offset within the slot, total bytes << 16 | bytes of the first piece}
    int4 *const desc = reinterpret_cast<int4 *>(reinterpret_cast<char *>(ring) + S::data_bytes +
                                                S::bar_bytes);
    constexpr int NW = S::NT / 32;
    // set once any wait of the block has run out: from then on no copy is issued
    volatile int *const abort_flag = reinterpret_cast<volatile int *>(desc + S::NDESC);
    if (tid == 0) {
        *abort_flag = 0;
        for (int s = 0; s < NR; s++) {
            mbar_init(bfull + 8u * s, 1);
            mbar_init(bempty + 8u * s, NW);
        }
        for (int s = 0; s < NV; s++) mbar_init(bzfull + 8u * s, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0 && lane < S::H) {
        const int r = lane;
        const bool centre = r >= R && r < R + BY;
        const int n = centre ? W : BX;
        const int rowoff = wrapi(y0 - R + r, p.Ny) * p.Nx;
        const int gx = wrapi(centre ? x0 - XO : x0, p.Nx);
        const int len0 = min(n, p.Nx - gx);
        desc[r] = make_int4(rowoff + gx, rowoff, (r * W + (centre ? 0 : XO)) * 4,
                            (n * 4) << 16 | len0 * 4);
    } else if (warp == 1 && lane < BY) {
        const int rowoff = wrapi(y0 + lane, p.Ny) * p.Nx;
        const int len0 = min(BX, p.Nx - x0);
        desc[32 + lane] = make_int4(rowoff + x0, rowoff, lane * BX * 4, (BX * 4) << 16 | len0 * 4);
    }
    __syncthreads();
    const bool narrow = p.Nx < W;  // a tile row may wrap more than once: general split

    const int i0 = x0 + 2 * tx, j0 = y0 + 2 * ty;
    const bool in0 = i0 < p.Nx, in1 = i0 + 1 < p.Nx;
    const bool r0ok = j0 < p.Ny, r1ok = j0 + 1 < p.Ny;
    const int gx0 = wrapi(i0, p.Nx), gx1 = wrapi(i0 + 1, p.Nx);
    const int row0 = wrapi(j0, p.Ny) * p.Nx, row1 = wrapi(j0 + 1, p.Ny) * p.Nx;
    const int NxNy = p.Nx * p.Ny;
    const float *__restrict__ xc = p.x + (long)col * p.ldx;
    const float *__restrict__ zc = p.z ? p.z + (long)col * p.ldz : nullptr;
    float *__restrict__ oc = p.out + (long)col * p.ldo;
    const float *vsrc = p.v ? p.v + gx0 + row0 : nullptr;
    const int drow = row1 - row0, dx = gx1 - gx0;

    bool alive = true;    // false once one of this thread's waits has run out
    unsigned ph = 0;      // parity of the next wait: bits 0..NR-1 full, NR.. zfull
    unsigned phe = 0;     // parity of the next wait on empty (issuing warps)
    int ring_end = zs;    // ring planes zs .. ring_end-1 issued (warp 0)
    int z_end = zs;       // recurrence-term planes zs .. z_end-1 issued (warp 1)
    auto wait = [&](unsigned bar, int bit, unsigned &bits) {
        if (alive && !mbar_wait_bounded(bar, (bits >> bit) & 1u)) {
            alive = false;
            *abort_flag = 1;  // visible to an issuing warp through its next empty wait
            if (p.status) atomicOr(p.status, 1);
        }
        bits ^= 1u << bit;
    };
    // an issuing warp stops for good once its own wait or any other warp's has run out: a
    // copy into a slot whose release was not seen could overwrite data still being read
    auto may_issue = [&]() { return alive && *abort_flag == 0; };
    // one row per lane: ring rows from warp 0 (descriptors 0..H-1), recurrence-term rows from
    // warp 1 (32..32+BY-1); pb = the plane's first element, sbase = the slot's shared address
    auto issue_row = [&](const int4 d, const float *pb, unsigned sbase, unsigned bar, int xs) {
        const unsigned b0 = (unsigned)d.w & 0xffffu, tot = (unsigned)d.w >> 16;
        if (narrow) {
            bulk_row_general(sbase + d.z, pb + d.y, xs, (int)(tot / 4), p.Nx, bar);
        } else {
            bulk_g2s(sbase + d.z, pb + d.x, b0, bar);
            if (b0 < tot) bulk_g2s(sbase + d.z + b0, pb + d.y, tot - b0, bar);
        }
    };
    // ring plane pl (zs <= pl < 2 Nz) into ring slot s
    auto issue_ring = [&](int pl, int s) {
        ring_end = pl + 1;
        const unsigned bar = bfull + 8u * s;
        if (lane == 0) mbar_arrive_tx(bar, S::plane_bytes);
        __syncwarp();
        if (lane < S::H) {
            const bool centre = lane >= R && lane < R + BY;
            issue_row(desc[lane], xc + (long)(pl >= p.Nz ? pl - p.Nz : pl) * NxNy,
                      sring + (unsigned)(s * S::SLOT * 4), bar, centre ? x0 - XO : x0);
        }
    };
    // recurrence-term plane pl (zs <= pl < Nz) into its slot s
    auto issue_z = [&](int pl, int s) {
        z_end = pl + 1;
        const unsigned bar = bzfull + 8u * s;
        if (lane == 0) mbar_arrive_tx(bar, S::zplane_bytes);
        __syncwarp();
        if (lane < BY)
            issue_row(desc[32 + lane], zc + (long)pl * NxNy,
                      sring + (unsigned)((NR * S::SLOT + s * BX * BY) * 4), bar, x0);
    };

    // prologue: the register queue holds planes zs-R .. zs+R-1 (read directly); the ring
    // receives planes zs .. zs+R+D-1 and the recurrence term planes zs .. zs+D-1
    float2 qa[Q], qb[Q];
#pragma unroll
    for (int m = 0; m < 2 * R; m++) {
        const int pl = wrapi(zs - R + m, p.Nz) * NxNy;
        qa[m] = ld_pair<true>(xc, pl + gx0 + row0, pl + gx1 + row0);
        qb[m] = ld_pair<true>(xc, pl + gx0 + row1, pl + gx1 + row1);
    }
    if (warp == 0) {
        for (int pl = zs; pl < zs + R + D && pl < ze + R; pl++) issue_ring(pl, pl % NR);
    } else if (warp == 1 && zc) {
        for (int pl = zs; pl < zs + D && pl < ze; pl++) issue_z(pl, pl % NV);
    }
    int sk = zs % NR;     // ring slot of plane k
    int svk = zs % NV;    // recurrence-term slot of plane k
    int ko = zs * NxNy;   // offset of plane k

#define SGPU_BULK_STEP(U)                                                                        \
    {                                                                                            \
        const int k = kb + (U);                                                                  \
        if (k < ze) {                                                                            \
            /* slots of plane k-1 receive ring plane k+R+D and recurrence-term plane k+D */      \
            if (k + D < ze && (warp == 0 || (warp == 1 && zc))) {                                \
                const int se = sk == 0 ? NR - 1 : sk - 1;                                        \
                if (k > zs) wait(bempty + 8u * se, se, phe);                                     \
                const bool go = __all_sync(0xffffffffu, may_issue());                            \
                if (go && warp == 0) issue_ring(k + R + D, se);                                  \
                else if (go) issue_z(k + D, svk == 0 ? NV - 1 : svk - 1);                       \
            }                                                                                    \
            const int skr = sk + R >= NR ? sk + R - NR : sk + R;                                 \
            if (k < zs + R) wait(bfull + 8u * sk, sk, ph);                                       \
            wait(bfull + 8u * skr, skr, ph);                                                     \
            if (zc) wait(bzfull + 8u * svk, NR + svk, ph);                                       \
            const float *sl = ring + sk * S::SLOT;                                               \
            const float *sq = ring + skr * S::SLOT + (2 * ty + R) * W + XO + 2 * tx;             \
            qa[((U) + 2 * R) % Q] = *reinterpret_cast<const float2 *>(sq);                       \
            qb[((U) + 2 * R) % Q] = *reinterpret_cast<const float2 *>(sq + W);                   \
            float2 vcs[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};                      \
            float2 zcs[2] = {vcs[0], vcs[1]};                                                    \
            if (vsrc) {                                                                          \
                vcs[0] = ld_pair<true>(vsrc, ko, ko + dx);                                       \
                vcs[1] = ld_pair<true>(vsrc, ko + drow, ko + drow + dx);                         \
            }                                                                                    \
            if (zc) {                                                                            \
                const float *zz = zsl + svk * BX * BY + 2 * ty * BX + 2 * tx;                    \
                zcs[0] = *reinterpret_cast<const float2 *>(zz);                                  \
                zcs[1] = *reinterpret_cast<const float2 *>(zz + BX);                             \
            }                                                                                    \
            float2 yv[2 * R + 2];                                                                \
            _Pragma("unroll") for (int t = 0; t < 2 * R + 2; t++)                                \
                yv[t] = *reinterpret_cast<const float2 *>(sl + (2 * ty + t) * W + XO + 2 * tx);  \
            float2 o[2];                                                                         \
            b22_block<R, Q, (U)>(p, sl + (2 * ty + R) * W + XO - R + 2 * tx, W, yv, qa, qb,     \
                                 vcs, zcs, vsrc != nullptr, zc != nullptr, o);                   \
            __syncwarp();                                                                        \
            if (lane == 0) mbar_arrive(bempty + 8u * sk);                                        \
            b22_store<true>(oc, ko, row0, row1, gx0, gx1, r0ok, r1ok, in0, in1, o);              \
            sk = sk + 1 == NR ? 0 : sk + 1;                                                      \
            svk = svk + 1 == NV ? 0 : svk + 1;                                                   \
            ko += NxNy;                                                                          \
        }                                                                                        \
    }

    for (int kb = zs; kb < ze; kb += Q) {
        SGPU_BULK_STEP(0) SGPU_BULK_STEP(1) SGPU_BULK_STEP(2) SGPU_BULK_STEP(3)
        SGPU_BULK_STEP(4) SGPU_BULK_STEP(5) SGPU_BULK_STEP(6) SGPU_BULK_STEP(7)
        SGPU_BULK_STEP(8) SGPU_BULK_STEP(9) SGPU_BULK_STEP(10) SGPU_BULK_STEP(11)
        SGPU_BULK_STEP(12)
    }
#undef SGPU_BULK_STEP
    // no copy may land after the block exits: each issuing warp waits for the last fill it
    // issued into each of its slots (ring planes zs .. ring_end-1 from warp 0, recurrence-term
    // planes zs .. z_end-1 from warp 1; fewer than planned if a wait ran out)
    if ((warp == 0 || (warp == 1 && zc)) && lane == 0) {
        bool ok = true;
        const int nslot = warp == 0 ? NR : NV;
        const int end = warp == 0 ? ring_end : z_end;
        const unsigned base = warp == 0 ? bfull : bzfull;
        for (int s = 0; s < nslot; s++) {
            const int last = end - 1 - ((end - 1 - s) % nslot + nslot) % nslot;
            if (last >= zs && !mbar_wait_bounded(base + 8u * s, ((last - zs) / nslot) & 1))
                ok = false;
        }
        if (!ok && p.status) atomicOr(p.status, 1);
    }
}

template <int R, int BX, int BY, int MINB, int D>
int launch_bulk(const StencilParams<float> &q, dim3 grid, cudaStream_t st)
{
    constexpr size_t smem = BulkShape<R, BX, BY, D>::smem_bytes;
    auto kern = k_stencil_f32_bulk<R, BX, BY, MINB, D>;
    SGPU_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    kern<<<grid, dim3(BX / 2, BY / 2), smem, st>>>(q);
    return SGPU_OK;
}

}  // namespace

template <typename T>
int launch_stencil(sgpu_ctx *ctx, int ncol, double a, double bv, double c, const T *v,
                   const T *x, long ldx, T *out, long ldo, double s1, double s2, const T *z,
                   long ldz, cudaStream_t st)
{
    constexpr int R = 6, BX = 32, BY = 8;       // FP64 tile (one point per thread)
    constexpr int BXP = 32, BYP = 16;          // FP32 tile (two points per thread)
    if (ctx->FDn != R) {
        set_error("stencil: only FD order 12 (radius 6) is built");
        return SGPU_ERR_ARG;
    }
    if (ncol <= 0) return SGPU_OK;
    if (sizeof(T) == 4 && ctx->Nd >= (1L << 31)) {
        set_error("stencil: FP32 kernel needs Nx*Ny*Nz < 2^31");
        return SGPU_ERR_ARG;
    }
    StencilParams<T> p;
    p.x = x; p.out = out; p.z = z; p.v = v;
    p.ldx = ldx; p.ldo = ldo; p.ldz = ldz;
    p.Nx = ctx->Nx; p.Ny = ctx->Ny; p.Nz = ctx->Nz;
    for (int r = 0; r <= R; r++) {
        p.wx[r] = (T)(ctx->cx[r] * a);
        p.wy[r] = (T)(ctx->cy[r] * a);
        p.wz[r] = (T)(ctx->cz[r] * a);
    }
    // centre weight as the reference forms it: a*wx0 + a*wy0 + a*wz0 + c
    double c0 = ctx->cx[0] * a;
    c0 += ctx->cy[0] * a;
    c0 += ctx->cz[0] * a;
    c0 += c;
    p.c0 = (T)c0;
    p.bv = (T)bv; p.s1 = (T)s1; p.s2 = (T)s2;
    p.status = ctx->kstatus;
    if (!v || fabs(bv) < 1e-14) p.v = nullptr;
    if (!z || s2 == 0.0) p.z = nullptr;

    const bool f32 = sizeof(T) == 4;
    // FP32 variants (autotune.cu): 0 paired 32x16, 1 2x2-blocked 32x16, 2 2x2-blocked 64x8,
    // 3 paired 64x8, 4 2x2-blocked 32x16 with 3 blocks per SM, 5 and 6 2x2-blocked 32x16 fed
    // from the shared-memory plane ring one and two planes ahead (6: potential from L2), 7 and
    // 8 the plane ring fed by bulk copies two and one planes ahead, 9 and 10 the cp.async
    // plane ring on 32x32 tiles (256 threads, 2 blocks per SM) one and two planes ahead
    const int variant = f32 ? ctx->stencil_variant : 0;
    const bool wide = variant == 2 || variant == 3;
    const bool tall = variant == 9 || variant == 10;
    const int tbx = f32 ? (wide ? 64 : BXP) : BX;
    const int tby = f32 ? (wide ? 8 : tall ? 32 : BYP) : BY;
    const int tilesx = (ctx->Nx + tbx - 1) / tbx;
    const int tilesy = (ctx->Ny + tby - 1) / tby;
    // split z into slabs until there are enough blocks to fill 152 SMs several times over
    long blocks1 = (long)tilesx * tilesy * ncol;
    int nslab = 1;
    while (blocks1 * nslab < 152L * 8 && ctx->Nz / (nslab * 2) >= 8) nslab *= 2;
    p.zlen = (ctx->Nz + nslab - 1) / nslab;
    p.nslab = nslab;
    // FP32 variant (chosen by sgpu_autotune or sgpu_set_stencil_variant); the 2x2 kernel uses
    // 8-byte global accesses when every base is 8-byte aligned and every stride is even
    auto al8 = [](const void *ptr) { return ((uintptr_t)ptr & 7u) == 0; };
    const bool vec = (ctx->Nx % 2 == 0) && al8(x) && al8(out) && ldx % 2 == 0 && ldo % 2 == 0 &&
                     (!p.z || (al8(z) && ldz % 2 == 0)) && (!p.v || al8(v));
    // the plane ring copies x in 16-byte pieces when every row of every column is 16-byte
    // aligned (the potential and recurrence term still move in 8-byte pieces)
    auto al16 = [](const void *ptr) { return ((uintptr_t)ptr & 15u) == 0; };
    const bool quad = vec && ctx->Nx % 4 == 0 && al16(x) && ldx % 4 == 0;
    // the bulk-copy ring also moves the recurrence term by rows of 16-byte pieces
    const bool bulk = quad && (!p.z || (al16(z) && ldz % 4 == 0));
    const int maxz = 65535 / nslab;
    for (int c0i = 0; c0i < ncol; c0i += maxz) {
        int nc = ncol - c0i < maxz ? ncol - c0i : maxz;
        StencilParams<T> q = p;
        q.x = x + (long)c0i * ldx;
        q.out = out + (long)c0i * ldo;
        if (q.z) q.z = z + (long)c0i * ldz;
        dim3 grid(tilesx, tilesy, nc * nslab);
        ProfScope ps(ctx, SGPU_KERNEL_STENCIL, st);
        if constexpr (sizeof(T) == 4) {
            switch (variant) {
            case 1:
                if (vec)
                    k_stencil_f32_b22<R, 32, 16, 4, true><<<grid, dim3(16, 8), 0, st>>>(q);
                else
                    k_stencil_f32_b22<R, 32, 16, 3, false><<<grid, dim3(16, 8), 0, st>>>(q);
                break;
            case 2:
                if (vec)
                    k_stencil_f32_b22<R, 64, 8, 4, true><<<grid, dim3(32, 4), 0, st>>>(q);
                else
                    k_stencil_f32_b22<R, 64, 8, 3, false><<<grid, dim3(32, 4), 0, st>>>(q);
                break;
            case 3:
                k_stencil_f32x2<R, 64, 8, 3><<<grid, dim3(32, 8), 0, st>>>(q);
                break;
            case 4:  // 2x2 32x16 capped at 3 blocks per SM (no register spills)
                if (vec)
                    k_stencil_f32_b22<R, 32, 16, 3, true><<<grid, dim3(16, 8), 0, st>>>(q);
                else
                    k_stencil_f32_b22<R, 32, 16, 3, false><<<grid, dim3(16, 8), 0, st>>>(q);
                break;
            case 5:  // 2x2 32x16 from the plane ring, planes one step ahead
                if (quad)
                    SGPU_TRY((launch_ring<R, 32, 16, 4, 4, 1, false>(q, grid, st)));
                else if (vec)
                    SGPU_TRY((launch_ring<R, 32, 16, 4, 2, 1, false>(q, grid, st)));
                else
                    SGPU_TRY((launch_ring<R, 32, 16, 4, 1, 1, false>(q, grid, st)));
                break;
            case 6:  // 2x2 32x16 from the plane ring, planes two steps ahead; the potential
                     // (one vector for all columns) read from L2 so 4 blocks fit per SM
                if (quad)
                    SGPU_TRY((launch_ring<R, 32, 16, 4, 4, 2, true>(q, grid, st)));
                else if (vec)
                    SGPU_TRY((launch_ring<R, 32, 16, 4, 2, 2, true>(q, grid, st)));
                else
                    SGPU_TRY((launch_ring<R, 32, 16, 4, 1, 2, true>(q, grid, st)));
                break;
            case 7:  // plane ring fed by bulk copies, two planes ahead (else as variant 6)
            case 8:  // the same, one plane ahead
                if (bulk && variant == 7)
                    SGPU_TRY((launch_bulk<R, 32, 16, 4, 2>(q, grid, st)));
                else if (bulk)
                    SGPU_TRY((launch_bulk<R, 32, 16, 4, 1>(q, grid, st)));
                else if (quad)
                    SGPU_TRY((launch_ring<R, 32, 16, 4, 4, 2, true>(q, grid, st)));
                else if (vec)
                    SGPU_TRY((launch_ring<R, 32, 16, 4, 2, 2, true>(q, grid, st)));
                else
                    SGPU_TRY((launch_ring<R, 32, 16, 4, 1, 2, true>(q, grid, st)));
                break;
            case 9:  // plane ring on 32x32 tiles, one plane ahead
                if (quad)
                    SGPU_TRY((launch_ring<R, 32, 32, 2, 4, 1, false>(q, grid, st)));
                else if (vec)
                    SGPU_TRY((launch_ring<R, 32, 32, 2, 2, 1, false>(q, grid, st)));
                else
                    SGPU_TRY((launch_ring<R, 32, 32, 2, 1, 1, false>(q, grid, st)));
                break;
            case 10:  // plane ring on 32x32 tiles, two planes ahead (potential from L2)
                if (quad)
                    SGPU_TRY((launch_ring<R, 32, 32, 2, 4, 2, true>(q, grid, st)));
                else if (vec)
                    SGPU_TRY((launch_ring<R, 32, 32, 2, 2, 2, true>(q, grid, st)));
                else
                    SGPU_TRY((launch_ring<R, 32, 32, 2, 1, 2, true>(q, grid, st)));
                break;
            default:
                k_stencil_f32x2<R, BXP, BYP, 3><<<grid, dim3(BXP / 2, BYP), 0, st>>>(q);
            }
        } else {
            k_stencil_orth<T, R, BX, BY><<<grid, dim3(BX, BY), 0, st>>>(q);
        }
    }
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

int wait_bound_check(sgpu_ctx *ctx)
{
    k_wait_bound_check<<<1, 32, 0, ctx->stream>>>(ctx->kstatus, 2000000LL);
    SGPU_CUDA_TRY(cudaGetLastError());
    return SGPU_OK;
}

template int launch_stencil<double>(sgpu_ctx *, int, double, double, double, const double *,
                                    const double *, long, double *, long, double, double,
                                    const double *, long, cudaStream_t);
template int launch_stencil<float>(sgpu_ctx *, int, double, double, double, const float *,
                                   const float *, long, float *, long, double, double,
                                   const float *, long, cudaStream_t);

}  // namespace sgpu
