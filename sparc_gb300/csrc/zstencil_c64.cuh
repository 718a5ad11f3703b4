// complex64 plane-ring stencil (two points per thread) for the k-point (Bloch) Hamiltonian;
// included by kpoint.cu.
#pragma once

#include "cpasync.cuh"
#include "zmath.cuh"

namespace sgpu {
namespace {

using zm::floordiv;
using zm::wrapz;

// complex64 stencil with two x-neighbouring points per thread, fed from a shared-memory plane
// ring. Every plane (tile plus x/y halo, raw values) reaches the ring by 16-byte cp.async
// copies R + D planes before the block computes it, the potential and recurrence-term pairs D
// planes before, and the register z-queue is topped up from the ring (plane k+R), so no step
// waits on a global load issued in the same step. The thread that copied an entry from
// outside the cell multiplies it in place by its Bloch factor one step before the plane is
// used (between the barriers, beside the computation of the current plane, so no step waits
// on it); the z-queue entries get theirs when they are topped up. The factors come from a
// per-k table e^{i d k_a L_a} (d = -1, 0, 1), so the kernel evaluates no sine or cosine. The
// host checks that every fetch is at most one period away, that Nx, the leading dimensions
// and the column bases give 16-byte aligned pairs, and that the copies fit kPairCopies per
// thread. The plane loop is unrolled by the queue length 2R+1 so the queue rotates by
// renaming; neighbour sums use the packed f32x2 add and the weighted sums three FMA chains
// per point whose weights stay in the parameter bank.
struct ZPairConst {               // launch-wide: read from the parameter bank
    float wx[kMaxFDn + 1], wy[kMaxFDn + 1], wz[kMaxFDn + 1];
    int Nx, Ny, Nz, zlen, nslab;
};
struct ZPairParams {              // per column
    const float2 *__restrict__ x;
    float2 *__restrict__ out;
    const float2 *__restrict__ z;
    const float *__restrict__ v32;
    long ldx, ldo, ldz;           // complex elements
    float c0, s1, s2;
    float2 bf[9];                 // e^{i d k_a L_a}, index 3 a + d + 1
};

// bf[3 a + d + 1] for d in {-1, 0, 1}, without dynamic indexing
__device__ __forceinline__ float2 bsel(const float2 *bf, int a, int d)
{
    return d < 0 ? bf[3 * a] : (d > 0 ? bf[3 * a + 2] : bf[3 * a + 1]);
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float4 cmul2f(float4 v, float2 f)
{
    const float2 lo = cmulf(make_float2(v.x, v.y), f), hi = cmulf(make_float2(v.z, v.w), f);
    return make_float4(lo.x, lo.y, hi.x, hi.y);
}
__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float2 wfma(float2 s, float w, float2 acc)
{
    return make_float2(fmaf(s.x, w, acc.x), fmaf(s.y, w, acc.y));
}

constexpr int kPairCopies = 4;    // ring copies per thread and plane (host-checked)
constexpr int kPairAhead = 4;     // D: planes copied ahead of their use

// shared-memory layout of the ring kernel for a BX2 x BY block
struct ZRing {
    int W, H, SLOT, NR, NV, ncopy;
    size_t bytes;
};
__host__ __device__ inline ZRing zring_shape(int bx2, int by, int R, int D)
{
    ZRing z;
    z.W = 2 * bx2 + 2 * R;                 // complex entries per ring row (x-halo R each side)
    z.H = by + 2 * R;
    z.SLOT = z.W * z.H;
    z.NR = R + D + 1;                      // ring slots: planes k .. k+R+D
    z.NV = D + 1;                          // potential / recurrence slots: planes k .. k+D
    z.ncopy = by * (z.W / 2) + 2 * R * bx2;  // pair copies per plane
    z.bytes = sizeof(float2) * ((size_t)z.NR * z.SLOT + (size_t)z.NV * by * 2 * bx2) +
              sizeof(float) * (size_t)z.NV * by * 2 * bx2;
    return z;
}

template <int R>
__device__ __forceinline__ void stencil_c64_pairs(const ZPairConst &g, const ZPairParams &p,
                                                  int col, int slab)
{
    constexpr int Q = 2 * R + 1;
    constexpr int D = kPairAhead;
    constexpr int NU = kPairCopies;
    static_assert(Q == 13 && R % 2 == 0, "the unrolled z-loop is written for radius 6");
    extern __shared__ __align__(16) unsigned char zst_raw[];
    const int BX2 = blockDim.x, BY = blockDim.y, BX = 2 * BX2;
    const ZRing S = zring_shape(BX2, BY, R, D);
    float2 *ring = reinterpret_cast<float2 *>(zst_raw);
    float2 *zslots = ring + S.NR * S.SLOT;                        // [NV][BY][BX]
    float *vslots = reinterpret_cast<float *>(zslots + S.NV * BY * BX);  // [NV][BY][BX]
    const int tx = threadIdx.x, ty = threadIdx.y, NT = BX2 * BY;
    const int tid = ty * BX2 + tx;
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    const int zs = slab * g.zlen;
    const int ze = min(zs + g.zlen, g.Nz);
    if (zs >= ze) return;
    const int i0 = x0 + 2 * tx, j = y0 + ty;
    const bool active = (i0 < g.Nx) && (j < g.Ny);
    const int dxo = floordiv(i0, g.Nx), dyo = floordiv(j, g.Ny);
    const int own = (wrapz(i0, g.Nx) + wrapz(j, g.Ny) * g.Nx) >> 1;  // pair index
    const int NxNy2 = (g.Nx * g.Ny) >> 1;
    const float4 *__restrict__ xc = reinterpret_cast<const float4 *>(p.x + (long)col * p.ldx);
    const float4 *__restrict__ zc =
        p.z ? reinterpret_cast<const float4 *>(p.z + (long)col * p.ldz) : nullptr;
    const float2 *__restrict__ vc = p.v32 ? reinterpret_cast<const float2 *>(p.v32) : nullptr;
    float4 *__restrict__ oc = reinterpret_cast<float4 *>(p.out + (long)col * p.ldo);
    const float2 fo = cmulf(bsel(p.bf, 0, dxo), bsel(p.bf, 1, dyo));
    const float2 fzm = cmulf(fo, p.bf[6]), fzp = cmulf(fo, p.bf[8]);
    const bool own_cell = dxo == 0 && dyo == 0;

    // this thread's ring copies of a plane: source pair offset, destination byte offset in a
    // slot, and the Bloch factor of entries outside the cell (bit u of fix)
    int gofs[NU], sofs[NU];
    float2 fct[NU];
    unsigned fix = 0;
    const int CROW = S.W / 2;
#pragma unroll
    for (int u = 0; u < NU; u++) {
        const int e = tid + u * NT;
        gofs[u] = 0;
        sofs[u] = -1;
        fct[u] = make_float2(1.f, 0.f);
        if (e < S.ncopy) {
            int r, c;
            if (e < BY * CROW) {
                r = R + e / CROW;
                c = 2 * (e % CROW);
            } else {
                const int e2 = e - BY * CROW, hr = e2 / BX2;
                r = hr < R ? hr : hr + BY;
                c = R + 2 * (e2 % BX2);
            }
            const int xg = x0 - R + c, yg = y0 - R + r;
            gofs[u] = (wrapz(yg, g.Ny) * g.Nx + wrapz(xg, g.Nx)) >> 1;
            sofs[u] = (int)sizeof(float2) * (r * S.W + c);
            const int dx = floordiv(xg, g.Nx), dy = floordiv(yg, g.Ny);
            if (dx != 0 || dy != 0) {
                fix |= 1u << u;
                fct[u] = cmulf(bsel(p.bf, 0, dx), bsel(p.bf, 1, dy));
            }
        }
    }
    const unsigned sring = (unsigned)__cvta_generic_to_shared(ring);
    const unsigned szs = (unsigned)__cvta_generic_to_shared(zslots + ty * BX + 2 * tx);
    const unsigned svs = (unsigned)__cvta_generic_to_shared(vslots + ty * BX + 2 * tx);
    const int NzNxNy2 = g.Nz * NxNy2;

    int pw = zs * NxNy2, rs = zs % S.NR;  // next ring plane to copy (offset, slot)
    int vo = zs * NxNy2, vsl = zs % S.NV; // next potential / recurrence plane
    auto issue = [&](bool ringon, bool vzon) {
        if (ringon) {
            const float4 *pl = xc + pw;
            const unsigned dst = sring + (unsigned)(rs * S.SLOT * (int)sizeof(float2));
#pragma unroll
            for (int u = 0; u < NU; u++)
                if (sofs[u] >= 0) cp_async16s(dst + sofs[u], pl + gofs[u]);
            pw += NxNy2;
            if (pw == NzNxNy2) pw = 0;
            rs = rs + 1 == S.NR ? 0 : rs + 1;
        }
        if (vzon) {
            if (zc) cp_async16s(szs + (unsigned)(vsl * BY * BX * (int)sizeof(float2)), zc + own + vo);
            if (vc) cp_async8s(svs + (unsigned)(vsl * BY * BX * (int)sizeof(float)), vc + own + vo);
            vo += NxNy2;
            vsl = vsl + 1 == S.NV ? 0 : vsl + 1;
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
    // Bloch factors on this thread's (landed) copies of the ring plane in slot sl
    auto fixup = [&](int sl) {
        if (!fix) return;
        char *base = reinterpret_cast<char *>(ring + sl * S.SLOT);
#pragma unroll
        for (int u = 0; u < NU; u++) {
            if (fix & (1u << u)) {
                float4 *e = reinterpret_cast<float4 *>(base + sofs[u]);
                *e = cmul2f(*e, fct[u]);
            }
        }
    };
    auto zfac = [&](float4 v, int kr) -> float4 {  // own pair of unwrapped plane kr
        const int d = kr < 0 ? -1 : (kr >= g.Nz ? 1 : 0);
        if (own_cell && d == 0) return v;
        return cmul2f(v, d == 0 ? fo : (d < 0 ? fzm : fzp));
    };

    // prologue: the queue holds planes zs-R .. zs+R-1 (from global memory); the ring receives
    // planes zs .. zs+R+D-1 and the potential planes zs .. zs+D-1 (the groups of steps
    // zs-R-D .. zs-1: group jj copies ring plane zs+jj and potential plane zs+jj-R)
    float4 q[Q];
#pragma unroll
    for (int m = 0; m < 2 * R; m++) {
        const int kr = zs - R + m;
        const int d = kr < 0 ? -1 : (kr >= g.Nz ? 1 : 0);
        q[m] = zfac(__ldg(xc + own + (kr - d * g.Nz) * NxNy2), kr);
    }
    for (int jj = 0; jj < R + D; jj++) {
        const int kstep = zs - R - D + jj;
        issue(kstep + D < ze, jj >= R && kstep + D < ze);
    }
    cp_async_wait_group<D>();  // ring planes zs .. zs+R-1 have landed
    fixup(zs % S.NR);          // plane zs; each later plane one step before its use
    int sk = zs % S.NR, svk = zs % S.NV;
    int ko = zs * NxNy2;
    const float c0 = p.c0, s1 = p.s1, s2 = p.s2;

#define SGPU_ZRING_STEP(U)                                                                       \
    {                                                                                            \
        const int k = kb + (U);                                                                  \
        if (k < ze) {                                                                            \
            cp_async_wait_group<D - 1>(); /* ring plane k+R and potential plane k landed */      \
            const int skr = sk + R >= S.NR ? sk + R - S.NR : sk + R;                             \
            __syncthreads();                                                                     \
            issue(k + D < ze, k + D < ze);                                                       \
            const float2 *sl = ring + sk * S.SLOT;                                               \
            const float2 *srow = sl + (ty + R) * S.W + R + 2 * tx;                               \
            if (active)                                                                          \
                q[((U) + 2 * R) % Q] = zfac(*reinterpret_cast<const float4 *>(                   \
                    ring + skr * S.SLOT + (ty + R) * S.W + R + 2 * tx), k + R);                  \
            if (k + 1 < ze) fixup(sk + 1 == S.NR ? 0 : sk + 1);                                  \
            if (active) {                                                                        \
                const float4 cen = q[((U) + R) % Q];                                             \
                float2 xa[2 * R + 2];                                                            \
                _Pragma("unroll") for (int t = -R; t <= R; t += 2) {                             \
                    const float4 v = t == 0 ? cen : *reinterpret_cast<const float4 *>(srow + t); \
                    xa[t + R] = lo2(v);                                                          \
                    xa[t + R + 1] = hi2(v);                                                      \
                }                                                                                \
                float2 rx0 = make_float2(c0 * xa[R].x, c0 * xa[R].y);                            \
                float2 rx1 = make_float2(c0 * xa[R + 1].x, c0 * xa[R + 1].y);                    \
                float2 ry0{0.f, 0.f}, ry1{0.f, 0.f}, rz0{0.f, 0.f}, rz1{0.f, 0.f};               \
                _Pragma("unroll") for (int r = 1; r <= R; r++) {                                 \
                    const float4 up = *reinterpret_cast<const float4 *>(srow - r * S.W);         \
                    const float4 dn = *reinterpret_cast<const float4 *>(srow + r * S.W);         \
                    const float4 zm_ = q[((U) + R - r + Q) % Q], zp_ = q[((U) + R + r) % Q];     \
                    const float a = g.wx[r], b = g.wy[r], c = g.wz[r];                           \
                    rx0 = wfma(__fadd2_rn(xa[R - r], xa[R + r]), a, rx0);                        \
                    rx1 = wfma(__fadd2_rn(xa[R + 1 - r], xa[R + 1 + r]), a, rx1);                \
                    ry0 = wfma(__fadd2_rn(lo2(up), lo2(dn)), b, ry0);                            \
                    ry1 = wfma(__fadd2_rn(hi2(up), hi2(dn)), b, ry1);                            \
                    rz0 = wfma(__fadd2_rn(lo2(zm_), lo2(zp_)), c, rz0);                          \
                    rz1 = wfma(__fadd2_rn(hi2(zm_), hi2(zp_)), c, rz1);                          \
                }                                                                                \
                float2 res0 = __fadd2_rn(rx0, __fadd2_rn(ry0, rz0));                             \
                float2 res1 = __fadd2_rn(rx1, __fadd2_rn(ry1, rz1));                             \
                if (vc) {                                                                        \
                    const float2 vv = *reinterpret_cast<const float2 *>(                         \
                        vslots + (svk * BY + ty) * BX + 2 * tx);                                 \
                    res0 = wfma(lo2(cen), vv.x, res0);                                           \
                    res1 = wfma(hi2(cen), vv.y, res1);                                           \
                }                                                                                \
                float2 o0 = make_float2(s1 * res0.x, s1 * res0.y);                               \
                float2 o1 = make_float2(s1 * res1.x, s1 * res1.y);                               \
                if (zc) {                                                                        \
                    const float4 zz = *reinterpret_cast<const float4 *>(                         \
                        zslots + (svk * BY + ty) * BX + 2 * tx);                                 \
                    o0 = wfma(lo2(zz), s2, o0);                                                  \
                    o1 = wfma(hi2(zz), s2, o1);                                                  \
                }                                                                                \
                oc[own + ko] = make_float4(o0.x, o0.y, o1.x, o1.y);                              \
            }                                                                                    \
            sk = sk + 1 == S.NR ? 0 : sk + 1;                                                    \
            svk = svk + 1 == S.NV ? 0 : svk + 1;                                                 \
            ko += NxNy2;                                                                         \
        }                                                                                        \
    }

    for (int kb = zs; kb < ze; kb += Q) {
        SGPU_ZRING_STEP(0) SGPU_ZRING_STEP(1) SGPU_ZRING_STEP(2) SGPU_ZRING_STEP(3)
        SGPU_ZRING_STEP(4) SGPU_ZRING_STEP(5) SGPU_ZRING_STEP(6) SGPU_ZRING_STEP(7)
        SGPU_ZRING_STEP(8) SGPU_ZRING_STEP(9) SGPU_ZRING_STEP(10) SGPU_ZRING_STEP(11)
        SGPU_ZRING_STEP(12)
    }
#undef SGPU_ZRING_STEP
    cp_async_wait_all();
}

}  // namespace
}  // namespace sgpu
