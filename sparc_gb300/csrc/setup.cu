// Atom-dependent set-up on the device: pseudopotential tables, pseudocharge cut-off radii,
// pseudocharge density with its reference-potential correction (self and correction energy),
// atomic superposition and model core densities, and the nonlocal projectors.
//
// Restates, for orthogonal periodic cells:
//   getYD_gen                     src/tools.c:372   (cubic-spline slopes, not-a-knot ends)
//   SplineInterpUniform/Nonuniform src/tools.c:552, :605
//   RealSphericalHarmonic         src/tools.c:1231  (l <= 3 here)
//   Calculate_PseudochargeCutoff  src/electrostatics.c:44
//   GetInfluencingAtoms           src/electrostatics.c:578
//   Generate_PseudoChargeDensity  src/electrostatics.c:772
//   Calculate_Pseudopot_Ref       src/electrostatics.c:1465
//   GetInfluencingAtoms_nloc      src/nlocVecRoutines.c:43
//   CalculateNonlocalProjectors   src/nlocVecRoutines.c:394
//
// Host code does the index work (which periodic images touch the cell, which grid points lie
// inside a projector sphere) and the one-off cut-off search on a small atom-centred box; the
// grid-sized work runs on the device: one thread per (image, point) evaluates the splined local
// potential on the 37-point stencil around its point, applies -Lap/(4 pi), and accumulates the
// pseudocharge, the reference pseudocharge, the potential difference Vc and both densities
// with atomics; a second kernel reduces the charges and energy terms. The projector values
// (spline of UdV times a real spherical harmonic) are one thread per (image, point).
#include "sgpu_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace sgpu {

constexpr int kMaxTypes = 8;
constexpr double kTinyR = 1e-12;  // TEMP_TOL of the reference set-up files

// ------------------------------------------------------------------ splines

// Slopes YD of the cubic spline through (X, Y) with not-a-knot end conditions, by one
// tridiagonal solve (getYD_gen, src/tools.c:372-409).
static void spline_slopes(const double *X, const double *Y, double *YD, int n)
{
    std::vector<double> A(n, 0.0), B(n, 0.0), C(n, 0.0);
    double h0 = X[1] - X[0], h1 = X[2] - X[1];
    double r0 = (Y[1] - Y[0]) / h0, r1 = (Y[2] - Y[1]) / h1;
    B[0] = h1 * (h0 + h1);
    C[0] = (h0 + h1) * (h0 + h1);
    YD[0] = r0 * (3 * h0 * h1 + 2 * h1 * h1) + r1 * h0 * h0;
    int i;
    for (i = 1; i < n - 1; i++) {
        h0 = X[i] - X[i - 1];
        h1 = X[i + 1] - X[i];
        r0 = (Y[i] - Y[i - 1]) / h0;
        r1 = (Y[i + 1] - Y[i]) / h1;
        A[i] = h1;
        B[i] = 2 * (h0 + h1);
        C[i] = h0;
        YD[i] = 3 * (r0 * h1 + r1 * h0);
    }
    A[i] = (h0 + h1) * (h0 + h1);
    B[i] = h0 * (h0 + h1);
    YD[i] = r0 * h1 * h1 + r1 * (3 * h0 * h1 + 2 * h0 * h0);
    // Thomas algorithm (tridiag_gen, src/tools.c:413)
    std::vector<double> F(n, 0.0);
    double piv = B[0];
    YD[0] /= piv;
    for (i = 1; i < n; i++) {
        F[i] = C[i - 1] / piv;
        piv = B[i] - A[i] * F[i];
        YD[i] = (YD[i] - YD[i - 1] * A[i]) / piv;
    }
    for (i = n - 2; i >= 0; i--) YD[i] -= YD[i + 1] * F[i + 1];
}

// Cubic Hermite evaluation on interval j of (X, Y, YD) at x (SplineInterpUniform /
// SplineInterpNonuniform body). The caller keeps x within [X[0], X[n-1]].
__host__ __device__ inline double spline_at(const double *X, const double *Y, const double *YD,
                                            int n, int uniform, double x)
{
    int j;
    if (uniform) {
        j = (int)floor((x - X[0]) / (X[1] - X[0]));
    } else {
        int lo = 0, hi = n - 1;  // X[lo] <= x < X[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (X[mid] <= x) lo = mid; else hi = mid;
        }
        j = lo;
    }
    j = j < 0 ? 0 : (j > n - 2 ? n - 2 : j);
    const double p1 = X[j], p3 = X[j + 1];
    const double dx = 1.0 / (p3 - p1);
    const double dy = (Y[j + 1] - Y[j]) * dx;
    const double a1 = YD[j];
    const double a2 = dx * (3.0 * dy - 2.0 * YD[j] - YD[j + 1]);
    const double a3 = dx * dx * (-2.0 * dy + YD[j] + YD[j + 1]);
    const double t = x - p1;
    return ((a3 * t + a2) * t + a1) * t + Y[j];
}

// ------------------------------------------------------------------ per-type tables

struct PsdDev {
    const double *grid, *rvloc, *yd_rvloc, *rhoiso, *yd_rhoiso, *rhoc, *yd_rhoc, *udv, *yd_udv;
    int size, uniform, Znucl;
    double Vloc0, rchrg;
};

struct PsdTable {
    int size = 0, lmax = 0, lloc = 0, uniform = 0, Znucl = 0, nproj_atom = 0, nrad = 0;
    double Vloc0 = 0.0, fchrg = 0.0, rchrg = 0.0, rc_max = 0.0;
    std::vector<int> ppl, lpos;
    std::vector<double> rc, grid, udv, rvloc, rhoiso, rhoc, gamma;
    std::vector<double> yd_udv, yd_rvloc, yd_rhoiso, yd_rhoc;
    double cutoff[3] = {0.0, 0.0, 0.0};
    bool has_cutoff = false;
    double *dev = nullptr;
    PsdDev view{};
};

struct SetupState {
    std::vector<PsdTable> types;
    ~SetupState()
    {
        for (auto &t : types)
            if (t.dev) cudaFree(t.dev);
    }
};

void setup_free(sgpu_ctx *ctx)
{
    delete ctx->setup;
    ctx->setup = nullptr;
}

struct PsdDevSet {
    PsdDev t[kMaxTypes];
};

// ------------------------------------------------------------------ device helpers

// V_J(R): the splined local potential rVloc/R, Vloc(0) at the centre and -Z/R beyond the
// table (Generate_PseudoChargeDensity, src/electrostatics.c:978-986)
__host__ __device__ inline double vloc_at(const PsdDev &p, double R)
{
    if (R < kTinyR) return p.Vloc0;
    if (R > p.rchrg) return -(double)p.Znucl / R;
    return spline_at(p.grid, p.rvloc, p.yd_rvloc, p.size, p.uniform, R) / R;
}

// reference potential of a smeared charge -Z inside rcut (Calculate_Pseudopot_Ref,
// src/electrostatics.c:1465, after J.E. Pask, N. Sukumar and S.E. Mousavi)
__host__ __device__ inline double vref_at(double R, double rcut, double Z)
{
    if (R <= rcut) {
        const double R2 = R * R, C3 = rcut * rcut * rcut, C6 = C3 * C3;
        const double v = R2 * (R2 * R * (5.6 / C6 + R * (1.8 * R / (C6 * rcut * rcut) -
                                                          6.0 / (C6 * rcut))) -
                               2.8 / C3) + 2.4 / rcut;
        return -Z * v;
    }
    return -Z / R;
}

struct PcImage {
    double x0, y0, z0;  // image position
    int xs, ys, zs;     // first grid index of the clipped rb-box
    int nx, ny, nz;     // box extents
    int type;
    int atom;           // index of the atom (type-major order)
};

struct PcWeights {
    double w[3 * (kMaxFDn + 1)];  // (x, y, z) weights per offset, times -1/(4 pi)
    double w0;                    // centre weight
};

__device__ inline double block_sum(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
    return s;
}

// One thread per point of the rb-box of one image: bJ = -Lap(V_J)/(4 pi) and the reference
// twin, accumulated into the cell (src/electrostatics.c:1040-1076); rho_J and rho_c_J as well
// (:1005-1034). The image's -sum(bJ_ref * VJ_ref) goes to esc_acc.
__global__ void __launch_bounds__(256) k_pseudocharge(
    const PcImage *__restrict__ imgs, PsdDevSet P, PcWeights W, int FDn, int Nx, int Ny,
    double dx, double dy, double dz, double ref_cutoff, double *__restrict__ b,
    double *__restrict__ bref, double *__restrict__ vc, double *__restrict__ rho_at,
    double *__restrict__ rho_core, double *__restrict__ esc_acc)
{
    __shared__ double red[8];
    const PcImage im = imgs[blockIdx.y];
    const long npts = (long)im.nx * im.ny * im.nz;
    const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    double esc = 0.0;
    if (p < npts) {
        const PsdDev &ps = P.t[im.type];
        const double Z = (double)ps.Znucl;
        const int i = (int)(p % im.nx);
        const int j = (int)((p / im.nx) % im.ny);
        const int k = (int)(p / ((long)im.nx * im.ny));
        // coordinates as the reference forms them on its extended box: index * h - shifted
        // image position, with the box corner at (xs - FDn, ys - FDn, zs - FDn)
        const double xsh = im.x0 - dx * (im.xs - FDn);
        const double ysh = im.y0 - dy * (im.ys - FDn);
        const double zsh = im.z0 - dz * (im.zs - FDn);
        const double xc = (i + FDn) * dx - xsh, yc = (j + FDn) * dy - ysh,
                     zc = (k + FDn) * dz - zsh;
        const double R0 = sqrt(xc * xc + yc * yc + zc * zc);
        const double v0 = vloc_at(ps, R0), vr0 = vref_at(R0, ref_cutoff, Z);
        double s = W.w0 * v0, sr = W.w0 * vr0;
        for (int r = 1; r <= FDn; r++) {
            const double xm = (i + FDn - r) * dx - xsh, xp = (i + FDn + r) * dx - xsh;
            const double ym = (j + FDn - r) * dy - ysh, yp = (j + FDn + r) * dy - ysh;
            const double zm = (k + FDn - r) * dz - zsh, zp = (k + FDn + r) * dz - zsh;
            const double Rxm = sqrt(xm * xm + yc * yc + zc * zc), Rxp = sqrt(xp * xp + yc * yc + zc * zc);
            const double Rym = sqrt(xc * xc + ym * ym + zc * zc), Ryp = sqrt(xc * xc + yp * yp + zc * zc);
            const double Rzm = sqrt(xc * xc + yc * yc + zm * zm), Rzp = sqrt(xc * xc + yc * yc + zp * zp);
            const double tx = (vloc_at(ps, Rxm) + vloc_at(ps, Rxp)) * W.w[3 * r];
            const double ty = (vloc_at(ps, Rym) + vloc_at(ps, Ryp)) * W.w[3 * r + 1];
            const double tz = (vloc_at(ps, Rzm) + vloc_at(ps, Rzp)) * W.w[3 * r + 2];
            s += tx + ty + tz;
            const double rx = (vref_at(Rxm, ref_cutoff, Z) + vref_at(Rxp, ref_cutoff, Z)) * W.w[3 * r];
            const double ry = (vref_at(Rym, ref_cutoff, Z) + vref_at(Ryp, ref_cutoff, Z)) * W.w[3 * r + 1];
            const double rz = (vref_at(Rzm, ref_cutoff, Z) + vref_at(Rzp, ref_cutoff, Z)) * W.w[3 * r + 2];
            sr += rx + ry + rz;
        }
        double rho = 0.0, rhoc = 0.0;
        if (R0 <= ps.rchrg) {
            rho = spline_at(ps.grid, ps.rhoiso, ps.yd_rhoiso, ps.size, ps.uniform, R0);
            rhoc = spline_at(ps.grid, ps.rhoc, ps.yd_rhoc, ps.size, ps.uniform, R0);
        }
        const long g = (long)(im.zs + k) * Nx * Ny + (long)(im.ys + j) * Nx + (im.xs + i);
        atomicAdd(&b[g], s);
        atomicAdd(&bref[g], sr);
        atomicAdd(&vc[g], vr0 - v0);
        atomicAdd(&rho_at[g], rho);
        atomicAdd(&rho_core[g], rhoc);
        esc = -sr * vr0;
    }
    const double tot = block_sum(esc, red);
    if (threadIdx.x == 0 && tot != 0.0) atomicAdd(esc_acc, tot);
}

// Initial magnetization of a collinear-spin run: each atom's isolated-atom density rho_J
// (within its rb-box and rchrg, as k_pseudocharge accumulates rho_at) weighted by
// w[atom] = spin_z / Znucl (src/electrostatics.c:1031-1034).
__global__ void __launch_bounds__(256) k_mag_at(const PcImage *__restrict__ imgs, PsdDevSet P,
                                                int FDn, int Nx, int Ny, double dx, double dy,
                                                double dz, const double *__restrict__ w,
                                                double *__restrict__ mag)
{
    const PcImage im = imgs[blockIdx.y];
    const long npts = (long)im.nx * im.ny * im.nz;
    const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    const double wa = w[im.atom];
    if (wa == 0.0) return;
    const PsdDev &ps = P.t[im.type];
    const int i = (int)(p % im.nx);
    const int j = (int)((p / im.nx) % im.ny);
    const int k = (int)(p / ((long)im.nx * im.ny));
    const double xc = (i + FDn) * dx - (im.x0 - dx * (im.xs - FDn));
    const double yc = (j + FDn) * dy - (im.y0 - dy * (im.ys - FDn));
    const double zc = (k + FDn) * dz - (im.z0 - dz * (im.zs - FDn));
    const double R0 = sqrt(xc * xc + yc * yc + zc * zc);
    if (R0 > ps.rchrg) return;
    const double rho = spline_at(ps.grid, ps.rhoiso, ps.yd_rhoiso, ps.size, ps.uniform, R0);
    const long g = (long)(im.zs + k) * Nx * Ny + (long)(im.ys + j) * Nx + (im.xs + i);
    atomicAdd(&mag[g], wa * rho);
}

struct D1Weights {
    double d[3 * (kMaxFDn + 1)];  // first-derivative weights per offset and direction (x, y, z)
};

// Local forces (Calculate_local_forces_linear, src/forces.c:157-434). One thread per point of
// one image's rb-box: bJ and bJ_ref as k_pseudocharge forms them, the D1 gradient of
// VcJ = VJ_ref - VJ from the values at the stencil points, and the cell fields b + b_ref,
// grad(phi) and grad(Vc) (gphi, gvc: three Nd blocks each). The image's sum of
//   -bJ grad(phi) + (grad(VcJ) (b + b_ref) - grad(Vc) (bJ + bJ_ref)) / 2
// times dV is added to the force of its atom.
__global__ void __launch_bounds__(256) k_local_forces(
    const PcImage *__restrict__ imgs, PsdDevSet P, PcWeights W, D1Weights G, int FDn, int Nx,
    int Ny, double dx, double dy, double dz, double ref_cutoff, const double *__restrict__ b,
    const double *__restrict__ bref, const double *__restrict__ gphi,
    const double *__restrict__ gvc, long Nd, double dV, double *__restrict__ forces)
{
    __shared__ double red[8];
    const PcImage im = imgs[blockIdx.y];
    const long npts = (long)im.nx * im.ny * im.nz;
    const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    double f[3] = {0.0, 0.0, 0.0};
    if (p < npts) {
        const PsdDev &ps = P.t[im.type];
        const double Z = (double)ps.Znucl;
        const int i = (int)(p % im.nx);
        const int j = (int)((p / im.nx) % im.ny);
        const int k = (int)(p / ((long)im.nx * im.ny));
        const double xsh = im.x0 - dx * (im.xs - FDn);
        const double ysh = im.y0 - dy * (im.ys - FDn);
        const double zsh = im.z0 - dz * (im.zs - FDn);
        const double xc = (i + FDn) * dx - xsh, yc = (j + FDn) * dy - ysh,
                     zc = (k + FDn) * dz - zsh;
        const double R0 = sqrt(xc * xc + yc * yc + zc * zc);
        double s = W.w0 * vloc_at(ps, R0), sr = W.w0 * vref_at(R0, ref_cutoff, Z);
        double dvc[3] = {0.0, 0.0, 0.0};
        for (int r = 1; r <= FDn; r++) {
            const double xm = (i + FDn - r) * dx - xsh, xp = (i + FDn + r) * dx - xsh;
            const double ym = (j + FDn - r) * dy - ysh, yp = (j + FDn + r) * dy - ysh;
            const double zm = (k + FDn - r) * dz - zsh, zp = (k + FDn + r) * dz - zsh;
            const double Rs[6] = {sqrt(xm * xm + yc * yc + zc * zc), sqrt(xp * xp + yc * yc + zc * zc),
                                  sqrt(xc * xc + ym * ym + zc * zc), sqrt(xc * xc + yp * yp + zc * zc),
                                  sqrt(xc * xc + yc * yc + zm * zm), sqrt(xc * xc + yc * yc + zp * zp)};
            double v[6], vr[6];
#pragma unroll
            for (int q = 0; q < 6; q++) {
                v[q] = vloc_at(ps, Rs[q]);
                vr[q] = vref_at(Rs[q], ref_cutoff, Z);
            }
            s += (v[0] + v[1]) * W.w[3 * r] + (v[2] + v[3]) * W.w[3 * r + 1] +
                 (v[4] + v[5]) * W.w[3 * r + 2];
            sr += (vr[0] + vr[1]) * W.w[3 * r] + (vr[2] + vr[3]) * W.w[3 * r + 1] +
                  (vr[4] + vr[5]) * W.w[3 * r + 2];
#pragma unroll
            for (int d = 0; d < 3; d++)
                dvc[d] += ((vr[2 * d + 1] - v[2 * d + 1]) - (vr[2 * d] - v[2 * d])) * G.d[3 * r + d];
        }
        const long g = (long)(im.zs + k) * Nx * Ny + (long)(im.ys + j) * Nx + (im.xs + i);
        const double bb = b[g] + bref[g], bj = s + sr;
#pragma unroll
        for (int d = 0; d < 3; d++)
            f[d] = -s * gphi[d * Nd + g] + 0.5 * (dvc[d] * bb - gvc[d * Nd + g] * bj);
    }
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const double t = block_sum(f[d], red);
        if (threadIdx.x == 0) atomicAdd(&forces[3 * im.atom + d], t * dV);
        __syncthreads();
    }
}

// Core-correction (NLCC) forces (Calculate_forces_xc_linear, src/forces.c:473-700): one thread
// per point of one image's rb-box; the D1 gradient of the splined core density rho_c,J (zero
// beyond the table) from its values at the stencil points, times Vxc, summed over the box and
// added (times dV) to the force of the image's atom.
__global__ void __launch_bounds__(256) k_xc_forces(
    const PcImage *__restrict__ imgs, PsdDevSet P, D1Weights G, int FDn, int Nx, int Ny,
    double dx, double dy, double dz, const double *__restrict__ vxc, double dV,
    double *__restrict__ forces)
{
    __shared__ double red[8];
    const PcImage im = imgs[blockIdx.y];
    const long npts = (long)im.nx * im.ny * im.nz;
    const long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
    double f[3] = {0.0, 0.0, 0.0};
    if (p < npts) {
        const PsdDev &ps = P.t[im.type];
        const int i = (int)(p % im.nx);
        const int j = (int)((p / im.nx) % im.ny);
        const int k = (int)(p / ((long)im.nx * im.ny));
        const double xsh = im.x0 - dx * (im.xs - FDn);
        const double ysh = im.y0 - dy * (im.ys - FDn);
        const double zsh = im.z0 - dz * (im.zs - FDn);
        const double xc = (i + FDn) * dx - xsh, yc = (j + FDn) * dy - ysh,
                     zc = (k + FDn) * dz - zsh;
        auto rhoc = [&](double R) {
            return R <= ps.rchrg ? spline_at(ps.grid, ps.rhoc, ps.yd_rhoc, ps.size, ps.uniform, R)
                                 : 0.0;
        };
        double drc[3] = {0.0, 0.0, 0.0};
        for (int r = 1; r <= FDn; r++) {
            const double xm = (i + FDn - r) * dx - xsh, xp = (i + FDn + r) * dx - xsh;
            const double ym = (j + FDn - r) * dy - ysh, yp = (j + FDn + r) * dy - ysh;
            const double zm = (k + FDn - r) * dz - zsh, zp = (k + FDn + r) * dz - zsh;
            drc[0] += (rhoc(sqrt(xp * xp + yc * yc + zc * zc)) -
                       rhoc(sqrt(xm * xm + yc * yc + zc * zc))) * G.d[3 * r];
            drc[1] += (rhoc(sqrt(xc * xc + yp * yp + zc * zc)) -
                       rhoc(sqrt(xc * xc + ym * ym + zc * zc))) * G.d[3 * r + 1];
            drc[2] += (rhoc(sqrt(xc * xc + yc * yc + zp * zp)) -
                       rhoc(sqrt(xc * xc + yc * yc + zm * zm))) * G.d[3 * r + 2];
        }
        const long g = (long)(im.zs + k) * Nx * Ny + (long)(im.ys + j) * Nx + (im.xs + i);
        const double v = vxc[g];
#pragma unroll
        for (int d = 0; d < 3; d++) f[d] = v * drc[d];
    }
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const double t = block_sum(f[d], red);
        if (threadIdx.x == 0) atomicAdd(&forces[3 * im.atom + d], t * dV);
        __syncthreads();
    }
}

// sums over the cell: [0] b, [1] rho_at, [2] (b + bref) * Vc
__global__ void __launch_bounds__(256) k_charge_sums(const double *__restrict__ b,
                                                     const double *__restrict__ bref,
                                                     const double *__restrict__ vc,
                                                     const double *__restrict__ rho, long n,
                                                     double *__restrict__ out)
{
    __shared__ double red[8];
    double sb = 0.0, sr = 0.0, se = 0.0;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x) {
        sb += b[i];
        sr += rho[i];
        se += (b[i] + bref[i]) * vc[i];
    }
    double t = block_sum(sb, red);
    if (threadIdx.x == 0) atomicAdd(&out[0], t);
    __syncthreads();
    t = block_sum(sr, red);
    if (threadIdx.x == 0) atomicAdd(&out[1], t);
    __syncthreads();
    t = block_sum(se, red);
    if (threadIdx.x == 0) atomicAdd(&out[2], t);
}

__global__ void k_scale(double *x, long n, double s)
{
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long)gridDim.x * blockDim.x)
        x[i] *= s;
}

// ------------------------------------------------------------------ projectors

struct NlImage {
    double x0, y0, z0;
    long pos_off;   // first entry in grid_pos
    long chi_off;   // first entry in Chi
    int ndc, type;
};

struct NlTypeDev {
    int lmax, lloc, nproj;
    int ppl[8], lpos[8];
};

struct NlTypeSet {
    NlTypeDev t[kMaxTypes];
};

// real spherical harmonics Y_lm(x/r, y/r, z/r), l <= 3, m = -l..l, with the reference's sign
// convention (RealSphericalHarmonic, src/tools.c:1231)
__host__ __device__ inline double real_ylm(int l, int m, double x, double y, double z, double r)
{
    const double pi = 3.14159265358979323846;
    if (l == 0) return 0.5 * sqrt(1.0 / pi);
    if (r == 0.0) return 0.0;  // the reference divides by r here and returns NaN
    if (l == 1) {
        const double c = sqrt(3.0 / (4.0 * pi));
        return c * ((m == -1 ? y : (m == 0 ? z : x)) / r);
    }
    if (l == 2) {
        const double r2 = r * r;
        switch (m) {
        case -2: return 0.5 * sqrt(15.0 / pi) * (x * y) / r2;
        case -1: return 0.5 * sqrt(15.0 / pi) * (y * z) / r2;
        case 0: return 0.25 * sqrt(5.0 / pi) * (-x * x - y * y + 2.0 * z * z) / r2;
        case 1: return 0.5 * sqrt(15.0 / pi) * (z * x) / r2;
        default: return 0.25 * sqrt(15.0 / pi) * (x * x - y * y) / r2;
        }
    }
    const double r3 = r * r * r;
    switch (m) {
    case -3: return 0.25 * sqrt(35.0 / (2.0 * pi)) * (3 * x * x - y * y) * y / r3;
    case -2: return 0.5 * sqrt(105.0 / pi) * (x * y * z) / r3;
    case -1: return 0.25 * sqrt(21.0 / (2.0 * pi)) * y * (4 * z * z - x * x - y * y) / r3;
    case 0: return 0.25 * sqrt(7.0 / pi) * z * (2 * z * z - 3 * x * x - 3 * y * y) / r3;
    case 1: return 0.25 * sqrt(21.0 / (2.0 * pi)) * x * (4 * z * z - x * x - y * y) / r3;
    case 2: return 0.25 * sqrt(105.0 / pi) * z * (x * x - y * y) / r3;
    default: return 0.25 * sqrt(35.0 / (2.0 * pi)) * x * (x * x - 3 * y * y) / r3;
    }
}

// Chi[col * ndc + ipos] = UdV_{l,np}(r) * Y_lm for the image's points, columns in the
// reference's (l != lloc, np, m) order (src/nlocVecRoutines.c:529-561)
__global__ void __launch_bounds__(128) k_projectors(const NlImage *__restrict__ imgs,
                                                    const int *__restrict__ grid_pos,
                                                    PsdDevSet P, NlTypeSet T, int Nx, int Ny,
                                                    double dx, double dy, double dz,
                                                    double *__restrict__ chi)
{
    const NlImage im = imgs[blockIdx.y];
    const int ip = blockIdx.x * blockDim.x + threadIdx.x;
    if (ip >= im.ndc) return;
    const PsdDev &ps = P.t[im.type];
    const NlTypeDev &ty = T.t[im.type];
    const int g = grid_pos[im.pos_off + ip];
    const int kk = g / (Nx * Ny), jj = (g / Nx) % Ny, ii = g % Nx;
    const double x = ii * dx - im.x0, y = jj * dy - im.y0, z = kk * dz - im.z0;
    const double r = sqrt(x * x + y * y + z * z);
    double *out = chi + im.chi_off;
    int col = 0;
    for (int l = 0; l <= ty.lmax; l++) {
        if (l == ty.lloc) continue;
        for (int np = 0; np < ty.ppl[l]; np++) {
            const int row = ty.lpos[l] + np;
            const double u = spline_at(ps.grid, ps.udv + (long)row * ps.size,
                                       ps.yd_udv + (long)row * ps.size, ps.size, ps.uniform, r);
            for (int m = -l; m <= l; m++, col++)
                out[(long)col * im.ndc + ip] = u * real_ylm(l, m, x, y, z, r);
        }
    }
}

// ------------------------------------------------------------------ host helpers

static int get_setup(sgpu_ctx *ctx, SetupState **out)
{
    if (!ctx->setup || ctx->setup->types.empty()) {
        set_error("set-up call: sgpu_set_psd has not been called");
        return SGPU_ERR_STATE;
    }
    *out = ctx->setup;
    return SGPU_OK;
}

static PsdDevSet device_views(const SetupState &s)
{
    PsdDevSet v{};
    for (size_t t = 0; t < s.types.size(); t++) v.t[t] = s.types[t].view;
    return v;
}

static void grid_spacing(const sgpu_ctx *ctx, const double *cell, double h[3])
{
    h[0] = cell[0] / ctx->Nx;
    h[1] = cell[1] / ctx->Ny;
    h[2] = cell[2] / ctx->Nz;
}

// periodic image range of a coordinate x0 in a cell of length L for a radius rb
// (src/electrostatics.c:622-633)
static void image_range(double x0, double L, double rb, int *lo, int *hi)
{
    *hi = (int)std::floor((rb + L - x0) / L + kTinyR);
    *lo = -(int)std::floor((rb + x0) / L + kTinyR);
}

// copy n doubles of a device buffer to a caller array that may be host or device memory
static int deliver(const double *src, double *dst, long n, cudaStream_t st)
{
    if (!dst) return SGPU_OK;
    SGPU_CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDefault, st));
    return SGPU_OK;
}

// Images of every atom whose rb-box meets the cell, with the box clipped to the cell
// (GetInfluencingAtoms, src/electrostatics.c:578): rb = cutoff[3 * type + d], or the values of
// the last cut-off call when cutoff is NULL. maxpts: the largest box.
static int pc_images(const sgpu_ctx *ctx, const SetupState &s, const double *cell,
                     const double h[3], const int *nAtomv, const double *atom_pos,
                     const double *cutoff, const char *who, std::vector<PcImage> &imgs,
                     long *maxpts)
{
    const int N[3] = {ctx->Nx, ctx->Ny, ctx->Nz};
    imgs.clear();
    *maxpts = 0;
    int atom = 0;
    for (size_t t = 0; t < s.types.size(); t++) {
        double rb[3];
        for (int d = 0; d < 3; d++) {
            rb[d] = cutoff ? cutoff[3 * t + d] : s.types[t].cutoff[d];
            if (!(rb[d] > 0)) {
                set_error(std::string(who) + ": no cut-off for type " + std::to_string(t) +
                          " (call sgpu_Calculate_PseudochargeCutoff)");
                return SGPU_ERR_STATE;
            }
        }
        for (int a = 0; a < nAtomv[t]; a++, atom++) {
            const double *p0 = atom_pos + 3 * atom;
            int lo[3], hi[3];
            for (int d = 0; d < 3; d++) image_range(p0[d], cell[d], rb[d], &lo[d], &hi[d]);
            for (int rr = lo[2]; rr <= hi[2]; rr++) {
                const double z = p0[2] + cell[2] * rr;
                if (z < -rb[2] || z >= N[2] * h[2] + rb[2]) continue;
                for (int qq = lo[1]; qq <= hi[1]; qq++) {
                    const double y = p0[1] + cell[1] * qq;
                    if (y < -rb[1] || y >= N[1] * h[1] + rb[1]) continue;
                    for (int pp = lo[0]; pp <= hi[0]; pp++) {
                        const double x = p0[0] + cell[0] * pp;
                        if (x < -rb[0] || x >= N[0] * h[0] + rb[0]) continue;
                        const double c[3] = {x, y, z};
                        int s0[3], e0[3];
                        for (int d = 0; d < 3; d++) {
                            s0[d] = std::max(0, (int)std::ceil((c[d] - rb[d]) / h[d]));
                            e0[d] = std::min(N[d] - 1, (int)std::floor((c[d] + rb[d]) / h[d]));
                        }
                        if (e0[0] < s0[0] || e0[1] < s0[1] || e0[2] < s0[2]) continue;
                        PcImage im{x, y, z, s0[0], s0[1], s0[2], e0[0] - s0[0] + 1,
                                   e0[1] - s0[1] + 1, e0[2] - s0[2] + 1, (int)t, atom};
                        *maxpts = std::max(*maxpts, (long)im.nx * im.ny * im.nz);
                        imgs.push_back(im);
                    }
                }
            }
        }
    }
    return SGPU_OK;
}

// Runs k_pseudocharge over the images into zeroed device arrays b, bref, vc, rho, core (each
// Nd) and esc_acc (one value).
static int pseudocharge_fields(sgpu_ctx *ctx, const SetupState &s, const double h[3],
                               const std::vector<PcImage> &imgs, long maxpts,
                               double ref_cutoff, double *db, double *dbref, double *dvc,
                               double *drho, double *dcore, double *esc_acc, cudaStream_t st)
{
    if (imgs.empty()) return SGPU_OK;
    PcImage *dimg = nullptr;
    SGPU_CUDA_TRY(cudaMallocAsync(&dimg, sizeof(PcImage) * imgs.size(), st));
    int rc = SGPU_OK;
    if (cudaMemcpyAsync(dimg, imgs.data(), sizeof(PcImage) * imgs.size(),
                        cudaMemcpyHostToDevice, st) != cudaSuccess) {
        rc = SGPU_ERR_CUDA;
    } else {
        PcWeights W{};
        const double s4 = -0.25 / M_PI;
        for (int r = 0; r <= ctx->FDn; r++) {
            W.w[3 * r] = ctx->cx[r] * s4;
            W.w[3 * r + 1] = ctx->cy[r] * s4;
            W.w[3 * r + 2] = ctx->cz[r] * s4;
        }
        W.w0 = (ctx->cx[0] + ctx->cy[0] + ctx->cz[0]) * s4;
        // one grid row of blocks per image; images beyond 65535 go in further launches
        for (size_t i0 = 0; i0 < imgs.size(); i0 += 65535) {
            const unsigned ny = (unsigned)std::min<size_t>(65535, imgs.size() - i0);
            dim3 grid((unsigned)((maxpts + 255) / 256), ny);
            ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
            k_pseudocharge<<<grid, 256, 0, st>>>(dimg + i0, device_views(s), W, ctx->FDn,
                                                 ctx->Nx, ctx->Ny, h[0], h[1], h[2],
                                                 ref_cutoff, db, dbref, dvc, drho, dcore,
                                                 esc_acc);
        }
        if (cudaGetLastError() != cudaSuccess) rc = SGPU_ERR_CUDA;
    }
    cudaFreeAsync(dimg, st);
    if (rc != SGPU_OK) set_error("pseudocharge: CUDA error");
    return rc;
}

}  // namespace sgpu

using namespace sgpu;

extern "C" {

int sgpu_set_psd(sgpu_ctx *ctx, int ntypes, const sgpu_psd *psd)
{
    if (!ctx || ntypes < 1 || ntypes > kMaxTypes || !psd) {
        set_error("sgpu_set_psd: bad arguments (1 <= ntypes <= 8)");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    auto *s = new SetupState();
    s->types.resize(ntypes);
    for (int t = 0; t < ntypes; t++) {
        const sgpu_psd &in = psd[t];
        PsdTable &T = s->types[t];
        if (in.size < 3 || in.lmax < 0 || in.lmax > 3 || !in.ppl || !in.rc || !in.RadialGrid ||
            !in.rVloc || !in.rhoIsoAtom || !in.Gamma) {
            delete s;
            set_error("sgpu_set_psd: type " + std::to_string(t) +
                      ": missing table or unsupported size/lmax (lmax <= 3)");
            return SGPU_ERR_ARG;
        }
        T.size = in.size; T.lmax = in.lmax; T.lloc = in.lloc; T.Znucl = in.Znucl;
        T.Vloc0 = in.Vloc_0; T.fchrg = in.fchrg;
        T.ppl.assign(in.ppl, in.ppl + in.lmax + 1);
        T.rc.assign(in.rc, in.rc + in.lmax + 1);
        T.lpos.assign(in.lmax + 2, 0);
        for (int l = 0; l <= in.lmax; l++) T.lpos[l + 1] = T.lpos[l] + T.ppl[l];
        T.nrad = T.lpos[in.lmax + 1];
        T.nproj_atom = 0;
        for (int l = 0; l <= in.lmax; l++)
            if (l != in.lloc) T.nproj_atom += T.ppl[l] * (2 * l + 1);
        if (T.nrad > 0 && !in.UdV) {
            delete s;
            set_error("sgpu_set_psd: UdV is required when projectors exist");
            return SGPU_ERR_ARG;
        }
        const int n = in.size;
        T.grid.assign(in.RadialGrid, in.RadialGrid + n);
        T.rvloc.assign(in.rVloc, in.rVloc + n);
        T.rhoiso.assign(in.rhoIsoAtom, in.rhoIsoAtom + n);
        T.rhoc.assign(n, 0.0);
        if (in.rho_c_table) T.rhoc.assign(in.rho_c_table, in.rho_c_table + n);
        T.udv.assign((size_t)T.nrad * n, 0.0);
        if (T.nrad) std::memcpy(T.udv.data(), in.UdV, sizeof(double) * T.nrad * n);
        T.gamma.assign(in.Gamma, in.Gamma + T.nrad);
        T.rchrg = T.grid[n - 1];
        T.rc_max = 0.0;
        for (int l = 0; l <= in.lmax; l++) T.rc_max = std::max(T.rc_max, T.rc[l]);
        double dr0 = T.grid[1] - T.grid[0];
        T.uniform = 1;
        for (int j = 1; j < n; j++) {
            const double d = T.grid[j] - T.grid[j - 1];
            if (!(d > kTinyR)) {
                delete s;
                set_error("sgpu_set_psd: radial grid must increase");
                return SGPU_ERR_ARG;
            }
            if (std::fabs(d - dr0) > kTinyR) T.uniform = 0;
        }
        T.yd_rvloc.resize(n); T.yd_rhoiso.resize(n); T.yd_rhoc.resize(n);
        T.yd_udv.assign((size_t)T.nrad * n, 0.0);
        spline_slopes(T.grid.data(), T.rvloc.data(), T.yd_rvloc.data(), n);
        spline_slopes(T.grid.data(), T.rhoiso.data(), T.yd_rhoiso.data(), n);
        spline_slopes(T.grid.data(), T.rhoc.data(), T.yd_rhoc.data(), n);
        for (int l = 0; l <= in.lmax; l++) {
            if (l == in.lloc) continue;
            for (int k = T.lpos[l]; k < T.lpos[l + 1]; k++)
                spline_slopes(T.grid.data(), T.udv.data() + (size_t)k * n,
                              T.yd_udv.data() + (size_t)k * n, n);
        }
        // device copy: grid | rvloc | yd | rhoiso | yd | rhoc | yd | udv | yd_udv
        const size_t tot = 7 * (size_t)n + 2 * (size_t)T.nrad * n;
        std::vector<double> pack(tot);
        double *q = pack.data();
        for (const auto *v : {&T.grid, &T.rvloc, &T.yd_rvloc, &T.rhoiso, &T.yd_rhoiso, &T.rhoc,
                              &T.yd_rhoc, &T.udv, &T.yd_udv}) {
            std::memcpy(q, v->data(), sizeof(double) * v->size());
            q += v->size();
        }
        if (cudaMalloc(&T.dev, sizeof(double) * tot) != cudaSuccess ||
            cudaMemcpy(T.dev, pack.data(), sizeof(double) * tot, cudaMemcpyHostToDevice) !=
                cudaSuccess) {
            delete s;
            set_error("sgpu_set_psd: device allocation failed");
            return SGPU_ERR_CUDA;
        }
        PsdDev &v = T.view;
        v.grid = T.dev; v.rvloc = v.grid + n; v.yd_rvloc = v.rvloc + n; v.rhoiso = v.yd_rvloc + n;
        v.yd_rhoiso = v.rhoiso + n; v.rhoc = v.yd_rhoiso + n; v.yd_rhoc = v.rhoc + n;
        v.udv = v.yd_rhoc + n; v.yd_udv = v.udv + (size_t)T.nrad * n;
        v.size = n; v.uniform = T.uniform; v.Znucl = T.Znucl; v.Vloc0 = T.Vloc0;
        v.rchrg = T.rchrg;
    }
    setup_free(ctx);
    ctx->setup = s;
    return SGPU_OK;
}

int sgpu_Calculate_PseudochargeCutoff(sgpu_ctx *ctx, const double *cell, double tol,
                                      double *cutoff)
{
    if (!ctx || !cell || !cutoff || !(tol > 0)) {
        set_error("sgpu_Calculate_PseudochargeCutoff: bad arguments");
        return SGPU_ERR_ARG;
    }
    SetupState *s;
    SGPU_TRY(get_setup(ctx, &s));
    double h[3];
    grid_spacing(ctx, cell, h);
    const int FDn = ctx->FDn;
    // box half-widths (RB_MAX, src/electrostatics.c:49)
    double rbmax[3];
    int nb[3], ne[3];
    for (int d = 0; d < 3; d++) {
        rbmax[d] = h[d] < 1.5 ? h[d] * 10 + 10 : 20 * h[d] - 9.5;
        nb[d] = (int)std::ceil(rbmax[d] / h[d] - kTinyR);
        ne[d] = nb[d] + 2 * FDn;
    }
    const double *cw[3] = {ctx->cx, ctx->cy, ctx->cz};
    const double w0 = ctx->cx[0] + ctx->cy[0] + ctx->cz[0];
    const long nex = (long)ne[0] * ne[1] * ne[2];
    std::vector<double> V(nex), bq((long)nb[0] * nb[1] * nb[2]);
    for (size_t t = 0; t < s->types.size(); t++) {
        PsdTable &T = s->types[t];
        // V on the atom-centred quadrant box with FDn ghost layers (electrostatics.c:115-219)
        const PsdDev hv{T.grid.data(), T.rvloc.data(), T.yd_rvloc.data(), nullptr, nullptr,
                        nullptr, nullptr, nullptr, nullptr, T.size, T.uniform, T.Znucl,
                        T.Vloc0, T.rchrg};
        for (int k = 0; k < ne[2]; k++) {
            const double z = (k - FDn) * h[2];
            for (int j = 0; j < ne[1]; j++) {
                const double y = (j - FDn) * h[1];
                for (int i = 0; i < ne[0]; i++) {
                    const double x = (i - FDn) * h[0];
                    const double R = std::sqrt(x * x + y * y + z * z);
                    V[i + (long)ne[0] * (j + (long)ne[1] * k)] = vloc_at(hv, R);
                }
            }
        }
        // b = Lap V on the quadrant (Calc_lapV with unit scale, electrostatics.c:232)
        for (int k = 0; k < nb[2]; k++)
            for (int j = 0; j < nb[1]; j++)
                for (int i = 0; i < nb[0]; i++) {
                    auto at = [&](int a, int bb, int c) {
                        return V[(a + FDn) + (long)ne[0] * ((bb + FDn) + (long)ne[1] * (c + FDn))];
                    };
                    double res = w0 * at(i, j, k);
                    for (int r = 1; r <= FDn; r++)
                        res += (at(i - r, j, k) + at(i + r, j, k)) * cw[0][r] +
                               (at(i, j - r, k) + at(i, j + r, k)) * cw[1][r] +
                               (at(i, j, k - r) + at(i, j, k + r)) * cw[2][r];
                    bq[i + (long)nb[0] * (j + (long)nb[1] * k)] = res;
                }
        auto charge_error = [&](const double *rb) {
            int nc[3];
            for (int d = 0; d < 3; d++) nc[d] = (int)std::ceil(rb[d] / h[d] - kTinyR);
            double sum = 0.0;
            for (int k = 0; k < nc[2]; k++)
                for (int j = 0; j < nc[1]; j++)
                    for (int i = 0; i < nc[0]; i++) {
                        double v = bq[i + (long)nb[0] * (j + (long)nb[1] * k)];
                        if (k == 0) v *= 0.5;
                        if (k == nc[2] - 1) v *= 0.5;
                        if (j == 0) v *= 0.5;
                        if (j == nc[1] - 1) v *= 0.5;
                        if (i == 0) v *= 0.5;
                        if (i == nc[0] - 1) v *= 0.5;
                        sum += v;
                    }
            sum = sum / (-4 * M_PI) * 8.0 * ctx->dV;
            return std::fabs(sum + T.Znucl);
        };
        // bisection on the box radius (electrostatics.c:238-509): shrink while the integrated
        // charge stays within tol of Z, grow while it does not, per axis, at most 20 steps
        double cur[3], prev[3], lo[3], hi[3], rtol[3];
        for (int d = 0; d < 3; d++) {
            cur[d] = prev[d] = lo[d] = T.rc_max;
            hi[d] = rbmax[d];
            rtol[d] = h[d];
        }
        double err = 100, err_prev = 100;
        auto all_close = [&](const double *a, const double *b2) {
            for (int d = 0; d < 3; d++)
                if (!(std::fabs(a[d] - b2[d]) < rtol[d])) return false;
            return true;
        };
        for (int count = 0; count < 20; count++) {
            if (err < tol) {
                if (err_prev >= tol) {
                    if (all_close(cur, prev)) break;
                    err_prev = err;
                    for (int d = 0; d < 3; d++) {
                        const double t0 = cur[d];
                        hi[d] = std::min(hi[d], cur[d]);
                        if (std::fabs(cur[d] - prev[d]) >= rtol[d]) cur[d] = 0.5 * (cur[d] + prev[d]);
                        prev[d] = t0;
                    }
                } else {
                    if (all_close(cur, lo)) break;
                    err_prev = err;
                    for (int d = 0; d < 3; d++) {
                        prev[d] = cur[d];
                        hi[d] = std::min(hi[d], cur[d]);
                        if (std::fabs(cur[d] - lo[d]) >= rtol[d]) cur[d] = 0.5 * (lo[d] + cur[d]);
                    }
                }
            } else {
                if (err_prev >= tol) {
                    if (all_close(hi, cur)) {
                        for (int d = 0; d < 3; d++) cur[d] = hi[d];
                        break;
                    }
                    err_prev = err;
                    for (int d = 0; d < 3; d++) {
                        prev[d] = cur[d];
                        lo[d] = std::max(lo[d], cur[d]);
                        if (std::fabs(hi[d] - cur[d]) >= rtol[d]) cur[d] = 0.5 * (hi[d] + cur[d]);
                    }
                } else {
                    if (all_close(prev, cur)) {
                        for (int d = 0; d < 3; d++) cur[d] = prev[d];
                        break;
                    }
                    err_prev = err;
                    for (int d = 0; d < 3; d++) {
                        const double t0 = cur[d];
                        lo[d] = std::max(lo[d], cur[d]);
                        if (std::fabs(prev[d] - cur[d]) >= rtol[d]) cur[d] = 0.5 * (cur[d] + prev[d]);
                        prev[d] = t0;
                    }
                }
            }
            err = charge_error(cur);
        }
        for (int d = 0; d < 3; d++) {
            T.cutoff[d] = std::ceil(cur[d] / h[d] - kTinyR) * h[d];
            cutoff[3 * t + d] = T.cutoff[d];
        }
        T.has_cutoff = true;
    }
    return SGPU_OK;
}

int sgpu_Generate_PseudoChargeDensity(sgpu_ctx *ctx, const double *cell, const int *nAtomv,
                                      const double *atom_pos, const double *cutoff,
                                      double ref_cutoff, int net_charge, double *b,
                                      double *b_ref, double *rho_at, double *rho_core,
                                      double *scalars)
{
    if (!ctx || !cell || !nAtomv || !atom_pos || !(ref_cutoff > 0) || !b || !rho_at) {
        set_error("sgpu_Generate_PseudoChargeDensity: bad arguments");
        return SGPU_ERR_ARG;
    }
    SetupState *s;
    SGPU_TRY(get_setup(ctx, &s));
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    double h[3];
    grid_spacing(ctx, cell, h);
    // images of every atom whose rb-box meets the cell (GetInfluencingAtoms)
    std::vector<PcImage> imgs;
    long maxpts = 0;
    SGPU_TRY(pc_images(ctx, *s, cell, h, nAtomv, atom_pos, cutoff,
                       "sgpu_Generate_PseudoChargeDensity", imgs, &maxpts));
    const long Nd = ctx->Nd;
    // device buffers: b, bref, vc, rho, core, sums(4)
    double *buf = nullptr;
    SGPU_CUDA_TRY(cudaMallocAsync(&buf, sizeof(double) * (5 * Nd + 8), st));
    double *db = buf, *dbref = buf + Nd, *dvc = buf + 2 * Nd, *drho = buf + 3 * Nd,
           *dcore = buf + 4 * Nd, *sums = buf + 5 * Nd;
    int rc = SGPU_OK;
    do {
        if (cudaMemsetAsync(buf, 0, sizeof(double) * (5 * Nd + 8), st) != cudaSuccess) {
            rc = SGPU_ERR_CUDA; break;
        }
        if ((rc = pseudocharge_fields(ctx, *s, h, imgs, maxpts, ref_cutoff, db, dbref, dvc,
                                      drho, dcore, sums + 3, st)) != SGPU_OK)
            break;
        {
            ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
            k_charge_sums<<<2 * 152, 256, 0, st>>>(db, dbref, dvc, drho, Nd, sums);
        }
        if (cudaGetLastError() != cudaSuccess) { rc = SGPU_ERR_CUDA; break; }
        double hs[4];
        if (cudaMemcpyAsync(hs, sums, sizeof(hs), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            rc = SGPU_ERR_CUDA; break;
        }
        const double dV = ctx->dV;
        const double pos_charge = -hs[0] * dV, neg_charge0 = -hs[1] * dV;
        const double esc = (hs[2] + hs[3]) * dV * 0.5;
        // scale the superposition so that PosCharge + NegCharge = NetCharge (:1111-1125)
        const double scal = (net_charge - pos_charge) / neg_charge0;
        k_scale<<<2 * 152, 256, 0, st>>>(drho, Nd, scal);
        double neg_charge = -(hs[1] * scal) * dV;
        if (scalars) {
            scalars[0] = esc;
            scalars[1] = pos_charge;
            scalars[2] = neg_charge;
        }
        if ((rc = deliver(db, b, Nd, st)) != SGPU_OK) break;
        if ((rc = deliver(dbref, b_ref, Nd, st)) != SGPU_OK) break;
        if ((rc = deliver(drho, rho_at, Nd, st)) != SGPU_OK) break;
        if ((rc = deliver(dcore, rho_core, Nd, st)) != SGPU_OK) break;
    } while (0);
    if (rc != SGPU_OK && rc == SGPU_ERR_CUDA) set_error("sgpu_Generate_PseudoChargeDensity: CUDA error");
    cudaFreeAsync(buf, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == SGPU_OK) {
        set_error("sgpu_Generate_PseudoChargeDensity: CUDA error");
        rc = SGPU_ERR_CUDA;
    }
    return rc;
}

int sgpu_Generate_InitialMagnetization(sgpu_ctx *ctx, const double *cell, const int *nAtomv,
                                       const double *atom_pos, const double *cutoff,
                                       const double *atom_spin_z, double *mag_at)
{
    if (!ctx || !cell || !nAtomv || !atom_pos || !atom_spin_z || !mag_at) {
        set_error("sgpu_Generate_InitialMagnetization: bad arguments");
        return SGPU_ERR_ARG;
    }
    SetupState *s;
    SGPU_TRY(get_setup(ctx, &s));
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    double h[3];
    grid_spacing(ctx, cell, h);
    std::vector<PcImage> imgs;
    long maxpts = 0;
    SGPU_TRY(pc_images(ctx, *s, cell, h, nAtomv, atom_pos, cutoff,
                       "sgpu_Generate_InitialMagnetization", imgs, &maxpts));
    int n_atom = 0;
    for (size_t t = 0; t < s->types.size(); t++) n_atom += nAtomv[t];
    std::vector<double> w(n_atom);
    for (size_t t = 0, a = 0; t < s->types.size(); t++)
        for (int i = 0; i < nAtomv[t]; i++, a++) w[a] = atom_spin_z[a] / (double)s->types[t].Znucl;
    const long Nd = ctx->Nd;
    double *buf = nullptr;
    SGPU_CUDA_TRY(cudaMallocAsync(&buf, sizeof(double) * (Nd + n_atom + 1), st));
    PcImage *dimg = nullptr;
    int rc = SGPU_OK;
    do {
        if (cudaMemsetAsync(buf, 0, sizeof(double) * Nd, st) != cudaSuccess ||
            cudaMemcpyAsync(buf + Nd, w.data(), sizeof(double) * n_atom, cudaMemcpyHostToDevice,
                            st) != cudaSuccess) {
            rc = SGPU_ERR_CUDA; break;
        }
        if (!imgs.empty()) {
            if (cudaMallocAsync(&dimg, sizeof(PcImage) * imgs.size(), st) != cudaSuccess ||
                cudaMemcpyAsync(dimg, imgs.data(), sizeof(PcImage) * imgs.size(),
                                cudaMemcpyHostToDevice, st) != cudaSuccess) {
                rc = SGPU_ERR_CUDA; break;
            }
            for (size_t i0 = 0; i0 < imgs.size(); i0 += 65535) {
                const unsigned ny = (unsigned)std::min<size_t>(65535, imgs.size() - i0);
                dim3 grid((unsigned)((maxpts + 255) / 256), ny);
                ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
                k_mag_at<<<grid, 256, 0, st>>>(dimg + i0, device_views(*s), ctx->FDn, ctx->Nx,
                                               ctx->Ny, h[0], h[1], h[2], buf + Nd, buf);
            }
            if (cudaGetLastError() != cudaSuccess) { rc = SGPU_ERR_CUDA; break; }
        }
        rc = deliver(buf, mag_at, Nd, st);
    } while (0);
    if (rc == SGPU_ERR_CUDA) set_error("sgpu_Generate_InitialMagnetization: CUDA error");
    if (dimg) cudaFreeAsync(dimg, st);
    cudaFreeAsync(buf, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == SGPU_OK) {
        set_error("sgpu_Generate_InitialMagnetization: CUDA error");
        rc = SGPU_ERR_CUDA;
    }
    return rc;
}

// shared by the force entry points: the images of the atoms' rb-boxes on the device
struct ForceImages {
    std::vector<PcImage> imgs;
    long maxpts = 0;
    int n_atom = 0;
    double h[3];
};

static int force_images(sgpu_ctx *ctx, SetupState *s, const double *cell, const int *nAtomv,
                        const double *atom_pos, const double *cutoff, const char *who,
                        ForceImages *fi)
{
    grid_spacing(ctx, cell, fi->h);
    fi->n_atom = 0;
    for (size_t t = 0; t < s->types.size(); t++) fi->n_atom += nAtomv[t];
    return pc_images(ctx, *s, cell, fi->h, nAtomv, atom_pos, cutoff, who, fi->imgs, &fi->maxpts);
}

static D1Weights d1_weights(const sgpu_ctx *ctx, const double h[3])
{
    D1Weights G{};
    for (int r = 1; r <= ctx->FDn; r++) {  // w1[r] = w2[r] r / 2, so D1 = D2 * h * r / 2
        G.d[3 * r] = ctx->cx[r] * h[0] * r * 0.5;
        G.d[3 * r + 1] = ctx->cy[r] * h[1] * r * 0.5;
        G.d[3 * r + 2] = ctx->cz[r] * h[2] * r * 0.5;
    }
    return G;
}

int sgpu_Calculate_local_forces(sgpu_ctx *ctx, const double *cell, const int *nAtomv,
                                const double *atom_pos, const double *cutoff, double ref_cutoff,
                                const double *phi, double *forces)
{
    if (!ctx || !cell || !nAtomv || !atom_pos || !(ref_cutoff > 0) || !phi || !forces) {
        set_error("sgpu_Calculate_local_forces: bad arguments");
        return SGPU_ERR_ARG;
    }
    SetupState *s;
    SGPU_TRY(get_setup(ctx, &s));
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    ForceImages fi;
    SGPU_TRY(force_images(ctx, s, cell, nAtomv, atom_pos, cutoff, "sgpu_Calculate_local_forces",
                          &fi));
    const long Nd = ctx->Nd;
    // b, bref, vc, rho, core, esc sums (8), grad phi (3 Nd), grad Vc (3 Nd), phi, forces
    const size_t nbuf = 5 * Nd + 8 + 6 * Nd + Nd + 3 * (size_t)fi.n_atom;
    double *buf = nullptr;
    SGPU_CUDA_TRY(cudaMallocAsync(&buf, sizeof(double) * nbuf, st));
    double *db = buf, *dbref = buf + Nd, *dvc = buf + 2 * Nd, *drho = buf + 3 * Nd,
           *dcore = buf + 4 * Nd, *sums = buf + 5 * Nd, *gphi = sums + 8, *gvc = gphi + 3 * Nd,
           *dphi = gvc + 3 * Nd, *dF = dphi + Nd;
    PcImage *dimg = nullptr;
    int rc = SGPU_OK;
    do {
        if (cudaMemsetAsync(buf, 0, sizeof(double) * nbuf, st) != cudaSuccess ||
            cudaMemcpyAsync(dphi, phi, sizeof(double) * Nd, cudaMemcpyDefault, st) != cudaSuccess) {
            rc = SGPU_ERR_CUDA; break;
        }
        if ((rc = pseudocharge_fields(ctx, *s, fi.h, fi.imgs, fi.maxpts, ref_cutoff, db, dbref,
                                      dvc, drho, dcore, sums, st)) != SGPU_OK)
            break;
        const D1Weights G = d1_weights(ctx, fi.h);
        for (int d = 0; d < 3 && rc == SGPU_OK; d++) {
            double w[kMaxFDn + 1];
            for (int r = 0; r <= ctx->FDn; r++) w[r] = G.d[3 * r + d];
            rc = launch_gradient(ctx, 1, dphi, Nd, gphi + d * Nd, Nd, d, w, st);
            if (rc == SGPU_OK) rc = launch_gradient(ctx, 1, dvc, Nd, gvc + d * Nd, Nd, d, w, st);
        }
        if (rc != SGPU_OK) break;
        if (!fi.imgs.empty()) {
            if (cudaMallocAsync(&dimg, sizeof(PcImage) * fi.imgs.size(), st) != cudaSuccess ||
                cudaMemcpyAsync(dimg, fi.imgs.data(), sizeof(PcImage) * fi.imgs.size(),
                                cudaMemcpyHostToDevice, st) != cudaSuccess) {
                rc = SGPU_ERR_CUDA; break;
            }
            PcWeights W{};
            const double s4 = -0.25 / M_PI;
            for (int r = 0; r <= ctx->FDn; r++) {
                W.w[3 * r] = ctx->cx[r] * s4;
                W.w[3 * r + 1] = ctx->cy[r] * s4;
                W.w[3 * r + 2] = ctx->cz[r] * s4;
            }
            W.w0 = (ctx->cx[0] + ctx->cy[0] + ctx->cz[0]) * s4;
            for (size_t i0 = 0; i0 < fi.imgs.size(); i0 += 65535) {
                const unsigned ny = (unsigned)std::min<size_t>(65535, fi.imgs.size() - i0);
                dim3 grid((unsigned)((fi.maxpts + 255) / 256), ny);
                ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
                k_local_forces<<<grid, 256, 0, st>>>(dimg + i0, device_views(*s), W, G, ctx->FDn,
                                                     ctx->Nx, ctx->Ny, fi.h[0], fi.h[1], fi.h[2],
                                                     ref_cutoff, db, dbref, gphi, gvc, Nd,
                                                     ctx->dV, dF);
            }
            if (cudaGetLastError() != cudaSuccess) { rc = SGPU_ERR_CUDA; break; }
        }
        if (cudaMemcpyAsync(forces, dF, sizeof(double) * 3 * fi.n_atom, cudaMemcpyDefault,
                            st) != cudaSuccess)
            rc = SGPU_ERR_CUDA;
    } while (0);
    if (dimg) cudaFreeAsync(dimg, st);
    cudaFreeAsync(buf, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == SGPU_OK) rc = SGPU_ERR_CUDA;
    if (rc == SGPU_ERR_CUDA) set_error("sgpu_Calculate_local_forces: CUDA error");
    return rc;
}

int sgpu_Calculate_forces_xc(sgpu_ctx *ctx, const double *cell, const int *nAtomv,
                             const double *atom_pos, const double *cutoff, const double *Vxc,
                             double *forces_xc)
{
    if (!ctx || !cell || !nAtomv || !atom_pos || !Vxc || !forces_xc) {
        set_error("sgpu_Calculate_forces_xc: bad arguments");
        return SGPU_ERR_ARG;
    }
    SetupState *s;
    SGPU_TRY(get_setup(ctx, &s));
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    ForceImages fi;
    SGPU_TRY(force_images(ctx, s, cell, nAtomv, atom_pos, cutoff, "sgpu_Calculate_forces_xc",
                          &fi));
    const long Nd = ctx->Nd;
    double *buf = nullptr;
    const size_t nbuf = Nd + 3 * (size_t)fi.n_atom;
    SGPU_CUDA_TRY(cudaMallocAsync(&buf, sizeof(double) * nbuf, st));
    double *dvxc = buf, *dF = buf + Nd;
    PcImage *dimg = nullptr;
    int rc = SGPU_OK;
    do {
        if (cudaMemsetAsync(dF, 0, sizeof(double) * 3 * fi.n_atom, st) != cudaSuccess ||
            cudaMemcpyAsync(dvxc, Vxc, sizeof(double) * Nd, cudaMemcpyDefault, st) != cudaSuccess) {
            rc = SGPU_ERR_CUDA; break;
        }
        if (!fi.imgs.empty()) {
            if (cudaMallocAsync(&dimg, sizeof(PcImage) * fi.imgs.size(), st) != cudaSuccess ||
                cudaMemcpyAsync(dimg, fi.imgs.data(), sizeof(PcImage) * fi.imgs.size(),
                                cudaMemcpyHostToDevice, st) != cudaSuccess) {
                rc = SGPU_ERR_CUDA; break;
            }
            const D1Weights G = d1_weights(ctx, fi.h);
            for (size_t i0 = 0; i0 < fi.imgs.size(); i0 += 65535) {
                const unsigned ny = (unsigned)std::min<size_t>(65535, fi.imgs.size() - i0);
                dim3 grid((unsigned)((fi.maxpts + 255) / 256), ny);
                ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
                k_xc_forces<<<grid, 256, 0, st>>>(dimg + i0, device_views(*s), G, ctx->FDn, ctx->Nx,
                                                  ctx->Ny, fi.h[0], fi.h[1], fi.h[2], dvxc,
                                                  ctx->dV, dF);
            }
            if (cudaGetLastError() != cudaSuccess) { rc = SGPU_ERR_CUDA; break; }
        }
        if (cudaMemcpyAsync(forces_xc, dF, sizeof(double) * 3 * fi.n_atom, cudaMemcpyDefault,
                            st) != cudaSuccess)
            rc = SGPU_ERR_CUDA;
    } while (0);
    if (dimg) cudaFreeAsync(dimg, st);
    cudaFreeAsync(buf, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && rc == SGPU_OK) rc = SGPU_ERR_CUDA;
    if (rc == SGPU_ERR_CUDA) set_error("sgpu_Calculate_forces_xc: CUDA error");
    return rc;
}

int sgpu_CalculateNonlocalProjectors(sgpu_ctx *ctx, const double *cell, const int *nAtomv,
                                     const double *atom_pos)
{
    if (!ctx || !cell || !nAtomv || !atom_pos) {
        set_error("sgpu_CalculateNonlocalProjectors: bad arguments");
        return SGPU_ERR_ARG;
    }
    SetupState *s;
    SGPU_TRY(get_setup(ctx, &s));
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    double h[3];
    grid_spacing(ctx, cell, h);
    const int N[3] = {ctx->Nx, ctx->Ny, ctx->Nz};
    // atoms and their projector offsets (IP_displ), type-major as the reference orders atoms
    int n_atom = 0;
    for (size_t t = 0; t < s->types.size(); t++) n_atom += nAtomv[t];
    std::vector<int> ip_displ(n_atom + 1, 0), atom_type(n_atom);
    {
        int a = 0;
        for (size_t t = 0; t < s->types.size(); t++)
            for (int i = 0; i < nAtomv[t]; i++, a++) {
                atom_type[a] = (int)t;
                ip_displ[a + 1] = ip_displ[a] + s->types[t].nproj_atom;
            }
    }
    std::vector<double> gamma(ip_displ[n_atom]);
    for (int a = 0; a < n_atom; a++) {
        const PsdTable &T = s->types[atom_type[a]];
        int col = ip_displ[a];
        for (int l = 0; l <= T.lmax; l++) {
            if (l == T.lloc) continue;
            for (int np = 0; np < T.ppl[l]; np++)
                for (int m = -l; m <= l; m++) gamma[col++] = T.gamma[T.lpos[l] + np];
        }
    }
    // images whose rc-sphere holds grid points (GetInfluencingAtoms_nloc): the sphere is
    // r^2 <= rc^2 with r^2 formed as the square of the distance, as the reference does
    std::vector<NlImage> imgs;
    std::vector<int> img_atom, img_ndc, grid_pos;
    std::vector<double> img_coords;
    long nchi = 0;
    int maxndc = 0;
    for (int a = 0; a < n_atom; a++) {
        const PsdTable &T = s->types[atom_type[a]];
        if (T.nproj_atom == 0) continue;
        const double rc = T.rc_max, rc2 = rc * rc;
        const double *p0 = atom_pos + 3 * a;
        int lo[3], hi[3];
        for (int d = 0; d < 3; d++) image_range(p0[d], cell[d], rc, &lo[d], &hi[d]);
        for (int rr = lo[2]; rr <= hi[2]; rr++) {
            const double z0 = p0[2] + cell[2] * rr;
            if (z0 < -rc || z0 >= (N[2] - 1) * h[2] + rc) continue;
            for (int qq = lo[1]; qq <= hi[1]; qq++) {
                const double y0 = p0[1] + cell[1] * qq;
                if (y0 < -rc || y0 >= (N[1] - 1) * h[1] + rc) continue;
                for (int pp = lo[0]; pp <= hi[0]; pp++) {
                    const double x0 = p0[0] + cell[0] * pp;
                    if (x0 < -rc || x0 >= (N[0] - 1) * h[0] + rc) continue;
                    const double c[3] = {x0, y0, z0};
                    int s0[3], e0[3];
                    for (int d = 0; d < 3; d++) {
                        s0[d] = std::max(0, (int)std::ceil((c[d] - rc) / h[d]));
                        e0[d] = std::min(N[d] - 1, (int)std::floor((c[d] + rc) / h[d]));
                    }
                    const long first = (long)grid_pos.size();
                    for (int k = s0[2]; k <= e0[2]; k++) {
                        const double dz = k * h[2] - z0;
                        for (int j = s0[1]; j <= e0[1]; j++) {
                            const double dy = j * h[1] - y0;
                            for (int i = s0[0]; i <= e0[0]; i++) {
                                const double dx = i * h[0] - x0;
                                double r = std::sqrt(dx * dx + dy * dy + dz * dz);
                                r *= r;
                                if (r <= rc2)
                                    grid_pos.push_back(i + N[0] * (j + N[1] * k));
                            }
                        }
                    }
                    const int ndc = (int)((long)grid_pos.size() - first);
                    if (ndc == 0) continue;
                    imgs.push_back(NlImage{x0, y0, z0, first, nchi, ndc, atom_type[a]});
                    img_atom.push_back(a);
                    img_ndc.push_back(ndc);
                    img_coords.insert(img_coords.end(), {x0, y0, z0});
                    nchi += (long)ndc * T.nproj_atom;
                    maxndc = std::max(maxndc, ndc);
                }
            }
        }
    }
    std::vector<double> chi(nchi);
    if (nchi > 0) {
        NlTypeSet TS{};
        for (size_t t = 0; t < s->types.size(); t++) {
            const PsdTable &T = s->types[t];
            TS.t[t].lmax = T.lmax; TS.t[t].lloc = T.lloc; TS.t[t].nproj = T.nproj_atom;
            for (int l = 0; l <= T.lmax; l++) { TS.t[t].ppl[l] = T.ppl[l]; TS.t[t].lpos[l] = T.lpos[l]; }
        }
        NlImage *dimg = nullptr;
        int *dpos = nullptr;
        double *dchi = nullptr;
        int rc = SGPU_OK;
        if (cudaMallocAsync(&dimg, sizeof(NlImage) * imgs.size(), st) != cudaSuccess ||
            cudaMallocAsync(&dpos, sizeof(int) * grid_pos.size(), st) != cudaSuccess ||
            cudaMallocAsync(&dchi, sizeof(double) * nchi, st) != cudaSuccess ||
            cudaMemcpyAsync(dimg, imgs.data(), sizeof(NlImage) * imgs.size(),
                            cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaMemcpyAsync(dpos, grid_pos.data(), sizeof(int) * grid_pos.size(),
                            cudaMemcpyHostToDevice, st) != cudaSuccess) {
            rc = SGPU_ERR_CUDA;
        } else {
            for (size_t i0 = 0; i0 < imgs.size(); i0 += 65535) {
                const unsigned ny = (unsigned)std::min<size_t>(65535, imgs.size() - i0);
                ProfScope ps(ctx, SGPU_KERNEL_OTHER, st);
                k_projectors<<<dim3((maxndc + 127) / 128, ny), 128, 0, st>>>(
                    dimg + i0, dpos, device_views(*s), TS, ctx->Nx, ctx->Ny, h[0], h[1], h[2],
                    dchi);
            }
            if (cudaGetLastError() != cudaSuccess ||
                cudaMemcpyAsync(chi.data(), dchi, sizeof(double) * nchi, cudaMemcpyDeviceToHost,
                                st) != cudaSuccess)
                rc = SGPU_ERR_CUDA;
        }
        if (dimg) cudaFreeAsync(dimg, st);
        if (dpos) cudaFreeAsync(dpos, st);
        if (dchi) cudaFreeAsync(dchi, st);
        if (cudaStreamSynchronize(st) != cudaSuccess) rc = SGPU_ERR_CUDA;
        if (rc != SGPU_OK) {
            set_error("sgpu_CalculateNonlocalProjectors: CUDA error");
            return rc;
        }
    }
    SGPU_TRY(sgpu_set_nonlocal(ctx, n_atom, ip_displ.data(), gamma.data(), (int)imgs.size(),
                               img_atom.data(), img_ndc.data(), grid_pos.data(), chi.data()));
    SGPU_TRY(sgpu_set_kpoint_geometry(ctx, cell[0], cell[1], cell[2], (int)imgs.size(),
                                      img_coords.empty() ? nullptr : img_coords.data()));
    return SGPU_OK;
}

}  // extern "C"
