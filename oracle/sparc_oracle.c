/*
 * CPU oracle: a plain-C restatement of the reference SPARC CheFSI hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker the GPU library is compared against
 * (and the "port" CPU baseline timed beside it). It is never linked into, called by, or used
 * as a fallback for the GPU library.
 *
 * Each function cites the reference function it restates. Layouts follow the reference:
 * orbital blocks are column-major with leading dimension ld >= Nd, grid index
 * i + j*Nx + k*Nx*Ny (x fastest), periodic boundaries in all three directions.
 *
 * Parity of this restatement is pinned against the reference program itself (built from the
 * reference sources by oracle/ref/Makefile) through the fixtures in tests/golden/.
 */
#include "sparc_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ FD weights */

/* fract(n,k) = n!^2 / ((n-k)! (n+k)!), src/tools.c:725 */
static double orc_fract(int n, int k)
{
    double Nr = 1.0, Dr = 1.0;
    for (int i = n - k + 1; i <= n; i++) Nr *= i;
    for (int i = n + 1; i <= n + k; i++) Dr *= i;
    return Nr / Dr;
}

/* Second-derivative central FD weights of half-order FDn divided by h^2:
 * w[0] = -2 sum_p 1/p^2, w[p] = 2 (-1)^(p+1) fract(FDn,p) / p^2
 * (src/initialization.c:2112-2121 FDweights_D2, :2141-2146 division by delta^2). */
void orc_fd_d2_weights(int FDn, double h, double *w)
{
    double w0 = 0.0;
    for (int p = 1; p <= FDn; p++) {
        w0 -= 2.0 / ((double)p * p);
        w[p] = 2.0 * ((p + 1) % 2 ? -1.0 : 1.0) * orc_fract(FDn, p) / ((double)p * p);
    }
    w[0] = w0;
    for (int p = 0; p <= FDn; p++) w[p] /= (h * h);
}

static inline int wrap(int i, int n)
{
    i %= n;
    return i < 0 ? i + n : i;
}

/* ------------------------------------------------------------------- stencil */

/* y = (a*Lap + b*diag(v) + c*I) x for ncol columns, periodic, orthogonal grid.
 * Restates Lap_plus_diag_vec_mult_orth (src/lapVecRoutines.c:306-611): coefficients are
 * pre-scaled by a (:358-373), the centre weight is a*(wx0+wy0+wz0)+c (:375-379), and the
 * per-point sum follows stencil_3axis_thread_radius6 (:185-227): res = c0*x, then for each
 * r, res += (x-r + x+r)*wx_r + (y-r + y+r)*wy_r + (z-r + z+r)*wz_r, and y = res + b*(v*x).
 * When v is NULL or |b| < 1e-14 the diagonal term is dropped (:334). */
void orc_lap_plus_diag_orth(int Nx, int Ny, int Nz, int FDn, const double *cx, const double *cy,
                            const double *cz, int ncol, double a, double b, double c,
                            const double *v, const double *x, long ldi, double *y, long ldo)
{
    double wx[ORC_MAX_FDN + 1], wy[ORC_MAX_FDN + 1], wz[ORC_MAX_FDN + 1];
    for (int p = 0; p <= FDn; p++) { wx[p] = cx[p] * a; wy[p] = cy[p] * a; wz[p] = cz[p] * a; }
    const double c0 = wx[0] + wy[0] + wz[0] + c;
    const int use_v = !(fabs(b) < 1e-14 || v == NULL);
    const long NxNy = (long)Nx * Ny;
#pragma omp parallel for collapse(2) schedule(static)
    for (int n = 0; n < ncol; n++) {
        for (int k = 0; k < Nz; k++) {
            const double *xn = x + (long)n * ldi;
            double *yn = y + (long)n * ldo;
            for (int j = 0; j < Ny; j++) {
                for (int i = 0; i < Nx; i++) {
                    long idx = i + (long)j * Nx + (long)k * NxNy;
                    double res = c0 * xn[idx];
                    for (int r = 1; r <= FDn; r++) {
                        double rx = (xn[wrap(i - r, Nx) + (long)j * Nx + (long)k * NxNy] +
                                     xn[wrap(i + r, Nx) + (long)j * Nx + (long)k * NxNy]) * wx[r];
                        double ry = (xn[i + (long)wrap(j - r, Ny) * Nx + (long)k * NxNy] +
                                     xn[i + (long)wrap(j + r, Ny) * Nx + (long)k * NxNy]) * wy[r];
                        double rz = (xn[i + (long)j * Nx + (long)wrap(k - r, Nz) * NxNy] +
                                     xn[i + (long)j * Nx + (long)wrap(k + r, Nz) * NxNy]) * wz[r];
                        res += rx + ry + rz;
                    }
                    yn[idx] = use_v ? res + b * (v[idx] * xn[idx]) : res;
                }
            }
        }
    }
}

/* ------------------------------------------------------------------ nonlocal */

/* Hx += Vnl x with Kleinman-Bylander projectors. Restates Vnl_vec_mult
 * (src/nlocVecRoutines.c:798-886): alpha_a = dV * sum over images of atom a of
 * Chi_imgᵀ x[grid_pos_img] (:803-833), alpha_a[j,n] *= Gamma_a[j] (:843-866), then
 * Hx[grid_pos_img] += Chi_img alpha_a (:869-884). Gamma is given expanded per projector
 * column (the reference's l, np, m ordering). */
void orc_vnl_vec_mult(const orc_nonlocal *nl, double dV, int ncol, const double *x, long ldi,
                      double *Hx, long ldo)
{
    const int ntot = nl->ip_displ[nl->natom];
    double *alpha = (double *)calloc((size_t)ntot * (ncol > 0 ? ncol : 1), sizeof(double));
    /* alpha layout as the reference: block of atom a starts at ip_displ[a]*ncol, nproj x ncol */
#pragma omp parallel for schedule(static)
    for (int n = 0; n < ncol; n++) {
        for (int g = 0; g < nl->nimg; g++) {
            const int a = nl->img_atom[g];
            const int np = nl->ip_displ[a + 1] - nl->ip_displ[a];
            const int ndc = nl->img_ndc[g];
            const int *gp = nl->grid_pos + nl->img_off[g];
            const double *chi = nl->chi + nl->img_chi_off[g];
            double *al = alpha + (long)nl->ip_displ[a] * ncol + (long)n * np;
            for (int j = 0; j < np; j++) {
                double s = 0.0;
                for (int i = 0; i < ndc; i++) s += chi[(long)j * ndc + i] * x[(long)n * ldi + gp[i]];
                al[j] += dV * s;
            }
        }
    }
    for (int a = 0; a < nl->natom; a++) {
        const int np = nl->ip_displ[a + 1] - nl->ip_displ[a];
        for (int n = 0; n < ncol; n++)
            for (int j = 0; j < np; j++)
                alpha[(long)nl->ip_displ[a] * ncol + (long)n * np + j] *= nl->gamma[nl->ip_displ[a] + j];
    }
#pragma omp parallel for schedule(static)
    for (int n = 0; n < ncol; n++) {
        for (int g = 0; g < nl->nimg; g++) {
            const int a = nl->img_atom[g];
            const int np = nl->ip_displ[a + 1] - nl->ip_displ[a];
            const int ndc = nl->img_ndc[g];
            const int *gp = nl->grid_pos + nl->img_off[g];
            const double *chi = nl->chi + nl->img_chi_off[g];
            const double *al = alpha + (long)nl->ip_displ[a] * ncol + (long)n * np;
            for (int i = 0; i < ndc; i++) {
                double s = 0.0;
                for (int j = 0; j < np; j++) s += chi[(long)j * ndc + i] * al[j];
                Hx[(long)n * ldo + gp[i]] += s;
            }
        }
    }
    free(alpha);
}

/* Hx = (-0.5 Lap + Veff + c) x + Vnl x. Restates Hamiltonian_vectors_mult for an orthogonal
 * cell with no exact exchange, meta-GGA or Hubbard terms (src/hamiltonianVecRoutines.c:45-121). */
void orc_hamiltonian(const orc_grid *gr, const orc_nonlocal *nl, const double *veff, int ncol,
                     double c, const double *x, long ldi, double *Hx, long ldo)
{
    orc_lap_plus_diag_orth(gr->Nx, gr->Ny, gr->Nz, gr->FDn, gr->cx, gr->cy, gr->cz, ncol, -0.5,
                           1.0, c, veff, x, ldi, Hx, ldo);
    if (nl && nl->nimg > 0) orc_vnl_vec_mult(nl, gr->dV, ncol, x, ldi, Hx, ldo);
}

/* Chebyshev filter of degree m on [a, b] with lower bound a0. Restates ChebyshevFiltering
 * (src/eigenSolver.c:722-798) including its side effects: on return Y holds the filtered
 * block and X holds the degree m-1 iterate. */
void orc_chebyshev_filter(const orc_grid *gr, const orc_nonlocal *nl, const double *veff,
                          double *X, long ldi, double *Y, long ldo, int ncol, int m, double a,
                          double b, double a0)
{
    const long Nd = (long)gr->Nx * gr->Ny * gr->Nz;
    const double e = 0.5 * (b - a);
    const double c = 0.5 * (b + a);
    double sigma = e / (a0 - c);
    const double sigma1 = sigma;
    const double gamma = 2.0 / sigma1;

    orc_hamiltonian(gr, nl, veff, ncol, -c, X, ldi, Y, ldo);
    double vscal = sigma1 / e;
    for (int n = 0; n < ncol; n++)
        for (long i = 0; i < Nd; i++) Y[i + n * ldo] *= vscal;

    double *Ynew = (double *)malloc(sizeof(double) * Nd * (ncol > 0 ? ncol : 1));
    for (int j = 1; j < m; j++) {
        double sigma2 = 1.0 / (gamma - sigma);
        orc_hamiltonian(gr, nl, veff, ncol, -c, Y, ldo, Ynew, Nd);
        vscal = 2.0 * sigma2 / e;
        double vscal2 = sigma * sigma2;
#pragma omp parallel for schedule(static)
        for (int n = 0; n < ncol; n++) {
            for (long i = 0; i < Nd; i++) {
                Ynew[i + n * Nd] *= vscal;
                Ynew[i + n * Nd] -= vscal2 * X[i + n * ldi];
                X[i + n * ldi] = Y[i + n * ldo];
                Y[i + n * ldo] = Ynew[i + n * Nd];
            }
        }
        sigma = sigma2;
    }
    free(Ynew);
}

/* r = b + (Lap + c) x, restating poisson_residual (src/lapVecRoutines.c:69-79). */
void orc_poisson_residual(const orc_grid *gr, double c, const double *x, const double *b,
                          double *r)
{
    const long Nd = (long)gr->Nx * gr->Ny * gr->Nz;
    orc_lap_plus_diag_orth(gr->Nx, gr->Ny, gr->Nz, gr->FDn, gr->cx, gr->cy, gr->cz, 1, 1.0, 0.0,
                           c, NULL, x, Nd, r, Nd);
    for (long i = 0; i < Nd; i++) r[i] += b[i];
}

/* ------------------------------------------------------------- k-point twins */

/* Bloch factor of a neighbour at raw index i (may lie outside [0, n)): ghost points left of
 * the cell carry e^{-i k L}, right of it e^{+i k L}, as the ghost copies of
 * Lap_plus_diag_vec_mult_orth_kpt (src/lapVecRoutinesKpt.c:370-382, :452-460). */
static inline double complex bloch(int i, int n, double kL)
{
    if (i < 0) return cexp(-I * kL);
    if (i >= n) return cexp(I * kL);
    return 1.0;
}

/* y = (a*Lap + b*diag(v) + c*I) x for complex Bloch columns at k = (kx, ky, kz), periodic
 * cell of lengths L. Restates Lap_plus_diag_vec_mult_orth_kpt (src/lapVecRoutinesKpt.c:179)
 * with the same per-point sum order as the real stencil. */
void orc_lap_plus_diag_orth_kpt(int Nx, int Ny, int Nz, int FDn, const double *cx,
                                const double *cy, const double *cz, const double *k,
                                const double *L, int ncol, double a, double b, double c,
                                const double *v, const double complex *x, long ldi,
                                double complex *y, long ldo)
{
    double wx[ORC_MAX_FDN + 1], wy[ORC_MAX_FDN + 1], wz[ORC_MAX_FDN + 1];
    for (int p = 0; p <= FDn; p++) { wx[p] = cx[p] * a; wy[p] = cy[p] * a; wz[p] = cz[p] * a; }
    const double c0 = wx[0] + wy[0] + wz[0] + c;
    const int use_v = !(fabs(b) < 1e-14 || v == NULL);
    const long NxNy = (long)Nx * Ny;
    const double kLx = k[0] * L[0], kLy = k[1] * L[1], kLz = k[2] * L[2];
#pragma omp parallel for collapse(2) schedule(static)
    for (int n = 0; n < ncol; n++) {
        for (int kk = 0; kk < Nz; kk++) {
            const double complex *xn = x + (long)n * ldi;
            double complex *yn = y + (long)n * ldo;
            for (int j = 0; j < Ny; j++) {
                for (int i = 0; i < Nx; i++) {
                    long idx = i + (long)j * Nx + (long)kk * NxNy;
                    double complex res = c0 * xn[idx];
                    for (int r = 1; r <= FDn; r++) {
                        double complex rx =
                            (xn[wrap(i - r, Nx) + (long)j * Nx + (long)kk * NxNy] * bloch(i - r, Nx, kLx) +
                             xn[wrap(i + r, Nx) + (long)j * Nx + (long)kk * NxNy] * bloch(i + r, Nx, kLx)) * wx[r];
                        double complex ry =
                            (xn[i + (long)wrap(j - r, Ny) * Nx + (long)kk * NxNy] * bloch(j - r, Ny, kLy) +
                             xn[i + (long)wrap(j + r, Ny) * Nx + (long)kk * NxNy] * bloch(j + r, Ny, kLy)) * wy[r];
                        double complex rz =
                            (xn[i + (long)j * Nx + (long)wrap(kk - r, Nz) * NxNy] * bloch(kk - r, Nz, kLz) +
                             xn[i + (long)j * Nx + (long)wrap(kk + r, Nz) * NxNy] * bloch(kk + r, Nz, kLz)) * wz[r];
                        res += rx + ry + rz;
                    }
                    yn[idx] = use_v ? res + b * (v[idx] * xn[idx]) : res;
                }
            }
        }
    }
}

/* Hx += Vnl x with Bloch factors per atom image: alpha_a += e^{i theta_g} dV Chi_gᵀ x[gp_g],
 * alpha *= Gamma, Hx[gp_g] += e^{-i theta_g} Chi_g alpha_a, theta_g = -k . (floor(c_g / L) L)
 * for image coordinates c_g. Restates Vnl_vec_mult_kpt (src/nlocVecRoutines.c:889-999). */
void orc_vnl_vec_mult_kpt(const orc_nonlocal *nl, const double *img_coords, const double *k,
                          const double *L, double dV, int ncol, const double complex *x,
                          long ldi, double complex *Hx, long ldo)
{
    const int ntot = nl->ip_displ[nl->natom];
    double complex *alpha = (double complex *)calloc((size_t)ntot * (ncol > 0 ? ncol : 1),
                                                     sizeof(double complex));
    double *theta = (double *)malloc(sizeof(double) * (nl->nimg > 0 ? nl->nimg : 1));
    for (int g = 0; g < nl->nimg; g++) {
        const double *cg = img_coords + 3 * g;
        theta[g] = -k[0] * (floor(cg[0] / L[0]) * L[0]) - k[1] * (floor(cg[1] / L[1]) * L[1]) -
                   k[2] * (floor(cg[2] / L[2]) * L[2]);
    }
#pragma omp parallel for schedule(static)
    for (int n = 0; n < ncol; n++) {
        for (int g = 0; g < nl->nimg; g++) {
            const int a = nl->img_atom[g];
            const int np = nl->ip_displ[a + 1] - nl->ip_displ[a];
            const int ndc = nl->img_ndc[g];
            const int *gp = nl->grid_pos + nl->img_off[g];
            const double *chi = nl->chi + nl->img_chi_off[g];
            const double complex ph = cexp(I * theta[g]) * dV;
            double complex *al = alpha + (long)nl->ip_displ[a] * ncol + (long)n * np;
            for (int j = 0; j < np; j++) {
                double complex s = 0.0;
                for (int i = 0; i < ndc; i++) s += chi[(long)j * ndc + i] * x[(long)n * ldi + gp[i]];
                al[j] += ph * s;
            }
        }
    }
    for (int a = 0; a < nl->natom; a++) {
        const int np = nl->ip_displ[a + 1] - nl->ip_displ[a];
        for (int n = 0; n < ncol; n++)
            for (int j = 0; j < np; j++)
                alpha[(long)nl->ip_displ[a] * ncol + (long)n * np + j] *= nl->gamma[nl->ip_displ[a] + j];
    }
#pragma omp parallel for schedule(static)
    for (int n = 0; n < ncol; n++) {
        for (int g = 0; g < nl->nimg; g++) {
            const int a = nl->img_atom[g];
            const int np = nl->ip_displ[a + 1] - nl->ip_displ[a];
            const int ndc = nl->img_ndc[g];
            const int *gp = nl->grid_pos + nl->img_off[g];
            const double *chi = nl->chi + nl->img_chi_off[g];
            const double complex ph = cexp(-I * theta[g]);
            const double complex *al = alpha + (long)nl->ip_displ[a] * ncol + (long)n * np;
            for (int i = 0; i < ndc; i++) {
                double complex s = 0.0;
                for (int j = 0; j < np; j++) s += chi[(long)j * ndc + i] * al[j];
                Hx[(long)n * ldo + gp[i]] += ph * s;
            }
        }
    }
    free(theta);
    free(alpha);
}

/* Hx = (-0.5 Lap + Veff + c) x + Vnl x for Bloch columns (Hamiltonian_vectors_mult_kpt,
 * src/hamiltonianVecRoutines.c:132). */
void orc_hamiltonian_kpt(const orc_grid *gr, const orc_nonlocal *nl, const double *img_coords,
                         const double *k, const double *L, const double *veff, int ncol,
                         double c, const double complex *x, long ldi, double complex *Hx,
                         long ldo)
{
    orc_lap_plus_diag_orth_kpt(gr->Nx, gr->Ny, gr->Nz, gr->FDn, gr->cx, gr->cy, gr->cz, k, L,
                               ncol, -0.5, 1.0, c, veff, x, ldi, Hx, ldo);
    if (nl && nl->nimg > 0)
        orc_vnl_vec_mult_kpt(nl, img_coords, k, L, gr->dV, ncol, x, ldi, Hx, ldo);
}

/* Chebyshev filter for Bloch columns (ChebyshevFiltering_kpt, src/eigenSolverKpt.c:458). */
void orc_chebyshev_filter_kpt(const orc_grid *gr, const orc_nonlocal *nl,
                              const double *img_coords, const double *k, const double *L,
                              const double *veff, double complex *X, long ldi,
                              double complex *Y, long ldo, int ncol, int m, double a, double b,
                              double a0)
{
    const long Nd = (long)gr->Nx * gr->Ny * gr->Nz;
    const double e = 0.5 * (b - a);
    const double c = 0.5 * (b + a);
    double sigma = e / (a0 - c);
    const double sigma1 = sigma;
    const double gamma = 2.0 / sigma1;
    orc_hamiltonian_kpt(gr, nl, img_coords, k, L, veff, ncol, -c, X, ldi, Y, ldo);
    double vscal = sigma1 / e;
    for (int n = 0; n < ncol; n++)
        for (long i = 0; i < Nd; i++) Y[i + n * ldo] *= vscal;
    double complex *Ynew = (double complex *)malloc(sizeof(double complex) * Nd * (ncol > 0 ? ncol : 1));
    for (int j = 1; j < m; j++) {
        double sigma2 = 1.0 / (gamma - sigma);
        orc_hamiltonian_kpt(gr, nl, img_coords, k, L, veff, ncol, -c, Y, ldo, Ynew, Nd);
        vscal = 2.0 * sigma2 / e;
        double vscal2 = sigma * sigma2;
#pragma omp parallel for schedule(static)
        for (int n = 0; n < ncol; n++) {
            for (long i = 0; i < Nd; i++) {
                Ynew[i + n * Nd] *= vscal;
                Ynew[i + n * Nd] -= vscal2 * X[i + n * ldi];
                X[i + n * ldi] = Y[i + n * ldo];
                Y[i + n * ldo] = Ynew[i + n * Nd];
            }
        }
        sigma = sigma2;
    }
    free(Ynew);
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
