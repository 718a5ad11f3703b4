/*
 * CPU oracle for the SPARC CheFSI hot path (test infrastructure only; see sparc_oracle.c).
 */
#ifndef SPARC_ORACLE_H
#define SPARC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_FDN 8

typedef struct {
    int Nx, Ny, Nz, FDn;
    const double *cx, *cy, *cz; /* FDn+1 second-derivative weights per direction, / h^2 */
    double dV;
} orc_grid;

/* Flattened nonlocal projector set: natom atoms, ip_displ[natom+1] projector offsets,
 * gamma[ip_displ[natom]] expanded per projector column; nimg atom images (periodic copies)
 * each with img_atom (owning atom), img_ndc points, grid_pos at img_off and Chi (ndc x nproj,
 * column-major) at img_chi_off. */
typedef struct {
    int natom;
    const int *ip_displ;
    const double *gamma;
    int nimg;
    const int *img_atom;
    const int *img_ndc;
    const long *img_off;
    const long *img_chi_off;
    const int *grid_pos;
    const double *chi;
} orc_nonlocal;

void orc_fd_d2_weights(int FDn, double h, double *w);
void orc_lap_plus_diag_orth(int Nx, int Ny, int Nz, int FDn, const double *cx, const double *cy,
                            const double *cz, int ncol, double a, double b, double c,
                            const double *v, const double *x, long ldi, double *y, long ldo);
void orc_vnl_vec_mult(const orc_nonlocal *nl, double dV, int ncol, const double *x, long ldi,
                      double *Hx, long ldo);
void orc_hamiltonian(const orc_grid *gr, const orc_nonlocal *nl, const double *veff, int ncol,
                     double c, const double *x, long ldi, double *Hx, long ldo);
void orc_chebyshev_filter(const orc_grid *gr, const orc_nonlocal *nl, const double *veff,
                          double *X, long ldi, double *Y, long ldo, int ncol, int m, double a,
                          double b, double a0);
void orc_poisson_residual(const orc_grid *gr, double c, const double *x, const double *b,
                          double *r);
#ifndef __cplusplus
#include <complex.h>
void orc_lap_plus_diag_orth_kpt(int Nx, int Ny, int Nz, int FDn, const double *cx,
                                const double *cy, const double *cz, const double *k,
                                const double *L, int ncol, double a, double b, double c,
                                const double *v, const double complex *x, long ldi,
                                double complex *y, long ldo);
void orc_vnl_vec_mult_kpt(const orc_nonlocal *nl, const double *img_coords, const double *k,
                          const double *L, double dV, int ncol, const double complex *x,
                          long ldi, double complex *Hx, long ldo);
void orc_hamiltonian_kpt(const orc_grid *gr, const orc_nonlocal *nl, const double *img_coords,
                         const double *k, const double *L, const double *veff, int ncol,
                         double c, const double complex *x, long ldi, double complex *Hx,
                         long ldo);
void orc_chebyshev_filter_kpt(const orc_grid *gr, const orc_nonlocal *nl,
                              const double *img_coords, const double *k, const double *L,
                              const double *veff, double complex *X, long ldi,
                              double complex *Y, long ldo, int ncol, int m, double a, double b,
                              double a0);
#endif
int orc_num_threads(void);
void orc_set_num_threads(int n);

#ifdef __cplusplus
}
#endif

#endif
