/*
 * k-point (complex) entry points of the reference kernel harness (test infrastructure only).
 * They act on the SPARC_OBJ that ref_init() in ref_harness.c built for a system with a
 * k-point grid, and call the reference's complex twins:
 *   Lap_plus_diag_vec_mult_orth_kpt  src/lapVecRoutinesKpt.c:179
 *   Vnl_vec_mult_kpt                 src/nlocVecRoutines.c:889
 *   Hamiltonian_vectors_mult_kpt     src/hamiltonianVecRoutines.c:132
 *   ChebyshevFiltering_kpt           src/eigenSolverKpt.c:458
 * Complex arrays are passed as interleaved (re, im) doubles.
 */
#include <complex.h>
#include <stdlib.h>
#include <string.h>
#include <mpi.h>

#include "isddft.h"
#include "lapVecRoutinesKpt.h"
#include "nlocVecRoutines.h"
#include "hamiltonianVecRoutines.h"
#include "eigenSolverKpt.h"

SPARC_OBJ *ref_harness_obj(void);

/* number of k-points; k (3 per point, Cartesian, 1/Bohr, as k1_loc/k2_loc/k3_loc) and weights */
int ref_kpoints(double *k, double *w)
{
    SPARC_OBJ *S = ref_harness_obj();
    for (int i = 0; i < S->Nkpts_kptcomm; i++) {
        k[3 * i] = S->k1_loc[i];
        k[3 * i + 1] = S->k2_loc[i];
        k[3 * i + 2] = S->k3_loc[i];
        w[i] = S->kptWts_loc[i];
    }
    return S->Nkpts_kptcomm;
}

/* image coordinates (Atom_Influence_nloc.coords) of image iat of type ityp */
void ref_nloc_image_coords(int ityp, int iat, double *xyz)
{
    SPARC_OBJ *S = ref_harness_obj();
    memcpy(xyz, S->Atom_Influence_nloc[ityp].coords + 3 * iat, 3 * sizeof(double));
}

/* the complex projector of image iat (real values; returns the largest |imag|) */
double ref_nloc_copy_kpt(int ityp, int iat, int *grid_pos, double *chi)
{
    SPARC_OBJ *S = ref_harness_obj();
    int ndc = S->Atom_Influence_nloc[ityp].ndc[iat];
    int np = S->nlocProj[ityp].nproj;
    double mi = 0.0;
    memcpy(grid_pos, S->Atom_Influence_nloc[ityp].grid_pos[iat], sizeof(int) * ndc);
    for (int i = 0; i < ndc * np; i++) {
        chi[i] = creal(S->nlocProj[ityp].Chi_c[iat][i]);
        if (fabs(cimag(S->nlocProj[ityp].Chi_c[iat][i])) > mi)
            mi = fabs(cimag(S->nlocProj[ityp].Chi_c[iat][i]));
    }
    return mi;
}

static int g_dims1k[3] = {1, 1, 1};

void ref_lap_plus_diag_kpt(int kpt, int ncol, double a, double b, double c, const double *v,
                           const double *x, double *y)
{
    SPARC_OBJ *S = ref_harness_obj();
    Lap_plus_diag_vec_mult_orth_kpt(S, S->Nd, S->DMVertices_dmcomm, ncol, a, b, c, v,
                                    (const double _Complex *)x, S->Nd, (double _Complex *)y,
                                    S->Nd, S->dmcomm, g_dims1k, kpt);
}

void ref_vnl_kpt(int kpt, int ncol, double *x, double *hx)
{
    SPARC_OBJ *S = ref_harness_obj();
    Vnl_vec_mult_kpt(S, S->Nd, S->Atom_Influence_nloc, S->nlocProj, ncol,
                     (double _Complex *)x, S->Nd, (double _Complex *)hx, S->Nd, kpt, S->dmcomm);
}

void ref_hamiltonian_kpt(int kpt, int ncol, double *veff, double c, double *x, double *hx)
{
    SPARC_OBJ *S = ref_harness_obj();
    Hamiltonian_vectors_mult_kpt(S, S->Nd, S->DMVertices_dmcomm, veff, S->Atom_Influence_nloc,
                                 S->nlocProj, ncol, c, (double _Complex *)x, S->Nd,
                                 (double _Complex *)hx, S->Nd, 0, kpt, S->dmcomm);
}

void ref_chebyshev_kpt(int kpt, double *veff, int ncol, int m, double a, double b, double a0,
                       double *X, double *Y)
{
    SPARC_OBJ *S = ref_harness_obj();
    double t;
    double *save = S->Veff_loc_dmcomm;
    int save_spin = S->spin_start_indx;
    S->Veff_loc_dmcomm = veff;
    S->spin_start_indx = 0;
    ChebyshevFiltering_kpt(S, S->DMVertices_dmcomm, (double _Complex *)X, S->Nd,
                           (double _Complex *)Y, S->Nd, ncol, m, a, b, a0, kpt, 0, S->dmcomm, &t);
    S->Veff_loc_dmcomm = save;
    S->spin_start_indx = save_spin;
}
