/*
 * sparc_gb300_shim.c -- the SPARC side of the binding to libsparc_gpu.so (route ii: SPARC's
 * own accelerator hooks, enabled by compiling SPARC with -DSPARCX_ACCEL -DACCEL and this
 * directory on the include path; accel.h and accel_kpt.h map the hook names here).
 *
 * One library context per process, created from SPARC_OBJ on the first hook call: grid and
 * second-derivative weights (D2_stencil_coeffs_*), dV, the nonlocal projectors flattened from
 * Atom_Influence_nloc / nlocProj (src/include/isddft.h:200-216, :247-265) and, for k-point
 * runs, the image coordinates. The projectors are installed again whenever the atom positions
 * change (relaxation, MD); the local potential Veff_loc_dmcomm is copied on every filter call,
 * since SPARC updates it in place each SCF iteration. A non-zero library status becomes
 * SPARC's own error convention: print and exit (src/eigenSolver.c:1368-1371).
 *
 * Supported by the GPU hooks: one process owning the whole grid (Nd_d_dmcomm == Nd), an
 * orthogonal cell (cell_typ 0), FD order 12; the hooks fall back to SPARC's CPU routines or
 * stop with a message where the library has no counterpart.
 */
#include <complex.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <lapacke.h>

#include "isddft.h"
#include "forces.h"
#include "sparc_gpu.h"
#include "accel.h"
#include "accel_kpt.h"

static sgpu_ctx *g_ctx = NULL;
static double *g_pos = NULL;  /* atom positions the projectors were installed for */
static int g_npos = 0;

static void check(int rc, const char *where)
{
    if (rc != SGPU_OK) {
        printf("libsparc_gpu: %s failed (status %d): %s\n", where, rc, sgpu_last_error());
        exit(EXIT_FAILURE);
    }
}

void gb300_not_provided(const char *what)
{
    printf("libsparc_gpu: the %s hook has no GPU counterpart in this library; "
           "build SPARC without -DSPARCX_ACCEL for this input\n", what);
    exit(EXIT_FAILURE);
}

/* flatten Atom_Influence_nloc / nlocProj into the library's layout and install it */
static void install_projectors(SPARC_OBJ *pSPARC)
{
    int nimg = 0, npos = 0;
    long nchi = 0;
    for (int t = 0; t < pSPARC->Ntypes; t++) {
        ATOM_NLOC_INFLUENCE_OBJ *ai = &pSPARC->Atom_Influence_nloc[t];
        for (int i = 0; i < ai->n_atom; i++) {
            nimg++;
            npos += ai->ndc[i];
            nchi += (long)ai->ndc[i] * pSPARC->nlocProj[t].nproj;
        }
    }
    int *img_atom = malloc(sizeof(int) * (nimg + 1));
    int *img_ndc = malloc(sizeof(int) * (nimg + 1));
    int *grid_pos = malloc(sizeof(int) * (npos + 1));
    double *chi = malloc(sizeof(double) * (nchi + 1));
    double *coords = malloc(sizeof(double) * (3 * nimg + 1));
    double *gamma = malloc(sizeof(double) * (pSPARC->IP_displ[pSPARC->n_atom] + 1));
    if (!img_atom || !img_ndc || !grid_pos || !chi || !coords || !gamma) {
        printf("libsparc_gpu: out of host memory flattening the projectors\n");
        exit(EXIT_FAILURE);
    }
    int g = 0, p = 0, a0 = 0;
    long c = 0;
    for (int t = 0; t < pSPARC->Ntypes; t++) {
        ATOM_NLOC_INFLUENCE_OBJ *ai = &pSPARC->Atom_Influence_nloc[t];
        const int np = pSPARC->nlocProj[t].nproj;
        for (int i = 0; i < ai->n_atom; i++, g++) {
            img_atom[g] = ai->atom_index[i];
            img_ndc[g] = ai->ndc[i];
            for (int d = 0; d < 3; d++) coords[3 * g + d] = ai->coords[3 * i + d];
            for (int k = 0; k < ai->ndc[i]; k++) grid_pos[p++] = ai->grid_pos[i][k];
            for (long k = 0; k < (long)ai->ndc[i] * np; k++)
                chi[c++] = pSPARC->nlocProj[t].Chi[i][k];
        }
        /* Gamma per projector column, in the (l != lloc, p, m) order of Vnl_vec_mult
         * (src/nlocVecRoutines.c:843-866) */
        for (int a = 0; a < pSPARC->nAtomv[t]; a++, a0++) {
            int col = pSPARC->IP_displ[a0], ld = 0;
            for (int l = 0; l <= pSPARC->psd[t].lmax; l++) {
                if (l == pSPARC->localPsd[t]) {
                    ld += pSPARC->psd[t].ppl[l];
                    continue;
                }
                for (int q = 0; q < pSPARC->psd[t].ppl[l]; q++)
                    for (int m = -l; m <= l; m++) gamma[col++] = pSPARC->psd[t].Gamma[ld + q];
                ld += pSPARC->psd[t].ppl[l];
            }
        }
    }
    check(sgpu_set_nonlocal(g_ctx, pSPARC->n_atom, pSPARC->IP_displ, gamma, nimg, img_atom,
                            img_ndc, grid_pos, chi),
          "sgpu_set_nonlocal");
    if (!pSPARC->isGammaPoint)
        check(sgpu_set_kpoint_geometry(g_ctx, pSPARC->range_x, pSPARC->range_y,
                                       pSPARC->range_z, nimg, coords),
              "sgpu_set_kpoint_geometry");
    free(img_atom);
    free(img_ndc);
    free(grid_pos);
    free(chi);
    free(coords);
    free(gamma);
}

/* the context for this SPARC_OBJ: created once, projectors refreshed when atoms moved */
static void ensure_context(SPARC_OBJ *pSPARC)
{
    if (pSPARC->Nd_d_dmcomm != pSPARC->Nd || pSPARC->cell_typ != 0) {
        printf("libsparc_gpu: the GPU hooks need one process owning the whole grid of an "
               "orthogonal cell (Nd_d_dmcomm = %d, Nd = %d, cell_typ = %d)\n",
               pSPARC->Nd_d_dmcomm, pSPARC->Nd, pSPARC->cell_typ);
        exit(EXIT_FAILURE);
    }
    if (!g_ctx) {
        const char *dev = getenv("SPARC_GB300_DEVICE");
        check(sgpu_create(&g_ctx, dev ? atoi(dev) : 0, pSPARC->Nx_d_dmcomm,
                          pSPARC->Ny_d_dmcomm, pSPARC->Nz_d_dmcomm, pSPARC->order / 2,
                          pSPARC->D2_stencil_coeffs_x, pSPARC->D2_stencil_coeffs_y,
                          pSPARC->D2_stencil_coeffs_z, pSPARC->dV),
              "sgpu_create");
        printf("libsparc_gpu: CheFSI filter, subspace eigensolver and nonlocal forces on the "
               "GPU (library version %d)\n", sgpu_version());
    }
    const int n = 3 * pSPARC->n_atom;
    if (g_npos != n || !g_pos || memcmp(g_pos, pSPARC->atom_pos, sizeof(double) * n) != 0) {
        install_projectors(pSPARC);
        free(g_pos);
        g_pos = malloc(sizeof(double) * n);
        memcpy(g_pos, pSPARC->atom_pos, sizeof(double) * n);
        g_npos = n;
    }
}

void gb300_ChebyshevFiltering(SPARC_OBJ *pSPARC, int *DMVertices, double *X, int ldi,
                              double *Y, int ldo, int ncol, int m, double a, double b,
                              double a0, int k, int spn_i, MPI_Comm comm)
{
    (void)DMVertices; (void)k; (void)comm;
    ensure_context(pSPARC);
    check(sgpu_set_veff(g_ctx, pSPARC->Nspin_spincomm, pSPARC->Veff_loc_dmcomm),
          "sgpu_set_veff");
    /* Y = filtered block; X is not needed afterwards: it receives H Y, which
     * DP_Project_Hamiltonian expects from the hook (src/eigenSolver.c:953-958) */
    check(sgpu_ChebyshevFiltering_y(g_ctx, spn_i, X, ldi, Y, ldo, ncol, m, a, b, a0,
                                    SGPU_PREC_FP64),
          "sgpu_ChebyshevFiltering_y");
    check(sgpu_Hamiltonian_vectors_mult(g_ctx, spn_i, ncol, 0.0, Y, ldo, X, ldi),
          "sgpu_Hamiltonian_vectors_mult");
}

void gb300_ChebyshevFiltering_kpt(SPARC_OBJ *pSPARC, int *DMVertices, double _Complex *X,
                                  int ldi, double _Complex *Y, int ldo, int ncol, int m,
                                  double a, double b, double a0, int kpt, int spn_i,
                                  MPI_Comm comm)
{
    (void)DMVertices; (void)comm;
    ensure_context(pSPARC);
    check(sgpu_set_veff(g_ctx, pSPARC->Nspin_spincomm, pSPARC->Veff_loc_dmcomm),
          "sgpu_set_veff");
    const double kv[3] = {pSPARC->k1_loc[kpt], pSPARC->k2_loc[kpt], pSPARC->k3_loc[kpt]};
    check(sgpu_ChebyshevFiltering_kpt(g_ctx, spn_i, kv, (double *)X, ldi, (double *)Y, ldo,
                                      ncol, m, a, b, a0, SGPU_PREC_FP64),
          "sgpu_ChebyshevFiltering_kpt");
    check(sgpu_Hamiltonian_vectors_mult_kpt(g_ctx, spn_i, kv, ncol, 0.0, (const double *)Y,
                                            ldo, (double *)X, ldi),
          "sgpu_Hamiltonian_vectors_mult_kpt");
}

/* LAPACKE_dsygvd-shaped: column-major, itype 1, eigenvectors, upper triangles */
int gb300_dsygv(int layout, int itype, char jobz, char uplo, int n, double *A, int lda,
                double *B, int ldb, double *w)
{
    if (layout != LAPACK_COL_MAJOR || itype != 1 || jobz != 'V' || uplo != 'U' || lda != n ||
        ldb != n) {
        printf("libsparc_gpu: DSYGV hook supports column-major, itype 1, 'V', 'U', ld = n\n");
        exit(EXIT_FAILURE);
    }
    if (!g_ctx) {
        printf("libsparc_gpu: DSYGV hook called before the filter hook created the context\n");
        exit(EXIT_FAILURE);
    }
    const int rc = sgpu_Solve_Generalized_EigenProblem(g_ctx, n, A, B, w);
    if (rc == SGPU_ERR_LINALG) {
        printf("libsparc_gpu: %s\n", sgpu_last_error());
        return 1;  /* SPARC prints info and goes on, as with LAPACK's info */
    }
    check(rc, "sgpu_Solve_Generalized_EigenProblem");
    return 0;
}

int gb300_dsyev(int layout, char jobz, char uplo, int n, double *A, int lda, double *w)
{
    if (layout != LAPACK_COL_MAJOR || jobz != 'V' || uplo != 'U' || lda != n) {
        printf("libsparc_gpu: DSYEV hook supports column-major, 'V', 'U', ld = n\n");
        exit(EXIT_FAILURE);
    }
    if (!g_ctx) {
        printf("libsparc_gpu: DSYEV hook called before the filter hook created the context\n");
        exit(EXIT_FAILURE);
    }
    const int rc = sgpu_Solve_Standard_EigenProblem(g_ctx, n, A, w);
    if (rc == SGPU_ERR_LINALG) {
        printf("libsparc_gpu: %s\n", sgpu_last_error());
        return 1;
    }
    check(rc, "sgpu_Solve_Standard_EigenProblem");
    return 0;
}

/* Calculate_nonlocal_forces_linear (src/forces.c:750): added to pSPARC->forces on the GPU for
 * spin-unpolarised runs (one orbital block, occupations occ[0..Nstates-1]) */
void gb300_nonlocal_forces_linear(SPARC_OBJ *pSPARC)
{
    if (pSPARC->spin_typ != 0 || pSPARC->Nspinor_spincomm != 1 || !g_ctx) {
        Calculate_nonlocal_forces_linear(pSPARC);
        return;
    }
    ensure_context(pSPARC);
    const double cell[3] = {pSPARC->range_x, pSPARC->range_y, pSPARC->range_z};
    check(sgpu_Calculate_nonlocal_forces(g_ctx, pSPARC->Nband_bandcomm, pSPARC->Xorb,
                                         pSPARC->Nd_d_dmcomm, pSPARC->occ, pSPARC->occfac, cell,
                                         pSPARC->forces),
          "sgpu_Calculate_nonlocal_forces");
}
