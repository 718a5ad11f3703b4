/*
 * Kernel harness around the reference SPARC objects (test infrastructure only).
 *
 * ref_init() runs the reference's own set-up for an input file pair <name>.inpt/<name>.ion
 * (Initialize, src/initialization.c:229, then the influencing-atom, pseudocharge and nonlocal
 * projector steps of Calculate_EGS_elecDensEnergy, src/electronicGroundState.c:387-470), and
 * the ref_* entry points then call the reference's hot-path functions on caller-provided
 * arrays, so that golden vectors come from the reference code itself:
 *   Lap_plus_diag_vec_mult_orth  src/lapVecRoutines.c:306
 *   Vnl_vec_mult                 src/nlocVecRoutines.c:798
 *   Hamiltonian_vectors_mult     src/hamiltonianVecRoutines.c:45
 *   ChebyshevFiltering           src/eigenSolver.c:722
 *   poisson_residual             src/lapVecRoutines.c:69
 *   AAR                          src/linearSolver.c:37 (with Jacobi_preconditioner)
 *   Kerker_precond               src/mixing.c:462
 *   Mixing_periodic_pulay        src/mixing.c:213 (after Update_mixing_hist_xk), also with
 *                                collinear spin ([rho, magz], src/mixing.c:250-258)
 *   Calculate_Vxc (spin branch)  src/exchangeCorrelation.c:227
 * One system per process: the reference keeps its state in the SPARC_OBJ built here.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <mpi.h>

#include "isddft.h"
#include "initialization.h"
#include "electrostatics.h"
#include "nlocVecRoutines.h"
#include "lapVecRoutines.h"
#include "hamiltonianVecRoutines.h"
#include "eigenSolver.h"
#include "orbitalElecDensInit.h"
#include "linearSolver.h"
#include "mixing.h"
#include "electronicGroundState.h"

static SPARC_OBJ S;
static int g_ready = 0;

int ref_init(const char *name)
{
    char a0[] = "sparc", a1[] = "-name";
    char *nm = strdup(name);
    char *argv[] = {a0, a1, nm, NULL};
    int argc = 3;
    char **pargv = argv;
    MPI_Init(&argc, &pargv);
    memset(&S, 0, sizeof(S));
    Initialize(&S, argc, argv);
    GetInfluencingAtoms(&S);
    Generate_PseudoChargeDensity(&S);
    GetInfluencingAtoms_nloc(&S, &S.Atom_Influence_nloc, S.DMVertices_dmcomm, S.dmcomm);
    if (S.isGammaPoint)
        CalculateNonlocalProjectors(&S, &S.nlocProj, S.Atom_Influence_nloc, S.DMVertices_dmcomm,
                                    S.dmcomm);
    else
        CalculateNonlocalProjectors_kpt(&S, &S.nlocProj, S.Atom_Influence_nloc,
                                        S.DMVertices_dmcomm, S.dmcomm);
    Init_electronDensity(&S);
    g_ready = 1;
    return 0;
}

/* out[0..9] = Nx, Ny, Nz, Nd, order, n_atom, Ntypes, Nstates, IP_displ[n_atom], cell_typ */
void ref_dims(int *out)
{
    out[0] = S.Nx; out[1] = S.Ny; out[2] = S.Nz; out[3] = S.Nd;
    out[4] = S.order; out[5] = S.n_atom; out[6] = S.Ntypes; out[7] = S.Nstates;
    out[8] = S.IP_displ[S.n_atom]; out[9] = S.cell_typ;
}

/* out[0..6] = delta_x, delta_y, delta_z, dV, range_x, range_y, range_z */
void ref_grid(double *out)
{
    out[0] = S.delta_x; out[1] = S.delta_y; out[2] = S.delta_z; out[3] = S.dV;
    out[4] = S.range_x; out[5] = S.range_y; out[6] = S.range_z;
}

/* FDn+1 weights per direction, already divided by h^2 */
void ref_d2coeffs(double *cx, double *cy, double *cz)
{
    int FDn = S.order / 2;
    for (int p = 0; p <= FDn; p++) {
        cx[p] = S.D2_stencil_coeffs_x[p];
        cy[p] = S.D2_stencil_coeffs_y[p];
        cz[p] = S.D2_stencil_coeffs_z[p];
    }
}

/* per-type pseudopotential summary: lmax, lloc, nproj, ppl[0..lmax]; Gamma (sum ppl) */
void ref_psd(int ityp, int *ints, double *gamma)
{
    int lmax = S.psd[ityp].lmax;
    ints[0] = lmax;
    ints[1] = S.localPsd[ityp];
    ints[2] = S.nlocProj[ityp].nproj;
    ints[3] = S.nAtomv[ityp];
    int tot = 0;
    for (int l = 0; l <= lmax; l++) {
        ints[4 + l] = S.psd[ityp].ppl[l];
        tot += S.psd[ityp].ppl[l];
    }
    for (int i = 0; i < tot; i++) gamma[i] = S.psd[ityp].Gamma[i];
}

int ref_nloc_natom(int ityp) { return S.Atom_Influence_nloc[ityp].n_atom; }

/* out[0] = ndc, out[1] = atom_index of image iat of type ityp */
void ref_nloc_atom(int ityp, int iat, int *out)
{
    out[0] = S.Atom_Influence_nloc[ityp].ndc[iat];
    out[1] = S.Atom_Influence_nloc[ityp].atom_index[iat];
}

void ref_nloc_copy(int ityp, int iat, int *grid_pos, double *chi)
{
    int ndc = S.Atom_Influence_nloc[ityp].ndc[iat];
    int np = S.nlocProj[ityp].nproj;
    memcpy(grid_pos, S.Atom_Influence_nloc[ityp].grid_pos[iat], sizeof(int) * ndc);
    if (np > 0) memcpy(chi, S.nlocProj[ityp].Chi[iat], sizeof(double) * ndc * np);
}

void ref_atom_positions(double *xyz) { memcpy(xyz, S.atom_pos, sizeof(double) * 3 * S.n_atom); }

/* pseudocharge density b, reference b_ref, initial density (superposition of atoms) */
void ref_setup_fields(double *b, double *bref, double *rho0, double *scalars)
{
    memcpy(b, S.psdChrgDens, sizeof(double) * S.Nd);
    memcpy(bref, S.psdChrgDens_ref, sizeof(double) * S.Nd);
    memcpy(rho0, S.electronDens, sizeof(double) * S.Nd);
    scalars[0] = S.Esc;
    scalars[1] = S.PosCharge;
    scalars[2] = S.NegCharge;
    scalars[3] = S.Nelectron;
}

/* Parsed pseudopotential tables of type ityp (PSD_OBJ, src/include/isddft.h), as
 * read_pseudopotential_PSP (src/readfiles.c:1957) left them: ints = size, lmax, lloc,
 * is_r_uniform, Znucl, ppl[0..lmax]; scal = Vloc_0, fchrg, rc[0..lmax]; tables of `size`
 * points (UdV: sum(ppl) rows of `size`). Pass NULL table pointers to query ints only. */
void ref_psd_tables(int ityp, int *ints, double *scal, double *grid, double *udv,
                    double *rvloc, double *rhoiso, double *rhoc, double *gamma)
{
    PSD_OBJ *p = &S.psd[ityp];
    int lmax = p->lmax, n = p->size, tot = 0;
    ints[0] = n; ints[1] = lmax; ints[2] = S.localPsd[ityp]; ints[3] = p->is_r_uniform;
    ints[4] = S.Znucl[ityp];
    for (int l = 0; l <= lmax; l++) { ints[5 + l] = p->ppl[l]; tot += p->ppl[l]; }
    scal[0] = p->Vloc_0; scal[1] = p->fchrg;
    for (int l = 0; l <= lmax; l++) scal[2 + l] = p->rc[l];
    if (!grid) return;
    memcpy(grid, p->RadialGrid, sizeof(double) * n);
    memcpy(udv, p->UdV, sizeof(double) * n * tot);
    memcpy(rvloc, p->rVloc, sizeof(double) * n);
    memcpy(rhoiso, p->rhoIsoAtom, sizeof(double) * n);
    memcpy(rhoc, p->rho_c_table, sizeof(double) * n);
    memcpy(gamma, p->Gamma, sizeof(double) * tot);
}

/* pseudocharge cutoffs of type ityp (CUTOFF_x/y/z from Calculate_PseudochargeCutoff,
 * src/electrostatics.c:44), the atom count of the type and the set-up tolerances:
 * out = CUTOFF_x, CUTOFF_y, CUTOFF_z, nAtomv, TOL_PSEUDOCHARGE, REFERENCE_CUTOFF, NetCharge */
void ref_cutoff(int ityp, double *out)
{
    out[0] = S.CUTOFF_x[ityp]; out[1] = S.CUTOFF_y[ityp]; out[2] = S.CUTOFF_z[ityp];
    out[3] = S.nAtomv[ityp];
    out[4] = S.TOL_PSEUDOCHARGE; out[5] = S.REFERENCE_CUTOFF; out[6] = S.NetCharge;
}

/* pseudocharge density of the reference potentials (psdChrgDens_ref) and the atomic
 * superposition density before the charge scaling is undone: electronDens_at */
void ref_setup_fields2(double *bref, double *rho_at)
{
    memcpy(bref, S.psdChrgDens_ref, sizeof(double) * S.Nd);
    memcpy(rho_at, S.electronDens_at, sizeof(double) * S.Nd);
}

static int g_dims1[3] = {1, 1, 1};

void ref_lap_plus_diag(int ncol, double a, double b, double c, const double *v, const double *x,
                       double *y)
{
    Lap_plus_diag_vec_mult_orth(&S, S.Nd, S.DMVertices_dmcomm, ncol, a, b, c, v, x, S.Nd, y,
                                S.Nd, S.dmcomm, g_dims1);
}

void ref_vnl(int ncol, double *x, double *hx)
{
    Vnl_vec_mult(&S, S.Nd, S.Atom_Influence_nloc, S.nlocProj, ncol, x, S.Nd, hx, S.Nd,
                 S.dmcomm);
}

void ref_hamiltonian(int ncol, double *veff, double c, double *x, double *hx)
{
    Hamiltonian_vectors_mult(&S, S.Nd, S.DMVertices_dmcomm, veff, S.Atom_Influence_nloc,
                             S.nlocProj, ncol, c, x, S.Nd, hx, S.Nd, 0, S.dmcomm);
}

void ref_chebyshev(double *veff, int ncol, int m, double a, double b, double a0, double *X,
                   double *Y)
{
    double t;
    double *save = S.Veff_loc_dmcomm;
    int save_spin = S.spin_start_indx;
    S.Veff_loc_dmcomm = veff;
    S.spin_start_indx = 0;
    ChebyshevFiltering(&S, S.DMVertices_dmcomm, X, S.Nd, Y, S.Nd, ncol, m, a, b, a0, 0, 0,
                       S.dmcomm, &t);
    S.Veff_loc_dmcomm = save;
    S.spin_start_indx = save_spin;
}

void ref_poisson_residual(double c, double *x, double *b, double *r)
{
    double t;
    poisson_residual(&S, S.Nd, c, x, b, r, S.dmcomm, &t);
}

/* ---- SCF-side rows: the reference's own Calculate_Vxc / Calculate_elecstPotential on a
 * caller-provided density, and the set-up fields an SCF needs. */
#include "exchangeCorrelation.h"

/* model core density (NLCC, zeros when the psp has none); returns NLCC_flag */
int ref_core_density(double *rho_core)
{
    if (S.NLCC_flag && S.electronDens_core)
        memcpy(rho_core, S.electronDens_core, sizeof(double) * S.Nd);
    else
        memset(rho_core, 0, sizeof(double) * S.Nd);
    return S.NLCC_flag;
}

/* scalars of the SCF set-up: out = Beta, TOL_SCF, TOL_POISSON, TOL_PRECOND, TOL_LANCZOS,
 * xc_rhotol, ChebDegree, rhoTrigger, MixingParameter, MixingParameterSimple, MixingHistory,
 * PulayFrequency, MixingPrecond, precond_kerker_kTF, precond_kerker_thresh, MAXIT_POISSON,
 * MINIT_SCF, MAXIT_SCF, elec_T_type, Nchefsi */
void ref_scf_params(double *out)
{
    out[0] = S.Beta; out[1] = S.TOL_SCF; out[2] = S.TOL_POISSON; out[3] = S.TOL_PRECOND;
    out[4] = S.TOL_LANCZOS; out[5] = S.xc_rhotol; out[6] = S.ChebDegree; out[7] = S.rhoTrigger;
    out[8] = S.MixingParameter; out[9] = S.MixingParameterSimple; out[10] = S.MixingHistory;
    out[11] = S.PulayFrequency; out[12] = S.MixingPrecond; out[13] = S.precond_kerker_kTF;
    out[14] = S.precond_kerker_thresh; out[15] = S.MAXIT_POISSON; out[16] = S.MINIT_SCF;
    out[17] = S.MAXIT_SCF; out[18] = S.elec_T_type; out[19] = S.Nchefsi;
}

/* Vxc and e_xc of the reference for density rho (Calculate_Vxc on the LDA path) */
void ref_vxc(const double *rho, double *vxc, double *exc)
{
    memcpy(S.electronDens, rho, sizeof(double) * S.Nd);
    Calculate_Vxc(&S);
    memcpy(vxc, S.XCPotential, sizeof(double) * S.Nd);
    memcpy(exc, S.e_xc, sizeof(double) * S.Nd);
}

/* electrostatic potential of the reference for density rho; phi holds the initial guess */
void ref_poisson(const double *rho, double *phi)
{
    memcpy(S.electronDens, rho, sizeof(double) * S.Nd);
    memcpy(S.elecstPotential, phi, sizeof(double) * S.Nd);
    Calculate_elecstPotential(&S);
    memcpy(phi, S.elecstPotential, sizeof(double) * S.Nd);
}

/* AAR (src/linearSolver.c:37) with the reference's residual and Jacobi preconditioner and
 * its Poisson settings (omega = beta = 0.6, m = 7, p = 6, src/electrostatics.c:1653-1659):
 * solves b + (Lap + c) x = 0 in place from the initial x */
void ref_aar(double c, double *x, double *b, double tol, int max_iter)
{
    AAR(&S, poisson_residual, Jacobi_preconditioner, c, S.Nd_d, x, b, 0.6, 0.6, 7, 6, tol,
        max_iter, S.dmcomm_phi);
}

/* Kerker_precond (src/mixing.c:462) with the input's kTF, idiemac and TOL_PRECOND */
void ref_kerker(double *f, double a, double *Pf)
{
    Kerker_precond(&S, f, a, S.precond_kerker_kTF, S.precond_kerker_thresh, S.TOL_PRECOND,
                   S.Nd_d, S.DMVertices, Pf, S.dmcomm_phi);
}

/* periodic Pulay density mixing: ref_mix_init starts the history from rho0
 * (Update_mixing_hist_xk, src/electronicGroundState.c:1255), each ref_mix_step hands the
 * output density g of SCF iteration iter to Mixing_periodic_pulay and returns the mixed
 * density in g */
void ref_mix_init(const double *rho0)
{
    memcpy(S.electronDens, rho0, sizeof(double) * S.Nd_d);
    Update_mixing_hist_xk(&S);
}

void ref_mix_step(int iter, double *g)
{
    memcpy(S.electronDens, g, sizeof(double) * S.Nd_d);
    Mixing_periodic_pulay(&S, iter);
    memcpy(g, S.electronDens, sizeof(double) * S.Nd_d);
}

/* ---- collinear spin (spin_typ 1). ref_spin_fields: prm = MixingParameterMag,
 * MixingParameterSimpleMag, MixingPrecondMag; for a spin run also the initial [total, up,
 * down] density and magnetization as Init_electronDensity left them (src/orbitalElecDensInit.c
 * :145-151). Returns spin_typ. */
int ref_spin_fields(double *rho3, double *mag, double *prm)
{
    prm[0] = S.MixingParameterMag;
    prm[1] = S.MixingParameterSimpleMag;
    prm[2] = S.MixingPrecondMag;
    if (S.spin_typ == 1) {
        memcpy(rho3, S.electronDens, sizeof(double) * 3 * S.Nd);
        memcpy(mag, S.mag, sizeof(double) * S.Nd);
    }
    return S.spin_typ;
}

/* spin Vxc of the reference (Calculate_Vxc, spin branch) for [total, up, down] rho3:
 * vxc (2 Nd: up, down) and e_xc (Nd) */
void ref_vxc_spin(const double *rho3, double *vxc, double *exc)
{
    memcpy(S.electronDens, rho3, sizeof(double) * 3 * S.Nd);
    Calculate_Vxc(&S);
    memcpy(vxc, S.XCPotential, sizeof(double) * 2 * S.Nd);
    memcpy(exc, S.e_xc, sizeof(double) * S.Nd);
}

/* spin mixing: the history starts from [rho0, mag0]; each step hands [g, gmag] (output
 * density and magnetization of iteration iter) to Mixing_periodic_pulay and returns the
 * mixed pair in place */
void ref_mix_init_spin(const double *rho0, const double *mag0)
{
    memcpy(S.electronDens, rho0, sizeof(double) * S.Nd_d);
    memcpy(S.mag, mag0, sizeof(double) * S.Nd_d);
    Update_mixing_hist_xk(&S);
}

void ref_mix_step_spin(int iter, double *g, double *gmag)
{
    memcpy(S.electronDens, g, sizeof(double) * S.Nd_d);
    memcpy(S.mag, gmag, sizeof(double) * S.Nd_d);
    Mixing_periodic_pulay(&S, iter);
    memcpy(g, S.electronDens, sizeof(double) * S.Nd_d);
    memcpy(gmag, S.mag, sizeof(double) * S.Nd_d);
}

SPARC_OBJ *ref_harness_obj(void) { return &S; }
