/*
 * sparc_gpu.h — C ABI of the GB300 (sm_103a) CheFSI hot-path library, libsparc_gpu.so.
 *
 * The entry points mirror the reference SPARC functions on the Chebyshev-filtered subspace
 * iteration path. Each keeps the reference's argument order and meaning, with two changes:
 *   * the SPARC_OBJ* and MPI_Comm arguments are replaced by an opaque sgpu_ctx* that holds
 *     the device-resident copies of what those functions read from SPARC_OBJ (grid, FD
 *     weights, local potential, nonlocal projectors), filled once by the sgpu_set_* calls;
 *   * every function returns an int status (SGPU_OK or an SGPU_ERR_* code, with the text in
 *     sgpu_last_error()) where the reference returns void and exits on error. The SPARC-side
 *     shim translates a non-zero status into the reference's print-and-exit behaviour.
 *
 * Array arguments may be host memory (the reference's own malloc'ed buffers: the library
 * stages them through device memory inside the call) or device memory (used in place).
 * Orbital blocks are column-major with leading dimensions ldi/ldo >= Nd, grid index
 * i + j*Nx + k*Nx*Ny, exactly as in the reference (src/lapVecRoutines.c:313-314).
 * All calls on one context are serialised on that context's CUDA stream and return after
 * the stream has completed, so host buffers may be reused immediately.
 */
#ifndef SPARC_GPU_H
#define SPARC_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sgpu_ctx sgpu_ctx;

enum {
    SGPU_OK = 0,
    SGPU_ERR_ARG = 1,           /* invalid argument (size, pointer, unsupported option) */
    SGPU_ERR_CUDA = 2,          /* CUDA runtime / library error */
    SGPU_ERR_NOMEM = 3,         /* device allocation failed */
    SGPU_ERR_STATE = 4,         /* a required sgpu_set_* call has not been made */
    SGPU_ERR_NOT_CONVERGED = 5, /* an iterative solver hit its iteration cap */
    SGPU_ERR_LINALG = 6,        /* factorisation / eigensolver failure (non-SPD, no conv.) */
    SGPU_ERR_NONFINITE = 7,     /* NaN or Inf detected in an input or a result */
    SGPU_ERR_KERNEL_WAIT = 8    /* a kernel's bounded wait on its own copies ran out: the
                                 * results of the calls since the last check are invalid */
};

/* precision of the Chebyshev filter arithmetic */
enum { SGPU_PREC_FP64 = 64, SGPU_PREC_FP32 = 32 };

const char *sgpu_last_error(void);
int sgpu_version(void);

/* ---------------------------------------------------------------- context / set-up */

/* Grid and FD data that the reference reads from SPARC_OBJ: Nx, Ny, Nz, order/2 (FDn, must
 * be 6), D2_stencil_coeffs_{x,y,z}[0..FDn] (already divided by h^2, as built in
 * src/initialization.c:2141-2146) and dV. Periodic boundaries in all three directions.
 * device: CUDA ordinal to use. */
int sgpu_create(sgpu_ctx **ctx, int device, int Nx, int Ny, int Nz, int FDn,
                const double *D2_stencil_coeffs_x, const double *D2_stencil_coeffs_y,
                const double *D2_stencil_coeffs_z, double dV);
int sgpu_destroy(sgpu_ctx *ctx);

/* Replace the FD weights and dV of a context whose cell lengths changed at a fixed grid (a
 * strained geometry): the same data sgpu_create takes. */
int sgpu_set_grid_coeffs(sgpu_ctx *ctx, const double *D2_stencil_coeffs_x,
                         const double *D2_stencil_coeffs_y, const double *D2_stencil_coeffs_z,
                         double dV);

/* Local effective potential, nspin contiguous blocks of Nd values
 * (pSPARC->Veff_loc_dmcomm, src/include/isddft.h:540). */
int sgpu_set_veff(sgpu_ctx *ctx, int nspin, const double *Veff_loc);

/* Nonlocal projectors, flattened from the reference's ATOM_NLOC_INFLUENCE_OBJ and
 * NLOC_PROJ_OBJ (src/include/isddft.h:202-216, :247-265; built by GetInfluencingAtoms_nloc
 * and CalculateNonlocalProjectors, src/nlocVecRoutines.c:43, :394):
 *   n_atom, IP_displ[n_atom+1]      projector offsets per atom (pSPARC->IP_displ)
 *   Gamma[IP_displ[n_atom]]         psd[type].Gamma expanded per projector column, in the
 *                                   reference's (l != lloc, np, m) order
 *   n_img images (periodic copies of atoms whose rc-sphere meets the cell), image g has
 *   img_atom[g] (Atom_Influence_nloc.atom_index), img_ndc[g] points, and its grid_pos and
 *   Chi (ndc x nproj, column-major) stored back to back in image order. */
int sgpu_set_nonlocal(sgpu_ctx *ctx, int n_atom, const int *IP_displ, const double *Gamma,
                      int n_img, const int *img_atom, const int *img_ndc, const int *grid_pos,
                      const double *Chi);

/* ------------------------------------------------------------------------- hot path */

/* y = (a*Lap + b*diag(v) + c*I) x for ncol columns.
 * Replaces Lap_plus_diag_vec_mult_orth (src/lapVecRoutines.c:306); v may be NULL. */
int sgpu_Lap_plus_diag_vec_mult_orth(sgpu_ctx *ctx, int ncol, double a, double b, double c,
                                     const double *v, const double *x, int ldi, double *y,
                                     int ldo);

/* Lapx = (Lap + c*I) x. Replaces Lap_vec_mult (src/lapVecRoutines.c:37) for cell_typ == 0. */
int sgpu_Lap_vec_mult(sgpu_ctx *ctx, int ncol, double c, const double *x, int ldi,
                      double *Lapx, int ldo);

/* Hx += Vnl x. Replaces Vnl_vec_mult (src/nlocVecRoutines.c:798). */
int sgpu_Vnl_vec_mult(sgpu_ctx *ctx, int ncol, const double *x, int ldi, double *Hx, int ldo);

/* The same Hx += Vnl x for callers that cannot allocate device memory (for example a host
 * application whose own pool allocator reserves all GPU memory, or a caller that cannot
 * accept the device-wide synchronisation of cudaFree). No counterpart in the reference.
 * It allocates nothing: the projection coefficients live in a fixed 8 MiB scratch array
 * inside the library (held on every GPU that loads the library until exit), so
 * n_proj * round_up(ncol, 8) must not exceed 1048576 (larger requests return SGPU_ERR_ARG);
 * x and Hx must be device pointers. Each CUDA context holds its own copy of the array; the
 * first call in a context looks up its address there, so make it before any stream capture.
 * All calls in one context share that array (each clears it first): calls that overlap on
 * the GPU race and must be serialised. */
int sgpu_Vnl_vec_mult_noalloc(sgpu_ctx *ctx, int ncol, const double *x, int ldi, double *Hx,
                              int ldo);

/* Hx = (-0.5*Lap + Veff[spin] + c) x + Vnl x. Replaces Hamiltonian_vectors_mult
 * (src/hamiltonianVecRoutines.c:45) for an orthogonal cell without exact exchange,
 * meta-GGA, Hubbard or spin-orbit terms. */
int sgpu_Hamiltonian_vectors_mult(sgpu_ctx *ctx, int spin, int ncol, double c, const double *x,
                                  int ldi, double *Hx, int ldo);

/* Degree-m Chebyshev filter on [a, b] with lower bound a0, Hamiltonian of spin block spin.
 * On return Y holds the filtered block and X the degree m-1 iterate, as in the reference.
 * precision: SGPU_PREC_FP64 (the drop-in) or SGPU_PREC_FP32 (the recurrence and H apply in
 * FP32; inputs and outputs stay FP64 arrays). Replaces ChebyshevFiltering
 * (src/eigenSolver.c:722) and its ACCEL_ChebyshevFiltering hook (src/eigenSolver.c:314-321). */
int sgpu_ChebyshevFiltering(sgpu_ctx *ctx, int spin, double *X, int ldi, double *Y, int ldo,
                            int ncol, int m, double a, double b, double a0, int precision);

/* The same filter with X as input only: Y receives the filtered block and the host array X is
 * left as it was (no copy back). eigSolve_CheFSI never reads X after the filter:
 * Project_Hamiltonian writes H*Y into Xorb next (src/eigenSolver.c:349-364, :1596), so a
 * shim can bind ChebyshevFiltering here and save a third of the host-device copies. X must
 * be a host array (for device blocks use sgpu_ChebyshevFiltering, which works in place). */
int sgpu_ChebyshevFiltering_y(sgpu_ctx *ctx, int spin, const double *X, int ldi, double *Y,
                              int ldo, int ncol, int m, double a, double b, double a0,
                              int precision);

/* The same filter on FP32 blocks (host or device), for callers that keep the orbital block in
 * FP32 between filter calls (the mixed-precision SCF). No counterpart in the reference, which
 * filters in FP64 only; the recurrence scalars are the reference's, computed in FP64. */
int sgpu_ChebyshevFiltering_f32(sgpu_ctx *ctx, int spin, float *X, int ldi, float *Y, int ldo,
                                int ncol, int m, double a, double b, double a0);

/* r = b + (Lap + c*I) x for one grid vector. Replaces poisson_residual
 * (src/lapVecRoutines.c:69). */
int sgpu_poisson_residual(sgpu_ctx *ctx, double c, const double *x, const double *b,
                          double *r);

/* ------------------------------------------------------------ k-point (Bloch) rows */

/* Cell lengths (range_x/y/z) and the coordinates of the n_img atom images of the nonlocal
 * set, in the order given to sgpu_set_nonlocal (Atom_Influence_nloc.coords,
 * src/include/isddft.h:202-216); needed for the Bloch factors of the k-point calls. */
int sgpu_set_kpoint_geometry(sgpu_ctx *ctx, double Lx, double Ly, double Lz, int n_img,
                             const double *img_coords);

/* Complex blocks below are interleaved (re, im) doubles, i.e. SPARC's double _Complex arrays;
 * k = (k1_loc[kpt], k2_loc[kpt], k3_loc[kpt]) in 1/Bohr. */

/* y = (a*Lap + b*diag(v) + c*I) x for Bloch columns at k. Replaces
 * Lap_plus_diag_vec_mult_orth_kpt (src/lapVecRoutinesKpt.c:179). */
int sgpu_Lap_plus_diag_vec_mult_orth_kpt(sgpu_ctx *ctx, const double *k, int ncol, double a,
                                         double b, double c, const double *v, const double *x,
                                         int ldi, double *y, int ldo);

/* Hx += Vnl x at k. Replaces Vnl_vec_mult_kpt (src/nlocVecRoutines.c:889). */
int sgpu_Vnl_vec_mult_kpt(sgpu_ctx *ctx, const double *k, int ncol, const double *x, int ldi,
                          double *Hx, int ldo);

/* Hx = (-0.5*Lap + Veff[spin] + c) x + Vnl x at k. Replaces Hamiltonian_vectors_mult_kpt
 * (src/hamiltonianVecRoutines.c:132). */
int sgpu_Hamiltonian_vectors_mult_kpt(sgpu_ctx *ctx, int spin, const double *k, int ncol,
                                      double c, const double *x, int ldi, double *Hx, int ldo);

/* Chebyshev filter of Bloch columns at k (complex128, or complex64 arithmetic with
 * SGPU_PREC_FP32). Replaces ChebyshevFiltering_kpt (src/eigenSolverKpt.c:458). */
int sgpu_ChebyshevFiltering_kpt(sgpu_ctx *ctx, int spin, const double *k, double *X, int ldi,
                                double *Y, int ldo, int ncol, int m, double a, double b,
                                double a0, int precision);

/* ------------------------------------------------------------- Rayleigh-Ritz step */

/* HY = H Y (spin block spin), Hp = Yᵀ HY and Mp = Yᵀ Y (Ns x Ns = ncol x ncol, column-major,
 * full symmetric). Replaces DP_Project_Hamiltonian (src/eigenSolver.c:939) on one process,
 * including its ACCEL_DGEMM hooks (:1003-1017). */
int sgpu_Project_Hamiltonian(sgpu_ctx *ctx, int spin, const double *Y, int ldi, double *HY,
                             int ldo, int ncol, double *Hp, double *Mp);

/* The Cholesky-orthonormalising variant: Mp = Yᵀ Y, Mp = Rᵀ R, Y <- Y R^{-1} (Y is
 * overwritten by the orthonormal block), HY = H Y, Hp = Yᵀ HY. Replaces
 * DP_Project_Hamiltonian_std (src/eigenSolver.c:1088-1252). */
int sgpu_Project_Hamiltonian_std(sgpu_ctx *ctx, int spin, double *Y, int ldi, double *HY,
                                 int ldo, int ncol, double *Hp);

/* Hp q = lambda q (upper triangle referenced); Hp becomes Q. The standard-eigenproblem branch
 * of DP_Solve_Generalized_EigenProblem (LAPACKE_dsyevd, src/eigenSolver.c:1318-1321). */
int sgpu_Solve_Standard_EigenProblem(sgpu_ctx *ctx, int Ns, double *Hp, double *lambda);

/* Hp q = lambda Mp q for the Ns x Ns pencil (upper triangles referenced). On return Hp holds
 * the eigenvectors Q (column-major), lambda the eigenvalues in ascending order, and Mp its
 * Cholesky factor. Replaces DP_Solve_Generalized_EigenProblem (src/eigenSolver.c:1262),
 * i.e. LAPACKE_dsygvd(COL_MAJOR, 1, 'V', 'U', ...) at :1318. */
int sgpu_Solve_Generalized_EigenProblem(sgpu_ctx *ctx, int Ns, double *Hp, double *Mp,
                                        double *lambda);

/* X = Y Q with Q Ns x Ns (ncol = Ns). Replaces DP_Subspace_Rotation (src/eigenSolver.c:1386). */
int sgpu_Subspace_Rotation(sgpu_ctx *ctx, const double *Y, int ldi, const double *Q, int ncol,
                           double *X, int ldo);

/* The Rayleigh-Ritz products of the mixed SCF's FP32 phase on device FP32 blocks (for callers
 * that keep the orbitals in FP32, beside sgpu_ChebyshevFiltering_f32): HY = H Y in FP32, then
 * Hp = Yᵀ HY and Mp = Yᵀ Y, and X = Y Q, as FP32-accurate products with FP32 accumulation
 * (the library's tcgen05 split-slice kernels, sgpu_set_rr_products; or cuBLAS,
 * sgpu_set_gemm_emulation);
 * Hp, Mp and Q are FP64 (host or device). FP32-precision counterparts of the two calls
 * above. */
int sgpu_Project_Hamiltonian_f32(sgpu_ctx *ctx, int spin, const float *Y, int ldi, float *HY,
                                 int ldo, int ncol, double *Hp, double *Mp);
int sgpu_Subspace_Rotation_f32(sgpu_ctx *ctx, const float *Y, int ldi, const double *Q, int ncol,
                               float *X, int ldo);

/* Lanczos estimate of the smallest and largest eigenvalue of H (spin block spin) from start
 * vector x0 (Nd values), stopping when both change by less than tol between iterations.
 * Replaces Lanczos (src/eigenSolver.c:1920) as called by Chebyshevfilter_constants (:589). */
int sgpu_Lanczos(sgpu_ctx *ctx, int spin, const double *x0, double tol, int maxit,
                 double *eigmin, double *eigmax);

/* ------------------------------------------------------------------- SCF-side rows */

/* rho = (1/dV) sum_n occfac * occ[n] * psi_n^2 (Gamma point, one spin).
 * Replaces CalculateDensity_psi (src/electronDensity.c:104). occ: ncol values. */
int sgpu_CalculateDensity_psi(sgpu_ctx *ctx, const double *psi, int ld, int ncol,
                              const double *occ, double occfac, double *rho);

/* LDA exchange-correlation (Slater exchange + Perdew-Wang 92 correlation) on
 * max(rho + rho_core, xc_rhotol): vxc (potential) and exc (energy per particle).
 * rho_core may be NULL (no core correction). Replaces the LDA_PW branch of Calculate_Vxc
 * (src/exchangeCorrelation.c:36, slater :459, pw :475, add_rho_core :1254). */
int sgpu_Calculate_Vxc_LDA_PW(sgpu_ctx *ctx, const double *rho, const double *rho_core,
                              double xc_rhotol, double *vxc, double *exc);

/* Spin-polarised LDA (Slater exchange + PW92 correlation, collinear spin): each spin density
 * plus half of rho_core (may be NULL), clamped at xc_rhotol; vxc receives 2 Nd values (up,
 * then down), exc Nd values (energy per particle of the total). Replaces the spin branch of
 * Calculate_Vxc (src/exchangeCorrelation.c:227-347, slater_spin :759, pw_spin :787,
 * add_rho_core :1254 with three columns). */
int sgpu_Calculate_Vxc_LSDA_PW(sgpu_ctx *ctx, const double *rho_up, const double *rho_dn,
                               const double *rho_core, double xc_rhotol, double *vxc,
                               double *exc);

/* Alternating Anderson-Richardson solve of b + (Lap + c) x = 0 with the Jacobi preconditioner
 * (x: initial guess in, solution out). Replaces AAR (src/linearSolver.c:37) called with
 * poisson_residual and Jacobi_preconditioner (src/electrostatics.c:1682). Returns
 * SGPU_ERR_NOT_CONVERGED (x still written) when max_iter is reached. */
int sgpu_AAR(sgpu_ctx *ctx, double c, double *x, const double *b, double omega, double beta,
             int m, int p, double tol, int max_iter, int *iters);

/* phi with -Lap phi = 4 pi (b + rho), zero mean; phi holds the initial guess on entry.
 * Replaces Calculate_elecstPotential (src/electrostatics.c:1593) for a periodic cell
 * (AAR with omega = beta = 0.6, m = 7, p = 6). */
int sgpu_Calculate_elecstPotential(sgpu_ctx *ctx, const double *rho, const double *b,
                                   double *phi, double tol, int max_iter, int *iters);

/* Periodic-Pulay density mixing. sgpu_Mixing_init sets the parameters (the SPARC_OBJ fields
 * MixingHistory, PulayFrequency, PulayRestartFlag, MixingParameter, MixingParameterSimple,
 * MixingPrecond == 1 (Kerker), precond_kerker_kTF, precond_kerker_thresh, TOL_PRECOND,
 * NegCharge) and the first input density (Update_mixing_hist_xk); each
 * sgpu_Mixing_periodic_pulay call takes the output density of SCF iteration iter_count in
 * rho and returns the next input density in rho. The history stays on the device.
 * Replaces Mixing_periodic_pulay (src/mixing.c:213) and Kerker_precond (:462). */
int sgpu_Mixing_init(sgpu_ctx *ctx, int history, int pulay_frequency, int pulay_restart,
                     double mixing_parameter, double mixing_parameter_simple, int kerker,
                     double kTF, double idiemac, double tol_precond, double neg_charge,
                     const double *rho_in);
int sgpu_Mixing_periodic_pulay(sgpu_ctx *ctx, int iter_count, double *rho);

/* The same mixing for collinear spin (spin_typ 1): the mixed vector is [rho, magz]
 * (src/mixing.c:250-258); the total-density residual is preconditioned as above, the
 * magnetization residual by MixingParameterMag / MixingParameterSimpleMag alone
 * (MixingPrecondMag = 0, the reference's default), each part is shifted to keep its residual's
 * integral (src/mixing.c:376-385), and only rho is clamped and rescaled. rho and mag (Nd each)
 * hold the output density and magnetization of iteration iter_count on entry and the next
 * input on return. */
int sgpu_Mixing_init_spin(sgpu_ctx *ctx, int history, int pulay_frequency, int pulay_restart,
                          double mixing_parameter, double mixing_parameter_simple,
                          double mixing_parameter_mag, double mixing_parameter_simple_mag,
                          int kerker, double kTF, double idiemac, double tol_precond,
                          double neg_charge, const double *rho_in, const double *mag_in);
int sgpu_Mixing_periodic_pulay_spin(sgpu_ctx *ctx, int iter_count, double *rho, double *mag);

/* error = ||rho_out - rho_in|| / ||rho_out||. Replaces Evaluate_scf_error
 * (src/electronicGroundState.c:1160). */
int sgpu_Evaluate_scf_error(sgpu_ctx *ctx, const double *rho_out, const double *rho_in,
                            double *error);

/* One (k-point, spin, band-block) unit of a batched filter call. X and Y are device arrays of
 * complex values (re, im interleaved), complex128 for SGPU_PREC_FP64 and complex64 (float
 * pairs) for SGPU_PREC_FP32, Nd x ncol column-major with leading dimensions ldi, ldo. */
typedef struct {
    int spin;                   /* local-potential block (sgpu_set_veff nspin) */
    double k[3];                /* Bloch vector, Cartesian, 1/Bohr */
    void *X;
    int ldi;
    void *Y;
    int ldo;
    int ncol;                   /* may differ between blocks */
    double a, b, a0;            /* this block's filter interval and lower bound */
} sgpu_filter_block;

/* ChebyshevFiltering_kpt (src/eigenSolverKpt.c:458) over all blocks at once, degree m for
 * every block: each degree is one projection, one stencil and one apply launch covering all
 * blocks, and the m degrees run as one CUDA graph captured on the first call and replayed
 * while the blocks' shapes and buffers repeat. Same outputs as one sgpu_ChebyshevFiltering_kpt
 * call per block. The reference filters its (k, spin) blocks one after another
 * (src/eigenSolverKpt.c:165-215). */
int sgpu_ChebyshevFiltering_batched(sgpu_ctx *ctx, int nblk, const sgpu_filter_block *blocks,
                                    int m, int precision);

/* Rayleigh-Ritz step at a k-point, complex128 (interleaved) blocks Nd x ncol and Ns x Ns
 * column-major matrices, host or device. Project: HY = H_k Y (written to HY), Hp = Yᴴ HY,
 * Mp = Yᴴ Y; replaces DP_Project_Hamiltonian_kpt (src/eigenSolverKpt.c:676; its ZGEMMs at
 * :747-760). Solve: Hp q = lambda Mp q (upper triangles; cuSOLVER zhegvd), Hp becomes Q;
 * replaces DP_Solve_Generalized_EigenProblem_kpt (:836). Rotation: X = Y Q; replaces
 * DP_Subspace_Rotation_kpt (:947). */
int sgpu_Project_Hamiltonian_kpt(sgpu_ctx *ctx, int spin, const double *k, const double *Y,
                                 int ldi, double *HY, int ldo, int ncol, double *Hp, double *Mp);
int sgpu_Solve_Generalized_EigenProblem_kpt(sgpu_ctx *ctx, int Ns, double *Hp, double *Mp,
                                            double *lambda);
int sgpu_Subspace_Rotation_kpt(sgpu_ctx *ctx, const double *Y, int ldi, const double *Q,
                               int ncol, double *X, int ldo);

/* One CheFSI pass over all (k, spin) blocks (eigSolve_CheFSI_kpt's per-block filter,
 * projection, eigensolve and rotation, src/eigenSolverKpt.c:165-300): the batched filter of
 * sgpu_ChebyshevFiltering_batched, then per block H Y, Hp = Yᴴ HY, Mp = Yᴴ Y (ZGEMM, or
 * CGEMM for complex64 blocks), the FP64 generalized eigensolve and X = Y Q. On return each
 * block's X holds its Ritz vectors and Y its filtered block; lambda (host, sum of ncol)
 * receives the blocks' Ritz values, block after block, ascending within a block. */
int sgpu_CheFSI_batched(sgpu_ctx *ctx, int nblk, const sgpu_filter_block *blocks, int m,
                        int precision, double *lambda);

/* ----------------------------------------------------------------- set-up (per geometry) */

/* Radial tables of one atom type, as read_pseudopotential_PSP (src/readfiles.c:1957) leaves
 * them in PSD_OBJ (src/include/isddft.h): UdV holds sum(ppl) rows of `size` values (u_l/r,
 * rows of l == lloc unused), rVloc = r*Vloc(r), densities already divided by 4 pi, and rc[l]
 * the projector radii after the reader's extension to the last |UdV| > 1e-8. */
typedef struct {
    int size;                   /* radial points */
    int lmax, lloc;             /* psd.lmax, localPsd */
    int Znucl;                  /* valence charge (SPARC's Znucl) */
    const int *ppl;             /* projectors per l, lmax+1 */
    const double *rc;           /* lmax+1 */
    double Vloc_0, fchrg;       /* Vloc(0); model-core charge flag (> 0: NLCC) */
    const double *RadialGrid, *UdV, *rVloc, *rhoIsoAtom, *rho_c_table, *Gamma;
} sgpu_psd;

/* Store the tables of ntypes (<= 8) atom types on the device with their spline slopes
 * (getYD_gen, src/tools.c:372; src/initialization.c:3470-3492). lmax <= 3. */
int sgpu_set_psd(sgpu_ctx *ctx, int ntypes, const sgpu_psd *psd);

/* Pseudocharge cut-off radii per type by the reference's bisection on the integrated charge
 * (Calculate_PseudochargeCutoff, src/electrostatics.c:44). cell: range_x/y/z; tol:
 * TOL_PSEUDOCHARGE. cutoff receives CUTOFF_x/y/z per type (3*ntypes values). */
int sgpu_Calculate_PseudochargeCutoff(sgpu_ctx *ctx, const double *cell, double tol,
                                      double *cutoff);

/* Pseudocharge density b (psdChrgDens), its reference-potential twin b_ref
 * (psdChrgDens_ref), the atomic superposition density scaled to the electron count
 * (electronDens_at, the initial density) and the model core density (electronDens_core),
 * computed on the device for atoms at atom_pos (3*n_atom, type-major, nAtomv per type).
 * cutoff: 3 per type (NULL: the values of the last cut-off call); ref_cutoff:
 * REFERENCE_CUTOFF; net_charge: NetCharge. scalars (3, may be NULL) = Esc, PosCharge,
 * NegCharge. b_ref and rho_core may be NULL; arrays may be host or device memory. Replaces
 * GetInfluencingAtoms and Generate_PseudoChargeDensity (src/electrostatics.c:578, :772). */
int sgpu_Generate_PseudoChargeDensity(sgpu_ctx *ctx, const double *cell, const int *nAtomv,
                                      const double *atom_pos, const double *cutoff,
                                      double ref_cutoff, int net_charge, double *b,
                                      double *b_ref, double *rho_at, double *rho_core,
                                      double *scalars);

/* Initial magnetization density of a collinear-spin run (spin_typ 1): the atoms' isolated-
 * atom densities weighted by atom_spin_z[atom] / Znucl (n_atom values, type-major as
 * atom_pos), accumulated over the same atom images as rho_at and not rescaled; atoms and
 * cutoff as for sgpu_Generate_PseudoChargeDensity. mag_at (Nd) is overwritten. Replaces the
 * magz part of Generate_PseudoChargeDensity (src/electrostatics.c:1031-1034), which
 * Init_electronDensity copies into mag (src/orbitalElecDensInit.c:149-151). */
int sgpu_Generate_InitialMagnetization(sgpu_ctx *ctx, const double *cell, const int *nAtomv,
                                       const double *atom_pos, const double *cutoff,
                                       const double *atom_spin_z, double *mag_at);

/* Build the nonlocal projectors of the atoms on the device (spline of UdV times real
 * spherical harmonics over the grid points of each image's rc-sphere) and install them as
 * sgpu_set_nonlocal would, together with the image coordinates for the k-point calls.
 * Replaces GetInfluencingAtoms_nloc and CalculateNonlocalProjectors
 * (src/nlocVecRoutines.c:43, :394). */
int sgpu_CalculateNonlocalProjectors(sgpu_ctx *ctx, const double *cell, const int *nAtomv,
                                     const double *atom_pos);

/* Parameters of a single-point SCF (SPARC_OBJ fields of the same meaning). */
typedef struct {
    int Nstates;                /* Nstates */
    int n_atom;                 /* for per-atom reporting only */
    double Nelectron;           /* Nelectron */
    double Beta;                /* 1 / smearing (Ha^-1) */
    int elec_T_type;            /* 0 Fermi-Dirac, 1 Gaussian */
    int cheb_degree;            /* ChebDegree */
    int rho_trigger;            /* rhoTrigger: filter passes in the first SCF iteration */
    int nchefsi;                /* Nchefsi */
    double tol_scf, tol_poisson, tol_precond, tol_lanczos;
    int maxit_scf, minit_scf, maxit_poisson;
    int mixing_history, pulay_freq, pulay_restart;
    double mixing_param, mixing_param_simple;
    int kerker;                 /* MixingPrecond == 1 */
    double kerker_kTF, kerker_idiemac;
    double xc_rhotol;
    double Esc;                 /* self and correction energy of the pseudocharges */
    int precision;              /* SGPU_PREC_FP64, or SGPU_PREC_FP32 for the mixed mode */
    double fp64_switch_error;   /* mixed mode: SCF error below which filtering becomes FP64
                                   (also left early when the FP32 error stops falling) */
    int graded_tail;            /* mixed mode after the switch: 0 = plain FP64 CheFSI; 1 = FP32
                                   filter whose last tail_fp64_degrees degrees run in FP64,
                                   with the Rayleigh-Ritz step in FP64 (sgpu_scf_kpt: complex64
                                   filter, complex128 Rayleigh-Ritz step and density) */
    int tail_fp64_degrees;      /* 0 .. cheb_degree-1 (graded_tail = 1; 0 for sgpu_scf_kpt) */
    unsigned long long seed;    /* initial orbitals and Lanczos start vector */
    int verbose;
    double *history;            /* optional host array of 3 * maxit_scf: per SCF iteration the
                                   free energy, the SCF error and the seconds since the call
                                   began (NULL: not recorded) */
    double *psi_out;            /* optional (host or device) Nd x Nstates: the final orbitals,
                                   as the force calculation uses them (NULL: not returned) */
    double *phi_out;            /* optional Nd: electrostatic potential of the final density */
    double *vxc_out;            /* optional Nd: exchange-correlation potential of the same
                                   (2 Nd, up then down, with collinear spin) */
    int spin_typ;               /* 0: spin-unpolarised; 1: collinear spin (sgpu_scf_kpt only) */
    const double *mag_init;     /* spin_typ 1: initial magnetization density, Nd (the
                                   reference's mag after Init_electronDensity) */
    double mixing_param_mag;    /* MixingParameterMag (<= 0: mixing_param) */
    double mixing_param_simple_mag; /* MixingParameterSimpleMag (<= 0: the value above) */
    double *mag_out;            /* optional Nd: the final (mixed) magnetization density */
} sgpu_scf_params;

typedef struct {
    int scf_iters, converged, fp64_switch_iter;
    double Etot, Eband, E1, E2, E3, Exc, Esc, Entropy, Efermi, scf_error;
    double time_s;              /* wall time of the SCF (without the optional field outputs) */
    double filter_ms;           /* device time of filter + projection products */
    double net_mag;             /* collinear spin: net magnetization of the last output
                                   density, sum(mag) dV (Bohr magneton) */
} sgpu_scf_result;

/* Single-point SCF for an orthogonal periodic Gamma-point cell, spin-unpolarised, LDA (PW92),
 * density mixing: the scf()/scf_loop() flow of src/electronicGroundState.c:607-1155 with
 * eigSolve_CheFSI, Calculate_occupation and Calculate_Free_Energy, on the context's grid and
 * nonlocal projectors. b: pseudocharge density (psdChrgDens), rho_init: initial density,
 * rho_core: model core density for the nonlinear core correction (NULL if none). Outputs the
 * final input density, Nstates eigenvalues and occupations (any may be NULL). */
int sgpu_scf(sgpu_ctx *ctx, const sgpu_scf_params *prm, const double *b,
             const double *rho_init, const double *rho_core, double *rho_out,
             double *lambda_out, double *occ_out, sgpu_scf_result *res);

/* The same SCF on a k-point grid with complex Bloch orbitals (eigSolve_CheFSI_kpt,
 * src/eigenSolverKpt.c:72-215; Lanczos_kpt bounds per k-point; the Fermi level, band energy,
 * entropy and density weighted by kptWts / Nkpts, src/occupation.c:445,
 * src/electronDensity.c:128, src/energy.c:221-255). kpts: nkpt Cartesian Bloch vectors
 * (1/Bohr, 3 per point, as k1_loc/k2_loc/k3_loc); kpt_wts: their weights as kptWts_loc
 * (normalised by their sum, which is Nkpts for a symmetry-reduced full grid). Needs the
 * k-point geometry of the context (sgpu_set_kpoint_geometry or
 * sgpu_CalculateNonlocalProjectors). Each filter pass runs all k-points through one batched
 * filter and then each k-point's Rayleigh-Ritz step (sgpu_CheFSI_batched). precision
 * SGPU_PREC_FP32 runs complex64 orbitals until the error falls below fp64_switch_error (or
 * stops falling), then complex128 orbitals, or with graded_tail = 1 a complex64 filter whose
 * output is widened for a complex128 Rayleigh-Ritz step and density (tail_fp64_degrees must
 * be 0). lambda_out and occ_out (nkpt * Nstates) are k-point after k-point;
 * psi_out, when set, receives nkpt blocks of Nd x Nstates complex128 (interleaved). */
int sgpu_scf_kpt(sgpu_ctx *ctx, const sgpu_scf_params *prm, int nkpt, const double *kpts,
                 const double *kpt_wts, const double *b, const double *rho_init,
                 const double *rho_core, double *rho_out, double *lambda_out, double *occ_out,
                 sgpu_scf_result *res);

/* ------------------------------------------------------------------- forces */

/* Local (pseudocharge) force components of the atoms at atom_pos (as for
 * sgpu_Generate_PseudoChargeDensity: type-major, nAtomv per type, cutoff 3 per type or NULL,
 * ref_cutoff REFERENCE_CUTOFF) from the electrostatic potential phi (Nd, host or device),
 * written to forces (host, 3 * n_atom, overwritten). Replaces Calculate_local_forces_linear
 * (src/forces.c:157). */
int sgpu_Calculate_local_forces(sgpu_ctx *ctx, const double *cell, const int *nAtomv,
                                const double *atom_pos, const double *cutoff, double ref_cutoff,
                                const double *phi, double *forces);

/* Nonlocal force components of the context's projector atoms from ncol orbitals X (Nd x ncol,
 * leading dimension ldi, host or device) with occupations occ (ncol) and occfac (2 without
 * spin), ADDED to forces (host, 3 * n_atom). Replaces Calculate_nonlocal_forces_linear and
 * its integrals (src/forces.c:750, :849, :890, :926). */
int sgpu_Calculate_nonlocal_forces(sgpu_ctx *ctx, int ncol, const double *X, int ldi,
                                   const double *occ, double occfac, const double *cell,
                                   double *forces);

/* Core-correction (NLCC) force components from the exchange-correlation potential Vxc (Nd,
 * host or device), written to forces_xc (host, 3 * n_atom, overwritten); atoms and cutoff as
 * for sgpu_Calculate_local_forces. Replaces Calculate_forces_xc_linear (src/forces.c:473). */
int sgpu_Calculate_forces_xc(sgpu_ctx *ctx, const double *cell, const int *nAtomv,
                             const double *atom_pos, const double *cutoff, const double *Vxc,
                             double *forces_xc);

/* Dx = d x / d(direction dir: 0 x, 1 y, 2 z) for ncol columns, periodic FD gradient of the
 * context's order (host or device arrays). Replaces Gradient_vectors_dir
 * (src/gradVecRoutines.c:33) for orthogonal cells. */
int sgpu_Gradient_vectors_dir(sgpu_ctx *ctx, int ncol, const double *cell, const double *x,
                              int ldi, double *Dx, int ldo, int dir);

/* Subtract the mean force from every atom (Symmetrize_forces, src/forces.c:1399). */
int sgpu_Symmetrize_forces(int n_atom, double *forces);

/* Device time of the last sgpu_ChebyshevFiltering call's filter loop, in milliseconds. */
int sgpu_last_filter_ms(sgpu_ctx *ctx, float *ms);

/* The context's CUDA stream (cudaStream_t), on which every call of this context runs, so that
 * a caller can order its own work or record timing events against it. The stream does not
 * synchronise with the legacy default stream: device arrays produced on another stream must
 * be complete (or ordered before this stream) when a call starts. Calls synchronise this
 * stream before they return. */
int sgpu_get_stream(sgpu_ctx *ctx, void **stream);

/* Read and clear the context's kernel status word (synchronises the stream). Kernels that
 * wait on barriers for their own asynchronous copies give every wait a time limit; a wait
 * that runs out sets a bit here (1: a stencil plane copy) and the kernel finishes without
 * hanging. *status = 0 means no wait ran out; otherwise the call returns
 * SGPU_ERR_KERNEL_WAIT. sgpu_scf and sgpu_autotune check the word themselves. */
int sgpu_kernel_status(sgpu_ctx *ctx, int *status);

/* Diagnostic of the bounded waits: one block waits, with a bound of 2e6 SM cycles (about a
 * millisecond), on a barrier phase that nothing completes. The wait runs out, sets bit 2 of
 * the status word and the block exits; this call returns that word in *status (2 when the
 * bound works) and leaves it cleared. No copy is in flight and nothing faults. */
int sgpu_check_wait_bound(sgpu_ctx *ctx, int *status);

/* Measures this GPU's FP64 FMA rate (TFLOP/s, an FMA counted as two flops) with one
 * arithmetic-only kernel timed by CUDA events on the context stream: the ceiling of the FP64
 * stencil and nonlocal kernels, which on this part are bound by the FP64 pipe rather than by
 * HBM. No counterpart in the reference (a measurement aid). */
int sgpu_measure_fp64_rate(sgpu_ctx *ctx, double *tflops);

/* ------------------------------------------------------ learned initial density */
/* No counterpart in the reference, which starts each SCF from the superposition of atomic
 * densities (Init_electronDensity, src/orbitalElecDensInit.c:145). A network trained on
 * converged densities predicts rho_SCF - rho_at per grid point from descriptors of the atomic
 * environment; the caller adds it to rho_at, clips at zero and restores the electron count. */

/* 24 descriptors per grid point (point-major, desc[p*24 + f], device memory): for 8 Gaussian
 * radial bins of width `width` centred on 0 .. rcut and a cosine cut-off at rcut, the sums
 * over atom images within rcut of g_b(r), |sum g_b(r) r/|r||^2 and sum_m (sum g_b(r) Y_2m)^2. */
int sgpu_density_descriptors(sgpu_ctx *ctx, const double *cell, int n_atom,
                             const double *atom_pos, double rcut, double width, float *desc);

/* Multilayer perceptron nin -> 3 hidden layers of `width` (SiLU) -> 1, FP32 master parameters
 * and Adam moments, BF16 weights in the forward and backward products, FP32 accumulation.
 * Parameter order: W1 (nin x width), b1, W2 (width x width), b2, W3, b3, w4 (width), b4. */
typedef struct sgpu_mlp sgpu_mlp;
int sgpu_mlp_create(int device, int nin, int width, unsigned long long seed, sgpu_mlp **net);
int sgpu_mlp_destroy(sgpu_mlp *net);
int sgpu_mlp_nparam(sgpu_mlp *net, long *nparam);
/* which: 0 parameters, 1 accumulated gradient (get only), 2 input shift, 3 input scale; the
 * network normalises its input as (x - shift) * scale. Host arrays. */
int sgpu_mlp_get(sgpu_mlp *net, int which, float *out);
int sgpu_mlp_set(sgpu_mlp *net, int which, const float *in);
/* y[n] = net(x[n x nin]) (device arrays) */
int sgpu_mlp_forward(sgpu_mlp *net, const float *x, long n, float *y);
/* loss = mean (net(x) - tscale*target)^2 over the n rows; adds d loss / d params to the
 * accumulated gradient */
int sgpu_mlp_loss_grad(sgpu_mlp *net, const float *x, const float *target, long n, float tscale,
                       double *loss);
int sgpu_mlp_zero_grad(sgpu_mlp *net);
int sgpu_mlp_adam_step(sgpu_mlp *net, float lr, float beta1, float beta2, float eps);

/* ------------------------------------------------------------------- kernel tuning */

/* Number of FP32 stencil kernel variants (tile shape, register blocking, plane ring). */
#define SGPU_STENCIL_VARIANTS 11

/* Time every FP32 stencil kernel variant (tile shape and register blocking) on ncol scratch
 * columns of this context's grid, keep the fastest for later calls, and return its index in
 * *variant and per-variant milliseconds in ms (SGPU_STENCIL_VARIANTS values; may be NULL).
 * All variants give identical results. sgpu_scf runs this once per context before its first
 * FP32 filter. No counterpart in the reference. */
int sgpu_autotune(sgpu_ctx *ctx, int ncol, int *variant, double *ms);

/* Fix the FP32 stencil variant (0 .. SGPU_STENCIL_VARIANTS-1) without timing. */
int sgpu_set_stencil_variant(sgpu_ctx *ctx, int variant);

/* Fix the form of the real nonlocal apply (0: one thread per covered point over all column
 * blocks; 1: alpha rows staged in shared memory per chunk of covered points; 2: as 0 with the
 * point's Chi values loaded once before the column loop; 3: FP32 only, a dense product per
 * chunk of covered points over the alpha rows of the chunk's atoms; 4: FP32 only, per range of
 * covered points with the output tile in shared memory); sgpu_autotune times all five.
 * Forms 0-2 give identical results; forms 3 and 4 sum in other (fixed) orders, so they agree
 * with 0-2 to FP32 rounding. */
int sgpu_set_nonlocal_apply_variant(sgpu_ctx *ctx, int variant);

/* Fix the form of the FP32 nonlocal projection (0: one block per segment of one image's
 * points; 1: one block per range of consecutive covered points, each x element read once);
 * sgpu_autotune times both. The two sum in different orders (and both add per-block
 * partial sums atomically), so results agree to FP32 rounding. */
int sgpu_set_nonlocal_project_variant(sgpu_ctx *ctx, int variant);

/* How the FP32-block Rayleigh-Ritz products (mixed SCF, sgpu_Project_Hamiltonian_f32,
 * sgpu_Subspace_Rotation_f32) are formed, all FP32-accurate with FP32 accumulation.
 * mode 0: cuBLAS FP32 GEMM with the BF16x9 tensor-core emulation requested, used where cuBLAS
 * expects a gain (its default strategy); mode 1: the same with the eager strategy (with
 * cuBLAS of CUDA 13.0 on GB300 both keep the FP32 SIMT GEMM for these shapes); mode 2: each
 * FP32 operand split into three BF16 parts and the product formed from six BF16 GEMMs on the
 * tensor cores (the part products of order <= 2, smallest first). */
int sgpu_set_gemm_emulation(sgpu_ctx *ctx, int mode);

/* Where the Rayleigh-Ritz products Mp = Yᵀ Y, Hp = Yᵀ HY (DP_Project_Hamiltonian,
 * src/eigenSolver.c:1022-1033) and X = Y Q (DP_Subspace_Rotation, :1415) run.
 * mode 1 (default): on the library's own tcgen05 kernels, every operand row scaled by a power of two
 * and cut into 7-bit BF16 slices whose products accumulate exactly in tensor memory (chunks
 * of 512) and are then summed in compensated arithmetic: FP32-accurate (3 slices, 6 slice
 * products) for FP32 blocks (sgpu_Project_Hamiltonian_f32, sgpu_Subspace_Rotation_f32, the
 * mixed SCF's FP32 phase) and FP64-accurate (6 slices, 21 products) for the mixed SCF's FP64
 * phase after the switch; plain FP64 calls (sgpu_Project_Hamiltonian,
 * sgpu_Subspace_Rotation, the plain FP64 SCF) keep cuBLAS DSYRK/DGEMM, the drop-in.
 * mode 2: the FP64-accurate tensor-core products for the plain FP64 calls too.
 * mode 0: cuBLAS everywhere (sgpu_set_gemm_emulation then picks the FP32-block form).
 * The Gram products compute the upper triangle and mirror it. No counterpart in the
 * reference (which calls cblas_dgemm). */
int sgpu_set_rr_products(sgpu_ctx *ctx, int mode);

/* complex64 stencil form: 1 (default) two x-neighbouring points per thread with packed reads
 * and a per-k table of Bloch factors (used where Nx and the leading dimensions are even and
 * the blocks 16-byte aligned); 0 the one-point-per-thread kernel. Both compute the same
 * operation sequence per point up to the rounding of the Bloch factors. */
int sgpu_set_zstencil_pairs(sgpu_ctx *ctx, int on);

/* Rayleigh-Ritz step of sgpu_CheFSI_batched / sgpu_scf_kpt: 1 (default) batches blocks of one
 * width and leading dimensions (batched ZGEMM / CGEMM products, batched Cholesky reduction,
 * one cusolverDnXsyevBatched call for all standard eigenproblems, batched back-substitution
 * and rotation); 0 one block at a time (ZGEMM / CGEMM and zhegvd per block). Both solve the
 * same generalized problems Hp q = lambda Mp q (zhegvd reduces them the same way). */
int sgpu_set_rr_batched(sgpu_ctx *ctx, int on);

/* How sgpu_Solve_Generalized_EigenProblem and the SCF solve Hp q = lambda Mp q
 * (DP_Solve_Generalized_EigenProblem, src/eigenSolver.c:1262; LAPACKE_dsygvd at :1318):
 * mode 0 (default): cuSOLVER dsygvd; 1: the same reduction as separate calls (dpotrf, two
 * dtrsm, dsyevd, dtrsm); 2: the reduction with a Jacobi eigensolver (dsyevj). All FP64;
 * results agree to the eigensolvers' accuracy. */
int sgpu_set_eig_solver(sgpu_ctx *ctx, int mode);

/* FP32 filter with the projections carried across degrees (mode 1, 2, 3 or 4) or not (0).
 * When on, every degree's nonlocal apply is the range form with the projection of the iterate
 * it finishes fused in (alpha of the next degree is formed from the finished values while
 * they are on chip), so a filter of degree m launches one projection instead of m. The fused
 * kernel has three forms: on the CUDA cores with 2 or 4 columns per thread (mode 2 or 4; the
 * apply results bit-identical to form 4), and on the tensor cores (mode 3: per range of at
 * most 128 covered points and 64 projector rows, the apply and the projection as tcgen05
 * products of three-slice BF16 splits, FP32-accurate, accumulated in FP32); mode 1 keeps the
 * current form. The projections agree with the separate ones to FP32 rounding. Needs the
 * range tables of FP32 projector sets; mode 3 also the tensor-core tables (built unless a
 * covered point needs more than 64 rows: SGPU_ERR_STATE then; a later sgpu_set_nonlocal whose
 * set has none returns the fused form to 2 columns per thread). sgpu_autotune times every form
 * and turns fusion on when the fastest beats the fastest separate apply plus projection. */
int sgpu_set_nonlocal_fuse(sgpu_ctx *ctx, int mode);

/* Whether the tensor-core fused form is available for the installed projector set
 * (*available 0/1) and its last tuned time of one launch (*tc_ms, 0 before tuning); either
 * pointer may be NULL. */
int sgpu_get_nonlocal_fuse_tc(sgpu_ctx *ctx, int *available, double *tc_ms);

/* The fused form in use (*mode: 0 off, 2 or 4 columns per thread, 3 tensor cores) and the last tuned
 * times of one fused launch of each form (fused_ms[2]: 2 and 4 columns, 0 before tuning);
 * either pointer may be NULL. */
int sgpu_get_nonlocal_fuse(sgpu_ctx *ctx, int *mode, double *fused_ms);

/* The kernel forms in use (set by sgpu_autotune or the sgpu_set_*_variant calls); any
 * pointer may be NULL. */
int sgpu_get_variants(sgpu_ctx *ctx, int *stencil, int *nl_apply, int *nl_project);

/* Milliseconds per launch that the last sgpu_autotune measured for the five nonlocal apply
 * forms (apply_ms[5]) and the two FP32 projection forms (project_ms[2]); zeros before any
 * tuning or without projectors. Either pointer may be NULL. */
int sgpu_get_tuning(sgpu_ctx *ctx, double *apply_ms, double *project_ms);

/* ------------------------------------------------------------------- measurement */

/* kernel kinds reported by sgpu_profile_read */
enum {
    SGPU_KERNEL_STENCIL = 0,    /* fused stencil + potential + Chebyshev update */
    SGPU_KERNEL_NL_PROJECT = 1, /* nonlocal projection alpha = Chiᵀ x */
    SGPU_KERNEL_NL_APPLY = 2,   /* nonlocal owner-computes apply */
    SGPU_KERNEL_OTHER = 3,      /* everything else (conversions, reductions, ...) */
    SGPU_KERNEL_KINDS = 4
};

/* Turn per-kernel timing on (1) or off (0); either call resets the counters. While on, the
 * library records a CUDA event pair on its stream around every launch of the kinds above.
 * No counterpart in the reference (which times phases with MPI_Wtime under DEBUG). */
int sgpu_profile_enable(sgpu_ctx *ctx, int on);

/* Accumulated device time (ms) and launch count of one kernel kind since the last reset;
 * kind == SGPU_KERNEL_KINDS returns the total number of kernels launched (time = 0). */
int sgpu_profile_read(sgpu_ctx *ctx, int kind, double *total_ms, long *launches);

#ifdef __cplusplus
}
#endif

#endif
