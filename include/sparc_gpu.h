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
    SGPU_ERR_NONFINITE = 7      /* NaN or Inf detected in an input or a result */
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

/* The same filter on FP32 blocks (host or device), for callers that keep the orbital block in
 * FP32 between filter calls (the mixed-precision SCF). No counterpart in the reference, which
 * filters in FP64 only; the recurrence scalars are the reference's, computed in FP64. */
int sgpu_ChebyshevFiltering_f32(sgpu_ctx *ctx, int spin, float *X, int ldi, float *Y, int ldo,
                                int ncol, int m, double a, double b, double a0);

/* r = b + (Lap + c*I) x for one grid vector. Replaces poisson_residual
 * (src/lapVecRoutines.c:69). */
int sgpu_poisson_residual(sgpu_ctx *ctx, double c, const double *x, const double *b,
                          double *r);

/* Device time of the last sgpu_ChebyshevFiltering call's filter loop, in milliseconds. */
int sgpu_last_filter_ms(sgpu_ctx *ctx, float *ms);

/* The context's CUDA stream (cudaStream_t), on which every call of this context runs, so that
 * a caller can order its own work or record timing events against it. */
int sgpu_get_stream(sgpu_ctx *ctx, void **stream);

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
