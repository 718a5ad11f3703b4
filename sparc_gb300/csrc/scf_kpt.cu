// k-point CheFSI SCF on the device (complex Bloch orbitals, LDA, without spin or with
// collinear spin).
//
// Restates the reference's single-point SCF on a k-point grid for an orthogonal periodic cell:
//   eigSolve_CheFSI_kpt / CheFSI_kpt   src/eigenSolverKpt.c:72-215 / :224-345
//   Chebyshevfilter_constants_kpt      src/eigenSolverKpt.c:351-450 (Lanczos_kpt :1361)
//   Calculate_occupation with k weights src/occupation.c:43, local_occ_constraint :445-466
//   CalculateDensity_psi               src/electronDensity.c:104-160
//   Calculate_Eband / electronic entropy src/energy.c:205-262
// and, as in the Gamma-point driver, the potential (Poisson, LDA), mixing and energy terms of
// scf / scf_loop (src/electronicGroundState.c:607-1155). With collinear spin (spin_typ 1)
// every (spin, k) pair is a block with its own local potential phi + Vxc_s (LSDA,
// Calculate_Vxc, src/exchangeCorrelation.c:227-347), occfac is 1, the output density is
// [total, up, down] with magnetization up - down (Calculate_elecDens,
// src/electronDensity.c:28-80), the SCF error runs over [up, down]
// (src/electronicGroundState.c:1160), E3 pairs each spin density with its potential
// (src/energy.c:97-99), and the mixed vector is [total, magz] (src/mixing.c:250-258).
//
// Each filter pass runs the k-points as one batched complex filter (one CUDA graph for all
// k-points and degrees) followed by each k-point's Rayleigh-Ritz step (chefsi_batched); the
// reference filters its k-points one after another. Mixed precision (SGPU_PREC_FP32) keeps
// complex64 orbitals with complex64 projection / rotation products and the complex128
// eigensolve while the SCF error is above fp64_switch_error, then widens them to complex128;
// with graded_tail the filter stays complex64 after the switch and only the Rayleigh-Ritz step
// (H Y, projection, eigensolve, rotation) and the density run on complex128 copies, as in the
// Gamma-point driver's graded tail.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "sgpu_internal.h"

using namespace sgpu;

namespace {

int scf_kpt_check(sgpu_ctx *ctx, const sgpu_scf_params *prm, int nkpt, const double *kpts,
                  const double *wts, const double *b, const double *rho_init,
                  const sgpu_scf_result *res)
{
    if (!ctx || !prm || !b || !rho_init || !res || !kpts || !wts) {
        set_error("sgpu_scf_kpt: null argument");
        return SGPU_ERR_ARG;
    }
    SGPU_CUDA_TRY(cudaSetDevice(ctx->device));
    if (!ctx->kp) {
        set_error("sgpu_scf_kpt: sgpu_set_kpoint_geometry (or sgpu_CalculateNonlocalProjectors) "
                  "has not been called");
        return SGPU_ERR_STATE;
    }
    if (nkpt < 1) {
        set_error("sgpu_scf_kpt: need nkpt >= 1");
        return SGPU_ERR_ARG;
    }
    for (int k = 0; k < nkpt; k++) {
        if (!(wts[k] > 0.0)) {
            set_error("sgpu_scf_kpt: k-point weights must be positive");
            return SGPU_ERR_ARG;
        }
    }
    if (prm->Nstates <= 0 || prm->cheb_degree < 1) {
        set_error("sgpu_scf_kpt: need Nstates > 0 and a Chebyshev degree >= 1");
        return SGPU_ERR_ARG;
    }
    if (prm->precision != SGPU_PREC_FP64 && prm->precision != SGPU_PREC_FP32) {
        set_error("sgpu_scf_kpt: precision must be SGPU_PREC_FP64 or SGPU_PREC_FP32");
        return SGPU_ERR_ARG;
    }
    if (prm->graded_tail != 0 && prm->graded_tail != 1) {
        set_error("sgpu_scf_kpt: graded_tail must be 0 or 1");
        return SGPU_ERR_ARG;
    }
    if (prm->graded_tail && prm->tail_fp64_degrees != 0) {
        set_error("sgpu_scf_kpt: FP64 filter degrees in the graded tail are a Gamma-point "
                  "option; set tail_fp64_degrees to 0");
        return SGPU_ERR_ARG;
    }
    if (prm->spin_typ != 0 && prm->spin_typ != 1) {
        set_error("sgpu_scf_kpt: spin_typ must be 0 (unpolarised) or 1 (collinear)");
        return SGPU_ERR_ARG;
    }
    if (prm->spin_typ == 1 && !prm->mag_init) {
        set_error("sgpu_scf_kpt: collinear spin needs the initial magnetization mag_init");
        return SGPU_ERR_ARG;
    }
    return SGPU_OK;
}

struct DevFree {
    void *p = nullptr;
    ~DevFree() { if (p) cudaFree(p); }
};

}  // namespace

extern "C" {

int sgpu_scf_kpt(sgpu_ctx *ctx, const sgpu_scf_params *prm, int nkpt, const double *kpts,
                 const double *kpt_wts, const double *b, const double *rho_init,
                 const double *rho_core, double *rho_out, double *lambda_out, double *occ_out,
                 sgpu_scf_result *res)
{
    SGPU_TRY(scf_kpt_check(ctx, prm, nkpt, kpts, kpt_wts, b, rho_init, res));
    auto t0 = std::chrono::steady_clock::now();
    cudaStream_t st = ctx->stream;
    const int Ns = prm->Nstates;
    const long N = ctx->Nd;
    const long nb = N * (long)Ns;   // complex values per block
    const int m = prm->cheb_degree;
    const bool spin = prm->spin_typ == 1;
    const int nspin = spin ? 2 : 1;
    const int nblk = nspin * nkpt;  // block b = s * nkpt + k, as the reference's lambda layout

    // k weights as the reference keeps them (kptWts_loc); their sum is the grid's Nkpts
    double wsum = 0.0;
    for (int k = 0; k < nkpt; k++) wsum += kpt_wts[k];
    std::vector<double> wk(nkpt);
    for (int k = 0; k < nkpt; k++) wk[k] = kpt_wts[k] / wsum;

    // persistent device vectors: in3 / out3 = [total, up, down] input and output densities
    // (only the total without spin), g = the mixed vector ([total, magz] with spin)
    DevFree gv;
    SGPU_CUDA_TRY(cudaMalloc(&gv.p, sizeof(double) * ((size_t)N * 16 + (size_t)nblk * Ns) + 256));
    double *vec = static_cast<double *>(gv.p);
    double *d_b = vec, *d_core = vec + N, *d_phi = vec + 2 * N, *d_exc = vec + 3 * N;
    double *d_in3 = vec + 4 * N, *d_out3 = vec + 7 * N, *d_g = vec + 10 * N;
    double *d_vxc = vec + 12 * N, *d_veff = vec + 14 * N, *d_w = vec + 16 * N;
    SGPU_CUDA_TRY(cudaMemcpyAsync(d_b, b, sizeof(double) * N, cudaMemcpyDefault, st));
    if (rho_core)
        SGPU_CUDA_TRY(cudaMemcpyAsync(d_core, rho_core, sizeof(double) * N, cudaMemcpyDefault, st));
    SGPU_CUDA_TRY(cudaMemcpyAsync(d_in3, rho_init, sizeof(double) * N, cudaMemcpyDefault, st));
    SGPU_CUDA_TRY(cudaMemsetAsync(d_phi, 0, sizeof(double) * N, st));
    const double *core = rho_core ? d_core : nullptr;
    // the mixed vector's initial value, and the spin densities (Calculate_diagonal_Density)
    SGPU_CUDA_TRY(cudaMemcpyAsync(d_g, d_in3, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
    auto split_spin = [&](const double *tot, const double *mag, double *up, double *dn) -> int {
        SGPU_TRY(axpby_dev(ctx, N, 0.5, tot, 0.5, mag, up, st));
        SGPU_TRY(axpby_dev(ctx, N, 0.5, tot, -0.5, mag, dn, st));
        return SGPU_OK;
    };
    if (spin) {
        SGPU_CUDA_TRY(cudaMemcpyAsync(d_g + N, prm->mag_init, sizeof(double) * N,
                                      cudaMemcpyDefault, st));
        SGPU_TRY(split_spin(d_in3, d_g + N, d_in3 + N, d_in3 + 2 * N));
    }

    // orbital blocks: complex128 X, Y; complex64 pair in mixed mode
    bool mixed = prm->precision == SGPU_PREC_FP32;
    DevFree g64, g32;
    const long ncplx = nb * nblk;
    SGPU_CUDA_TRY(cudaMalloc(&g64.p, sizeof(double2) * (size_t)ncplx * 2));
    double2 *X64 = static_cast<double2 *>(g64.p), *Y64 = X64 + ncplx;
    float2 *X32 = nullptr, *Y32 = nullptr;
    if (mixed) {
        SGPU_CUDA_TRY(cudaMalloc(&g32.p, sizeof(float2) * (size_t)ncplx * 2));
        X32 = static_cast<float2 *>(g32.p);
        Y32 = X32 + ncplx;
    }
    // random start (SetRandMat_complex's role): uniform real and imaginary parts per block
    for (int bk = 0; bk < nblk; bk++)
        init_orbitals(ctx, reinterpret_cast<double *>(X64 + nb * bk), 2 * nb,
                      prm->seed + 0x632BE59BD9B4E019ull * (unsigned long long)(bk + 1), 152 * 8, st);
    if (mixed)
        SGPU_TRY(convert_cols<double, float>(reinterpret_cast<double *>(X64), 2 * ncplx,
                                             reinterpret_cast<float *>(X32), 2 * ncplx,
                                             2 * ncplx, 1, st));

    const double occfac = spin ? 1.0 : 2.0;  // 2 / Nspinor
    int pits = 0;
    // potential of the input density in3: phi, Vxc (per spin), Veff_s = phi + Vxc_s
    auto potential = [&]() -> int {
        SGPU_TRY(poisson_dev(ctx, d_in3, d_b, d_phi, prm->tol_poisson, prm->maxit_poisson, &pits, st));
        if (spin)
            SGPU_TRY(lsda_pw_dev(ctx, d_in3 + N, d_in3 + 2 * N, core, prm->xc_rhotol, d_vxc,
                                 d_vxc + N, d_exc, st));
        else
            SGPU_TRY(lda_pw_dev(ctx, d_in3, core, prm->xc_rhotol, d_vxc, d_exc, st));
        for (int sp = 0; sp < nspin; sp++)
            SGPU_TRY(axpby_dev(ctx, N, 1.0, d_phi, 1.0, d_vxc + sp * N, d_veff + sp * N, st));
        SGPU_TRY(sgpu_set_veff(ctx, nspin, d_veff));
        return SGPU_OK;
    };
    SGPU_TRY(potential());
    MixParams mp;
    mp.m = prm->mixing_history;
    mp.pulay_freq = std::max(1, prm->pulay_freq);
    mp.restart = prm->pulay_restart;
    mp.beta = prm->mixing_param;
    mp.omega = prm->mixing_param_simple;
    mp.kerker = prm->kerker;
    mp.kTF = prm->kerker_kTF;
    mp.idiemac = prm->kerker_idiemac;
    mp.precond_tol = prm->tol_precond;
    mp.neg_charge = -prm->Nelectron;
    mp.nspden = nspin;
    // the reference's defaults: MixingParameterMag = MixingParameter, the simple-mixing one
    // = MixingParameterMag (src/initialization.c:2275-2283)
    mp.beta_mag = prm->mixing_param_mag > 0.0 ? prm->mixing_param_mag : prm->mixing_param;
    mp.omega_mag = prm->mixing_param_simple_mag > 0.0 ? prm->mixing_param_simple_mag : mp.beta_mag;
    SGPU_TRY(mixing_init(ctx, mp, d_g));

    // per-block occupation weights for the Fermi level: occfac * kptWts / Nkpts
    std::vector<double> wocc((size_t)nblk * Ns);
    for (int bk = 0; bk < nblk; bk++)
        for (int n = 0; n < Ns; n++) wocc[(size_t)bk * Ns + n] = occfac * wk[bk % nkpt];
    std::vector<double> lam((size_t)nblk * Ns, 0.0), occ((size_t)nblk * Ns, 0.0);
    std::vector<double> eigmin(nblk, 0.0), eigmax(nblk, 0.0);
    std::vector<sgpu_filter_block> blk(nblk), blk64(nblk);
    bool graded = false;  // after the switch with graded_tail: complex64 filter, complex128 RR
    double efermi = 0.0, error = prm->tol_scf + 1.0, net_mag = 0.0;
    double Etot = 0, Eband = 0, E1 = 0, E2 = 0, E3 = 0, Exc = 0, Entropy = 0;
    int scf = 0, switch_iter = mixed ? -1 : 0;
    double best_error = 1e300;
    int stall = 0;
    double filter_ms = 0.0;
    while (scf < prm->maxit_scf) {
        // ---- eigSolve_CheFSI_kpt
        int count = scf == 0 ? 0 : prm->rho_trigger + (scf - 1) * prm->nchefsi;
        const int cend = prm->rho_trigger + scf * prm->nchefsi;
        for (; count < cend; count++) {
            for (int bk = 0; bk < nblk; bk++) {
                const int sp = bk / nkpt, k = bk % nkpt;
                const double *kv = kpts + 3 * k;
                double cutoff;
                if (count == 0) {
                    // Lanczos_kpt on H_(s,k) from one complex random start vector shared by
                    // the blocks, then the reference's margins (src/eigenSolverKpt.c:385-408)
                    double *x0 = nullptr;
                    SGPU_TRY(ws_get(ctx, WS_SCF, sizeof(double) * 2 * N, (void **)&x0));
                    init_orbitals(ctx, x0, 2 * N, prm->seed ^ 0x5bd1e995ull, 152, st);
                    SGPU_TRY(kpoint_set_phases(ctx, kv, st));
                    auto apply = [&](const double *in, double *out) {
                        return hamiltonian_z<double2>(
                            ctx, sp, kv, 1, 0.0, reinterpret_cast<const double2 *>(in), N,
                            reinterpret_cast<double2 *>(out), N, 1.0, 0.0, nullptr, 0, st);
                    };
                    SGPU_TRY(lanczos_run(ctx, 2 * N, apply, x0, prm->tol_lanczos, 1000,
                                         &eigmin[bk], &eigmax[bk], st));
                    eigmax[bk] *= 1.01;
                    eigmin[bk] -= 0.1;
                    cutoff = 0.5 * (eigmin[bk] + eigmax[bk]);
                } else {
                    if (count >= prm->rho_trigger) eigmin[bk] = lam[(size_t)bk * Ns];
                    cutoff = lam[(size_t)bk * Ns + Ns - 1] + 0.1;
                }
                sgpu_filter_block &f = blk[bk];
                f.spin = sp;
                f.k[0] = kv[0]; f.k[1] = kv[1]; f.k[2] = kv[2];
                const bool c64 = mixed || graded;  // the filter runs on complex64 blocks
                f.X = c64 ? (void *)(X32 + nb * bk) : (void *)(X64 + nb * bk);
                f.Y = c64 ? (void *)(Y32 + nb * bk) : (void *)(Y64 + nb * bk);
                f.ldi = f.ldo = (int)N;
                f.ncol = Ns;
                f.a = cutoff;
                f.b = eigmax[bk];
                f.a0 = eigmin[bk];
                if (!(f.b > f.a) || !(f.a > f.a0)) {
                    set_error("sgpu_scf_kpt: filter bounds out of order in block " +
                              std::to_string(bk));
                    return SGPU_ERR_LINALG;
                }
            }
            SGPU_CUDA_TRY(cudaEventRecord(ctx->ev0, st));
            if (graded) {
                for (int bk = 0; bk < nblk; bk++) {
                    blk64[bk] = blk[bk];
                    blk64[bk].X = X64 + nb * bk;
                    blk64[bk].Y = Y64 + nb * bk;
                }
                SGPU_TRY(chefsi_batched_graded(ctx, nblk, blk.data(), blk64.data(), m,
                                               lam.data(), st));
            } else if (mixed) {
                SGPU_TRY(chefsi_batched<float2>(ctx, nblk, blk.data(), m, lam.data(), st));
            } else {
                SGPU_TRY(chefsi_batched<double2>(ctx, nblk, blk.data(), m, lam.data(), st));
            }
            SGPU_CUDA_TRY(cudaEventRecord(ctx->ev1, st));
            SGPU_CUDA_TRY(cudaEventSynchronize(ctx->ev1));
            float ms = 0.f;
            SGPU_CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
            filter_ms += ms;
            // ---- Fermi level over all blocks (bracket: src/eigenSolverKpt.c:126-145)
            double lo = lam[0], hi = lam[Ns - 1];
            for (int bk = 0; bk < nblk; bk++) {
                lo = std::min(lo, lam[(size_t)bk * Ns]);
                hi = std::max(hi, lam[(size_t)bk * Ns + Ns - 1]);
            }
            int fst = 0;
            efermi = fermi_level(lam, wocc, prm->Nelectron, prm->Beta, prm->elec_T_type,
                                 lo - 1.0, hi + 1.0, 1e-12, 100, &fst);
            if (fst) {
                set_error("sgpu_scf_kpt: cannot bracket the Fermi level");
                return SGPU_ERR_LINALG;
            }
            for (size_t i = 0; i < lam.size(); i++)
                occ[i] = smearing(prm->Beta, lam[i], efermi, prm->elec_T_type);
        }
        // ---- density: per spin, the sum over k-points and bands of
        //      occfac kptWts/Nkpts occ |psi|^2 / dV; with spin the total is up + down
        {
            std::vector<double> w((size_t)nblk * Ns);
            for (size_t i = 0; i < w.size(); i++) w[i] = wocc[i] * occ[i] / ctx->dV;
            SGPU_CUDA_TRY(cudaMemcpyAsync(d_w, w.data(), sizeof(double) * w.size(),
                                          cudaMemcpyHostToDevice, st));
            for (int bk = 0; bk < nblk; bk++) {
                const int sp = bk / nkpt, k = bk % nkpt;
                double *rho_s = spin ? d_out3 + (1 + sp) * N : d_out3;
                if (mixed)
                    SGPU_TRY(density_z_dev<float2>(ctx, X32 + nb * bk, N, Ns, d_w + (long)bk * Ns,
                                                   rho_s, k > 0, st));
                else
                    SGPU_TRY(density_z_dev<double2>(ctx, X64 + nb * bk, N, Ns, d_w + (long)bk * Ns,
                                                    rho_s, k > 0, st));
            }
            if (spin) {
                SGPU_TRY(axpby_dev(ctx, N, 1.0, d_out3 + N, 1.0, d_out3 + 2 * N, d_out3, st));
                SGPU_TRY(axpby_dev(ctx, N, 1.0, d_out3 + N, -1.0, d_out3 + 2 * N, d_g + N, st));
            }
            SGPU_CUDA_TRY(cudaMemcpyAsync(d_g, d_out3, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
            // the host weights must outlive the copy
            SGPU_CUDA_TRY(cudaStreamSynchronize(st));
        }
        // ---- energy with the input density (Calculate_Free_Energy)
        double sb = 0, s2 = 0, s3 = 0, sx = 0;
        SGPU_TRY(dot_host(ctx, d_b, d_phi, N, &sb, st));
        SGPU_TRY(dot_host(ctx, d_in3, d_phi, N, &s2, st));
        if (spin)  // [up, down] against [Vxc_up, Vxc_down]
            SGPU_TRY(dot_host(ctx, d_in3 + N, d_vxc, 2 * N, &s3, st));
        else
            SGPU_TRY(dot_host(ctx, d_in3, d_vxc, N, &s3, st));
        {
            double *rxc = nullptr;
            SGPU_TRY(ws_get(ctx, WS_RHS, sizeof(double) * N, (void **)&rxc));
            SGPU_TRY(axpby_dev(ctx, N, 1.0, d_in3, 1.0, core, rxc, st));
            SGPU_TRY(dot_host(ctx, rxc, d_exc, N, &sx, st));
        }
        E1 = 0.5 * sb * ctx->dV;
        E2 = 0.5 * s2 * ctx->dV;
        E3 = s3 * ctx->dV;
        Exc = sx * ctx->dV;
        Eband = 0.0;
        Entropy = 0.0;
        for (int bk = 0; bk < nblk; bk++) {
            double eb = 0.0, en = 0.0;
            for (int n = 0; n < Ns; n++) {
                const size_t i = (size_t)bk * Ns + n;
                eb += occfac * occ[i] * lam[i];
                const double g = occ[i];
                if (prm->elec_T_type == 0) {
                    if (g > 1e-14 && (1.0 - g) > 1e-14)
                        en += -(g * std::log(g) + (1.0 - g) * std::log(1.0 - g));
                } else {
                    const double x = prm->Beta * (lam[i] - efermi);
                    en += 0.5 / std::sqrt(M_PI) * std::exp(-x * x);
                }
            }
            Eband += wk[bk % nkpt] * eb;
            Entropy += wk[bk % nkpt] * en;
        }
        Entropy *= -occfac / prm->Beta;
        Etot = Eband + E1 - E2 - E3 + Exc + prm->Esc + Entropy;
        if (Etot != Etot) {
            set_error("sgpu_scf_kpt: total energy is NaN");
            return SGPU_ERR_NONFINITE;
        }
        // ---- SCF error (over [up, down] with spin), mixing, new potential
        if (spin) {
            SGPU_TRY(scf_error_dev(ctx, d_out3 + N, d_in3 + N, &error, st, 2 * N));
            double sm = 0.0;
            SGPU_TRY(dot_host(ctx, d_g + N, nullptr, N, &sm, st));
            net_mag = sm * ctx->dV;
        } else {
            SGPU_TRY(scf_error_dev(ctx, d_out3, d_in3, &error, st));
        }
        if (prm->history && scf < prm->maxit_scf) {
            prm->history[3 * scf] = Etot;
            prm->history[3 * scf + 1] = error;
            prm->history[3 * scf + 2] =
                std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        }
        SGPU_TRY(mixing_step(ctx, scf, d_g, st));
        SGPU_CUDA_TRY(cudaMemcpyAsync(d_in3, d_g, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
        if (spin) SGPU_TRY(split_spin(d_in3, d_g + N, d_in3 + N, d_in3 + 2 * N));
        SGPU_TRY(potential());
        scf++;
        if (prm->verbose)
            printf("sgpu_scf_kpt: iter %3d  Etot/atom %.10f  error %.3e  %s%s\n", scf,
                   Etot / std::max(1, prm->n_atom), error,
                   mixed ? "complex64" : graded ? "complex64 filter, complex128 Rayleigh-Ritz"
                                                : "complex128",
                   spin ? "  (collinear spin)" : "");
        if (error < prm->tol_scf && scf >= prm->minit_scf) break;
        if (mixed) {
            // the Gamma-point driver's switch rule: below the threshold, or once the
            // complex64 error has stopped falling
            stall = (scf >= 4 && error > 0.8 * best_error) ? stall + 1 : 0;
            best_error = std::min(best_error, error);
            if (error < prm->fp64_switch_error || stall >= 2) {
                SGPU_TRY(convert_cols<float, double>(reinterpret_cast<float *>(X32), 2 * ncplx,
                                                     reinterpret_cast<double *>(X64), 2 * ncplx,
                                                     2 * ncplx, 1, st));
                mixed = false;
                graded = prm->graded_tail == 1;  // X32 keeps the Ritz vectors for the filter
                switch_iter = scf;
            }
        }
    }
    if (rho_out) SGPU_CUDA_TRY(cudaMemcpyAsync(rho_out, d_in3, sizeof(double) * N, cudaMemcpyDefault, st));
    if (spin && prm->mag_out)
        SGPU_CUDA_TRY(cudaMemcpyAsync(prm->mag_out, d_g + N, sizeof(double) * N, cudaMemcpyDefault, st));
    SGPU_CUDA_TRY(cudaStreamSynchronize(st));
    const double t_scf = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (prm->psi_out) {
        if (mixed)
            SGPU_TRY(convert_cols<float, double>(reinterpret_cast<float *>(X32), 2 * ncplx,
                                                 reinterpret_cast<double *>(X64), 2 * ncplx,
                                                 2 * ncplx, 1, st));
        SGPU_CUDA_TRY(cudaMemcpyAsync(prm->psi_out, X64, sizeof(double2) * (size_t)ncplx,
                                      cudaMemcpyDefault, st));
    }
    if (prm->phi_out)
        SGPU_CUDA_TRY(cudaMemcpyAsync(prm->phi_out, d_phi, sizeof(double) * N, cudaMemcpyDefault, st));
    if (prm->vxc_out)
        SGPU_CUDA_TRY(cudaMemcpyAsync(prm->vxc_out, d_vxc, sizeof(double) * N * nspin,
                                      cudaMemcpyDefault, st));
    if (lambda_out) std::copy(lam.begin(), lam.end(), lambda_out);
    if (occ_out) std::copy(occ.begin(), occ.end(), occ_out);
    SGPU_CUDA_TRY(cudaStreamSynchronize(st));
    res->scf_iters = scf;
    res->converged = error < prm->tol_scf ? 1 : 0;
    res->Etot = Etot; res->Eband = Eband; res->E1 = E1; res->E2 = E2; res->E3 = E3;
    res->Exc = Exc; res->Esc = prm->Esc; res->Entropy = Entropy; res->Efermi = efermi;
    res->scf_error = error;
    res->fp64_switch_iter = switch_iter;
    res->filter_ms = filter_ms;
    res->time_s = t_scf;
    res->net_mag = net_mag;
    return kernel_status_check(ctx);
}

}  // extern "C"
