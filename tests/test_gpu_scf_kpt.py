"""GPU parity of the k-point SCF (sgpu_scf_kpt) against the reference program's own runs:
the Si2 box with a 3x3x3 k-point grid (14 symmetry-reduced k-points) and, with collinear spin,
the Al4 FCC cell with a 2x2x2 grid from seeded +-0.2 moments. tests/golden/<name>_scf.npz
holds the reference's set-up, k-points and weights (and for Al4 the spin start, the
reference's spin Vxc and a spin mixing sequence), <name>_scf_ref.json its converged result;
both are made by tests/golden/make_golden.py --only scf_kpt.
Tolerances: free energy 1e-5 Ha/atom, Fermi level 1e-4 Ha, occupied eigenvalues of every
k-point 1e-5 Ha (the SCF's parity bars), electron count 1e-8."""
import numpy as np
import pytest

import sparc_gb300 as sg
from scf_io import load_scf, scf_params

pytestmark = pytest.mark.gpu


def make_kctx(d, grid, nl):
    ctx = sg.Context(grid["Nx"], grid["Ny"], grid["Nz"], grid["FDn"], grid["cx"], grid["cy"],
                     grid["cz"], grid["dV"])
    ctx.set_nonlocal(nl["ip_displ"], nl["gamma"], nl["img_atom"], nl["img_ndc"],
                     nl["grid_pos"], nl["chi"])
    ctx.set_kpoint_geometry(d["L"], d["img_coords"])
    return ctx


@pytest.mark.parametrize("precision,graded", [(64, 0), (32, 0), (32, 1)])
def test_scf_kpt_matches_reference_program(gpu_available, precision, graded):
    """graded: after the switch the filter stays complex64 and the Rayleigh-Ritz step and the
    density run in complex128."""
    d, grid, nl, ref = load_scf("Si2_kpt")
    ctx = make_kctx(d, grid, nl)
    prm = scf_params(sg, d, ref, precision=precision, switch=1e-4)
    prm.graded_tail = graded
    res, rho, lam, occ = ctx.scf_kpt(prm, d["kpts"], d["kpt_wts"], d["b"], d["rho0"],
                                     d["rho_core"])
    n_atom = int(d["n_atom"])
    nk, Ns = d["kpts"].shape[0], int(d["Nstates"])
    assert res["converged"] == 1
    assert abs(res["Etot"] / n_atom - ref["Etot_per_atom"]) < 1e-5
    assert abs(res["Efermi"] - ref["Efermi"]) < 1e-4
    assert abs(res["Eband"] - ref["Eband"]) < 1e-4
    lam_ref = np.array(ref["lambda"]).reshape(nk, Ns)
    occ_ref = np.array(ref["occ"]).reshape(nk, Ns)
    occupied = occ_ref > 1e-3
    assert np.abs(lam[occupied] - lam_ref[occupied]).max() < 1e-5
    assert np.abs(2.0 * occ - occ_ref).max() < 2e-3  # the reference prints occfac * occ
    assert abs(rho.sum() * grid["dV"] - float(d["Nelectron"])) < 1e-8
    assert abs(res["scf_iters"] - ref["scf_iters"]) <= (1 if precision == 64 else 2)
    if precision == 32:
        assert res["fp64_switch_iter"] > 0


def test_scf_kpt_gamma_only_grid_matches_gamma_scf(gpu_available):
    """A one-point grid at k = 0 is the Gamma-point SCF with complex orbitals: same energy and
    eigenvalues as sgpu_scf on the same system."""
    d, grid, nl, ref = load_scf("Si2_kpt")
    ctx = make_kctx(d, grid, nl)
    prm = scf_params(sg, d, ref, precision=64, switch=1e-4)
    prm.tol_scf = 1e-8
    res_k, _, lam_k, _ = ctx.scf_kpt(prm, np.zeros((1, 3)), np.ones(1), d["b"], d["rho0"],
                                     d["rho_core"])
    ctx2 = make_kctx(d, grid, nl)
    prm2 = scf_params(sg, d, ref, precision=64, switch=1e-4)
    prm2.tol_scf = 1e-8
    res_g, _, lam_g, occ_g = ctx2.scf(prm2, d["b"], d["rho0"], d["rho_core"])
    assert res_k["converged"] == 1 and res_g["converged"] == 1
    assert abs(res_k["Etot"] - res_g["Etot"]) < 1e-7
    occupied = occ_g > 1e-3
    assert np.abs(lam_k[0][occupied] - lam_g[occupied]).max() < 1e-6


def test_scf_kpt_rejects_bad_input(gpu_available):
    d, grid, nl, ref = load_scf("Si2_kpt")
    ctx = make_kctx(d, grid, nl)
    prm = scf_params(sg, d, ref, precision=64)
    with pytest.raises(sg.SgpuError):  # weights must be positive
        ctx.scf_kpt(prm, d["kpts"], -d["kpt_wts"], d["b"], d["rho0"], d["rho_core"])
    prm.graded_tail = 1
    prm.tail_fp64_degrees = 2
    with pytest.raises(sg.SgpuError):  # FP64 filter degrees in the tail: Gamma-point only
        ctx.scf_kpt(prm, d["kpts"], d["kpt_wts"], d["b"], d["rho0"], d["rho_core"])
    ctx3 = sg.Context(grid["Nx"], grid["Ny"], grid["Nz"], grid["FDn"], grid["cx"], grid["cy"],
                      grid["cz"], grid["dV"])
    prm.graded_tail = 0
    with pytest.raises(sg.SgpuError):  # no k-point geometry installed
        ctx3.scf_kpt(prm, d["kpts"], d["kpt_wts"], d["b"], d["rho0"], d["rho_core"])


def test_lsda_matches_reference(gpu_available):
    d, grid, nl, ref = load_scf("Al4_spin_kpt")
    ctx = make_kctx(d, grid, nl)
    rho3 = d["rho3_0"]
    vxc = np.zeros((2, ctx.Nd))
    exc = np.zeros(ctx.Nd)
    ctx.Calculate_Vxc_LSDA_PW(rho3[1], rho3[2], d["rho_core"], ref["params"]["xc_rhotol"], vxc,
                              exc)
    assert np.abs(vxc - d["vxc0_spin"]).max() <= 1e-12 * np.abs(d["vxc0_spin"]).max()
    assert np.abs(exc - d["exc0_spin"]).max() <= 1e-12 * np.abs(d["exc0_spin"]).max()


def test_spin_mixing_matches_reference(gpu_available):
    """Device [rho, magz] mixing against the reference's Mixing_periodic_pulay over nine
    iterations (past the history of seven)."""
    d, grid, nl, ref = load_scf("Al4_spin_kpt")
    p = ref["params"]
    ctx = make_kctx(d, grid, nl)
    ctx.Mixing_init_spin(d["rho3_0"][0], d["mag0"], -float(d["Nelectron"]),
                         history=int(p["MixingHistory"]), mixing_parameter=p["MixingParameter"],
                         mixing_parameter_simple=p["MixingParameterSimple"],
                         mixing_parameter_mag=p["MixingParameterMag"],
                         mixing_parameter_simple_mag=p["MixingParameterSimpleMag"],
                         kerker=int(p["MixingPrecond"] == 1), kTF=p["precond_kerker_kTF"],
                         idiemac=p["precond_kerker_thresh"], tol_precond=p["TOL_PRECOND"])
    for it, (g, gm) in enumerate(zip(d["mix_outputs"], d["mix_mag_outputs"])):
        r, m = ctx.Mixing_periodic_pulay_spin(it, g.copy(), gm.copy())
        assert np.abs(r - d["mix_rho"][it]).max() <= 1e-10 * np.abs(d["mix_rho"][it]).max(), it
        assert np.abs(m - d["mix_mag"][it]).max() <= 1e-10 * np.abs(d["mix_mag"][it]).max(), it
    with pytest.raises(sg.SgpuError):  # the unpolarised entry point refuses a spin history
        ctx.Mixing_periodic_pulay(9, d["mix_outputs"][0].copy())


@pytest.mark.parametrize("precision,graded", [(64, 0), (32, 0), (32, 1)])
def test_spin_scf_kpt_matches_reference_program(gpu_available, precision, graded):
    """Collinear-spin k-point SCF (Al4, 4 k-points x 2 spins = 8 blocks) against the
    reference program: free energy, Fermi level, occupied eigenvalues of every (spin, k)
    block, net magnetization (graded: complex64 filter with a complex128 Rayleigh-Ritz step
    after the switch)."""
    d, grid, nl, ref = load_scf("Al4_spin_kpt")
    p = ref["params"]
    ctx = make_kctx(d, grid, nl)
    prm = scf_params(sg, d, ref, precision=precision, switch=1e-4)
    prm.graded_tail = graded
    prm.mixing_param_mag = p["MixingParameterMag"]
    prm.mixing_param_simple_mag = p["MixingParameterSimpleMag"]
    fields = {}
    res, rho, lam, occ = ctx.scf_kpt(prm, d["kpts"], d["kpt_wts"], d["b"], d["rho3_0"][0],
                                     d["rho_core"], fields=fields, mag_init=d["mag0"])
    n_atom = int(d["n_atom"])
    nk, Ns = d["kpts"].shape[0], int(d["Nstates"])
    assert res["converged"] == 1
    assert abs(res["Etot"] / n_atom - ref["Etot_per_atom"]) < 1e-5
    assert abs(res["Efermi"] - ref["Efermi"]) < 1e-4
    lam_ref = np.array(ref["lambda"]).reshape(2 * nk, Ns)
    occ_ref = np.array(ref["occ"]).reshape(2 * nk, Ns)   # printed as occ / 2 with spin
    occupied = occ_ref > 1e-3
    assert np.abs(lam[occupied] - lam_ref[occupied]).max() < 1e-5
    assert np.abs(0.5 * occ - occ_ref).max() < 2e-3
    assert abs(res["net_mag"] - ref["net_mag"]) < 1e-3
    assert abs(fields["mag"].sum() * grid["dV"] - ref["net_mag"]) < 1e-3
    assert abs(rho.sum() * grid["dV"] - float(d["Nelectron"])) < 1e-8
    assert abs(res["scf_iters"] - ref["scf_iters"]) <= (1 if precision == 64 else 2)


def test_own_setup_spin_scf_matches_reference_program(gpu_available):
    """Al4 collinear spin from the library's own set-up (psp8 tables -> pseudocharges, atomic
    and core densities, projectors, the initial magnetization of the seeded moments) through
    sgpu_scf_kpt, against the reference program's run and its initial fields."""
    import os
    import sys
    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, golden)
    import systems
    from sparc_gb300.psp8 import load_tables
    from sparc_gb300.setup import CellSystem
    d, grid, nl, ref = load_scf("Al4_spin_kpt")
    sysd = systems.al4_spin_kpt()
    N = (grid["Nx"], grid["Ny"], grid["Nz"])
    cs = CellSystem(sysd["L"], N, sysd["species"],
                    {"Al": load_tables(os.path.join(golden, "psp_Al.npz"))})
    spins = sysd["spins"]["Al"]
    mag = cs.initial_magnetization(spins)
    assert np.abs(mag - d["mag0"]).max() <= 1e-10 * np.abs(d["mag0"]).max()
    assert np.abs(cs.fields["rho_at"] - d["rho3_0"][0]).max() <= 1e-10 * d["rho3_0"][0].max()
    p = ref["params"]
    prm = cs.scf_params(Nstates=int(d["Nstates"]), cheb_degree=int(p["ChebDegree"]),
                        smearing=1.0 / p["Beta"])
    res, rho, lam, occ = cs.scf_kpt(prm, d["kpts"], d["kpt_wts"], atom_spin_z=spins)
    assert res["converged"] == 1
    assert abs(res["Etot"] / cs.n_atom - ref["Etot_per_atom"]) < 1e-5
    nk, Ns = d["kpts"].shape[0], int(d["Nstates"])
    lam_ref = np.array(ref["lambda"]).reshape(2 * nk, Ns)
    occupied = np.array(ref["occ"]).reshape(2 * nk, Ns) > 1e-3
    assert np.abs(lam[occupied] - lam_ref[occupied]).max() < 1e-5
    assert abs(res["net_mag"] - ref["net_mag"]) < 1e-3
    cs.close()
