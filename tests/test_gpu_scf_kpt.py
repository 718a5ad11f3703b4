"""GPU parity of the k-point SCF (sgpu_scf_kpt) against the reference program's own run of the
Si2 box with a 3x3x3 k-point grid (14 symmetry-reduced k-points; tests/golden/Si2_kpt_scf.npz
holds the reference's set-up, k-points and weights, Si2_kpt_scf_ref.json its converged
result, both made by tests/golden/make_golden.py --only scf_kpt).
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


@pytest.mark.parametrize("precision", [64, 32])
def test_scf_kpt_matches_reference_program(gpu_available, precision):
    d, grid, nl, ref = load_scf("Si2_kpt")
    ctx = make_kctx(d, grid, nl)
    prm = scf_params(sg, d, ref, precision=precision, switch=1e-4)
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
    with pytest.raises(sg.SgpuError):  # the graded tail is a Gamma-point option
        ctx.scf_kpt(prm, d["kpts"], d["kpt_wts"], d["b"], d["rho0"], d["rho_core"])
    ctx3 = sg.Context(grid["Nx"], grid["Ny"], grid["Nz"], grid["FDn"], grid["cx"], grid["cy"],
                      grid["cz"], grid["dV"])
    prm.graded_tail = 0
    with pytest.raises(sg.SgpuError):  # no k-point geometry installed
        ctx3.scf_kpt(prm, d["kpts"], d["kpt_wts"], d["b"], d["rho0"], d["rho_core"])
