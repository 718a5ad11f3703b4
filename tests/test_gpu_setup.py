"""GPU parity of the per-geometry set-up against the reference's own set-up.

Fixtures tests/golden/<system>_setup.npz hold what the reference computed for the same input
(Calculate_PseudochargeCutoff, Generate_PseudoChargeDensity, Init_electronDensity,
GetInfluencingAtoms_nloc + CalculateNonlocalProjectors). Tolerances: cut-off radii exact to
rounding (1e-13 relative); grid fields 1e-11 of their largest magnitude (the device adds the
atoms' contributions in a different order); Esc and the integrated charges 1e-9 absolute;
projectors through Vnl applied to random vectors, 1e-12 relative. The full SCF from the
library's own set-up must reproduce the reference program's energy to 1e-5 Ha/atom.
"""
import json
import os
import sys

import numpy as np
import pytest

import sparc_gb300 as sg
from sparc_gb300.psp8 import load_tables
from sparc_gb300.setup import CellSystem

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import systems  # noqa: E402

SYSTEMS = ["Si2_small", "Si8_c1", "Al4_small"]


def load(system):
    f = np.load(os.path.join(GOLDEN, f"{system}_setup.npz"))
    d = {k: f[k] for k in f.files}
    tables = []
    for t in range(int(d["Ntypes"])):
        pre = f"t{t}_"
        tables.append({k[len(pre):]: v for k, v in d.items() if k.startswith(pre)})
    return d, tables


def ctx_for(d):
    return sg.Context(int(d["Nx"]), int(d["Ny"]), int(d["Nz"]), int(d["FDn"]), d["cx"], d["cy"],
                      d["cz"], float(d["dV"]))


def field_err(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("system", SYSTEMS)
def test_pseudocharge_cutoff(gpu_available, system):
    d, tables = load(system)
    ctx = ctx_for(d)
    ctx.set_psd(tables)
    cut = ctx.Calculate_PseudochargeCutoff(d["L"], float(d["tol_pseudocharge"]))
    for t in range(len(tables)):
        np.testing.assert_allclose(cut[t], d[f"t{t}_cutoff"], rtol=1e-13, atol=0)


@pytest.mark.parametrize("system", SYSTEMS)
def test_pseudocharge_and_densities(gpu_available, system):
    d, tables = load(system)
    ctx = ctx_for(d)
    ctx.set_psd(tables)
    cut = np.stack([d[f"t{t}_cutoff"] for t in range(len(tables))])
    f = ctx.Generate_PseudoChargeDensity(d["L"], d["nAtomv"], d["atom_pos"],
                                         ref_cutoff=float(d["ref_cutoff"]),
                                         net_charge=int(d["net_charge"]), cutoff=cut,
                                         want_bref=True)
    assert field_err(f["b"], d["b"]) < 1e-11
    assert field_err(f["b_ref"], d["b_ref"]) < 1e-11
    assert field_err(f["rho_at"], d["rho0"]) < 1e-11
    assert field_err(f["rho_core"], d["rho_core"]) < 1e-11
    assert abs(f["Esc"] - float(d["Esc"])) < 1e-9 * max(1.0, abs(float(d["Esc"])))
    assert abs(f["PosCharge"] - float(d["PosCharge"])) < 1e-9
    assert abs(f["NegCharge"] - float(d["NegCharge"])) < 1e-9


@pytest.mark.parametrize("system", SYSTEMS)
def test_projectors_match_reference(gpu_available, system):
    d, tables = load(system)
    mine = ctx_for(d)
    mine.set_psd(tables)
    mine.CalculateNonlocalProjectors(d["L"], d["nAtomv"], d["atom_pos"])
    ref = ctx_for(d)
    ref.set_nonlocal(d["nl_ip_displ"], d["nl_gamma"], d["nl_img_atom"], d["nl_img_ndc"],
                     d["nl_grid_pos"], d["nl_chi"])
    rng = np.random.default_rng(5)
    Nd = int(d["Nx"]) * int(d["Ny"]) * int(d["Nz"])
    x = rng.uniform(-1, 1, (3, Nd))
    y1, y2 = np.zeros_like(x), np.zeros_like(x)
    mine.Vnl_vec_mult(x, y1)
    ref.Vnl_vec_mult(x, y2)
    assert field_err(y1, y2) < 1e-12


@pytest.mark.parametrize("precision", [64, 32])
def test_scf_from_own_setup_matches_reference_program(gpu_available, precision):
    """Si8 (C1): psp8 tables -> device set-up -> SCF, against the reference program's run."""
    with open(os.path.join(GOLDEN, "Si8_c1_scf_ref.json")) as fh:
        ref = json.load(fh)
    sysd = systems.si8_c1()
    N = (26, 26, 26)
    cs = CellSystem(sysd["L"], N, sysd["species"], {"Si": load_tables(
        os.path.join(GOLDEN, "psp_Si.npz"))})
    prm = cs.scf_params(Nstates=32, cheb_degree=20, precision=precision)
    fields = {}
    res, rho, lam, occ = cs.scf(prm, fields=fields)
    assert res["converged"] == 1
    assert abs(res["Etot"] / cs.n_atom - ref["Etot_per_atom"]) < 1e-5
    occupied = np.array(ref["occ"]) > 1e-3
    assert np.abs(lam[occupied] - np.array(ref["lambda"])[occupied]).max() < 1e-5
    assert abs(res["Esc"] - ref["Esc"]) < 1e-6
    # forces (local + nonlocal + core correction, mean removed) within 1e-4 Ha/Bohr of the
    # reference program's
    F = cs.forces(fields, occ)
    Fref = np.array(ref["forces"])
    assert F.shape == Fref.shape
    assert np.abs(F - Fref).max() < 1e-4, np.abs(F - Fref).max()


def test_gradient_of_periodic_functions(gpu_available):
    """sgpu_Gradient_vectors_dir (order-12 FD, periodic) against analytic derivatives of
    resolved periodic functions, in each direction and for a non-cubic cell."""
    from sparc_gb300.synthetic import fd_d2_coeffs
    N = (24, 20, 28)
    L = (7.3, 6.1, 8.9)
    h = [L[d] / N[d] for d in range(3)]
    ctx = sg.Context(N[0], N[1], N[2], 6, fd_d2_coeffs(6, h[0]), fd_d2_coeffs(6, h[1]),
                     fd_d2_coeffs(6, h[2]), h[0] * h[1] * h[2])
    x = np.arange(N[0]) * h[0]
    y = np.arange(N[1]) * h[1]
    z = np.arange(N[2]) * h[2]
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    k = [2 * np.pi / L[d] for d in range(3)]
    f = np.sin(k[0] * X + 0.3) * np.cos(2 * k[1] * Y) * np.sin(k[2] * Z + 1.1)
    dfs = [k[0] * np.cos(k[0] * X + 0.3) * np.cos(2 * k[1] * Y) * np.sin(k[2] * Z + 1.1),
           -2 * k[1] * np.sin(k[0] * X + 0.3) * np.sin(2 * k[1] * Y) * np.sin(k[2] * Z + 1.1),
           k[2] * np.sin(k[0] * X + 0.3) * np.cos(2 * k[1] * Y) * np.cos(k[2] * Z + 1.1)]
    f2 = np.stack([f.reshape(-1), 2 * f.reshape(-1)])
    for d in range(3):
        out = np.zeros_like(f2)
        ctx.Gradient_vectors_dir(L, f2, out, d)
        ref = dfs[d].reshape(-1)
        assert np.abs(out[0] - ref).max() < 1e-6 * np.abs(ref).max(), d
        np.testing.assert_allclose(out[1], 2 * out[0], rtol=0, atol=1e-13)


def test_density_cube_from_cell_system(gpu_available, tmp_path):
    """The cube bridge on a device set-up: rho_at of Si8 written with its atoms and read back."""
    from sparc_gb300.cube import read_cube
    from sparc_gb300.learned_density import write_density_cube
    sysd = systems.si8_c1()
    cs = CellSystem(sysd["L"], (26, 26, 26), sysd["species"], {"Si": load_tables(
        os.path.join(GOLDEN, "psp_Si.npz"))})
    path = str(tmp_path / "rho_at.cube")
    write_density_cube(cs, cs.fields["rho_at"], path)
    rho, N, steps, atoms = read_cube(path)
    assert N == (26, 26, 26) and len(atoms) == cs.n_atom
    assert all(a[0] == 14 and a[1] == 4.0 for a in atoms)
    np.testing.assert_allclose(rho, cs.fields["rho_at"], rtol=1e-10, atol=0)
    np.testing.assert_allclose(rho.sum() * cs.dV, cs.Nelectron, rtol=1e-9)
