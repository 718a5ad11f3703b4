"""GPU parity of the k-point (Bloch) rows through the C ABI, against the reference program's
own complex kernels (tests/golden/si2_kpt_kernels.npz) and the k-point oracle.
Tolerances: complex128 1e-12 relative; complex64 filter 5e-4 relative."""
import numpy as np
import pytest

import sparc_gb300 as sg
from golden_io import rel_err
from oracle.oracle import Oracle
from sparc_gb300.synthetic import fd_d2_coeffs, synthetic_nonlocal
from test_oracle_kpt import load_kpt

pytestmark = pytest.mark.gpu


def make_ctx(d, grid, nl):
    ctx = sg.Context(grid["Nx"], grid["Ny"], grid["Nz"], grid["FDn"], grid["cx"], grid["cy"],
                     grid["cz"], grid["dV"])
    ctx.set_veff(d["veff"])
    ctx.set_nonlocal(nl["ip_displ"], nl["gamma"], nl["img_atom"], nl["img_ndc"],
                     nl["grid_pos"], nl["chi"])
    ctx.set_kpoint_geometry(d["L"], d["img_coords"])
    return ctx


@pytest.mark.parametrize("slot", [0, 1])
def test_kpt_kernels_match_reference(gpu_available, slot):
    d, grid, nl = load_kpt()
    ctx = make_ctx(d, grid, nl)
    k = d["kpts"][slot]
    x = d["x"]
    y = np.zeros_like(x)
    ctx.Lap_plus_diag_vec_mult_orth_kpt(k, -0.5, 1.0, 0.3, d["veff"], x, y)
    assert rel_err(y, d[f"lap_plus_diag_{slot}"]) < 1e-12
    h = np.zeros_like(x)
    ctx.Vnl_vec_mult_kpt(k, x, h)
    assert rel_err(h, d[f"vnl_{slot}"]) < 1e-12
    h2 = np.zeros_like(x)
    ctx.Hamiltonian_vectors_mult_kpt(k, -1.2, x, h2)
    assert rel_err(h2, d[f"hamiltonian_{slot}"]) < 1e-12
    b = d["cheb_bounds"]
    for prec, tol in ((sg.SGPU_PREC_FP64, 1e-12), (sg.SGPU_PREC_FP32, 5e-4)):
        X = x.copy()
        Y = np.zeros_like(x)
        ctx.ChebyshevFiltering_kpt(k, X, Y, int(d["cheb_m"]), b[0], b[1], b[2], precision=prec)
        assert rel_err(Y, d[f"cheb_Y_{slot}"]) < tol
        assert rel_err(X, d[f"cheb_X_{slot}"]) < tol


@pytest.mark.parametrize("shape", [(13, 17, 19), (40, 33, 12)])
def test_kpt_random_grids_vs_oracle(gpu_available, shape):
    rng = np.random.default_rng(sum(shape))
    h = 0.4
    c = fd_d2_coeffs(6, h)
    grid = dict(Nx=shape[0], Ny=shape[1], Nz=shape[2], FDn=6, cx=c, cy=c, cz=c, dV=h ** 3)
    Nd = shape[0] * shape[1] * shape[2]
    nl = synthetic_nonlocal(rng, shape, h, natom=3, rc=1.6)
    L = np.array(shape, dtype=float) * h
    # images inside the cell (shift 0) and shifted copies: coordinates decide the phases
    coords = rng.uniform(-1.0, 1.0, (len(nl["img_atom"]), 3)) * L * 1.5
    veff = rng.normal(0, 1, Nd)
    ctx = sg.Context(shape[0], shape[1], shape[2], 6, c, c, c, h ** 3)
    ctx.set_veff(veff)
    ctx.set_nonlocal(nl["ip_displ"], nl["gamma"], nl["img_atom"], nl["img_ndc"],
                     nl["grid_pos"], nl["chi"])
    ctx.set_kpoint_geometry(L, coords)
    o = Oracle(grid, nl)
    k = np.array([0.7, -0.3, 1.1]) / L
    x = rng.uniform(-1, 1, (3, Nd)) + 1j * rng.uniform(-1, 1, (3, Nd))
    hx = np.zeros_like(x)
    ctx.Hamiltonian_vectors_mult_kpt(k, 0.4, x, hx)
    assert rel_err(hx, o.hamiltonian_kpt(k, L, coords, veff, 0.4, x)) < 1e-12
    X = x.copy(); Y = np.zeros_like(x)
    ctx.ChebyshevFiltering_kpt(k, X, Y, 9, 0.2, 30.0, -3.0)
    Xo, Yo = o.chebyshev_kpt(k, L, coords, veff, 9, 0.2, 30.0, -3.0, x)
    assert rel_err(Y, Yo) < 1e-12 and rel_err(X, Xo) < 1e-12


def test_kpt_requires_geometry(gpu_available):
    d, grid, nl = load_kpt()
    ctx = sg.Context(grid["Nx"], grid["Ny"], grid["Nz"], grid["FDn"], grid["cx"], grid["cy"],
                     grid["cz"], grid["dV"])
    ctx.set_veff(d["veff"])
    x = d["x"]
    with pytest.raises(sg.SgpuError):
        ctx.Hamiltonian_vectors_mult_kpt(d["kpts"][0], 0.0, x, np.zeros_like(x))
