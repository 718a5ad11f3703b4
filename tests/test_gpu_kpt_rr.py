"""The k-point Rayleigh-Ritz step and a batched complex CheFSI through the C ABI, on the
Si2 system with Bloch vectors (the reference's own k-point set-up, tests/golden/
si2_kpt_kernels.npz; 14^3 grid).

H_k is formed densely from the CPU oracle (oracle/sparc_oracle.c, pinned to the reference's
Hamiltonian_vectors_mult_kpt) applied to the identity, and diagonalised with numpy.
* sgpu_Project_Hamiltonian_kpt / sgpu_Solve_Generalized_EigenProblem_kpt /
  sgpu_Subspace_Rotation_kpt (DP_Project_Hamiltonian_kpt src/eigenSolverKpt.c:676,
  DP_Solve_Generalized_EigenProblem_kpt :836, DP_Subspace_Rotation_kpt :947) against numpy:
  1e-12 relative (complex128).
* sgpu_CheFSI_batched: repeated passes over two k-point blocks from random starts converge
  to the lowest eigenvalues of each dense H_k: 1e-8 Ha (complex128), 1e-4 Ha (complex64)."""
import numpy as np
import pytest

import sparc_gb300 as sg
from oracle.oracle import Oracle
from test_oracle_kpt import load_kpt

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def si2k():
    d, grid, nl = load_kpt()
    o = Oracle(grid, nl)
    Nd = int(d["Nx"]) * int(d["Ny"]) * int(d["Nz"])
    dense = []
    for slot in (0, 1):
        k = d["kpts"][slot]
        Hk = o.hamiltonian_kpt(k, d["L"], d["img_coords"], d["veff"], 0.0,
                               np.eye(Nd, dtype=np.complex128))
        H = Hk.T  # row j of the result is H e_j, i.e. column j of H
        H = 0.5 * (H + H.conj().T)
        dense.append((H, np.linalg.eigvalsh(H)))
    ctx = sg.Context(grid["Nx"], grid["Ny"], grid["Nz"], grid["FDn"], grid["cx"], grid["cy"],
                     grid["cz"], grid["dV"])
    ctx.set_veff(d["veff"])
    ctx.set_nonlocal(nl["ip_displ"], nl["gamma"], nl["img_atom"], nl["img_ndc"],
                     nl["grid_pos"], nl["chi"])
    ctx.set_kpoint_geometry(d["L"], d["img_coords"])
    yield d, ctx, dense, Nd
    ctx.close()


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_kpt_rayleigh_ritz_step(gpu_available, si2k):
    import scipy.linalg as sl
    d, ctx, dense, Nd = si2k
    rng = np.random.default_rng(4)
    ncol = 10
    H, _ = dense[1]
    Y = rng.standard_normal((ncol, Nd)) + 1j * rng.standard_normal((ncol, Nd))
    HY = np.zeros_like(Y)
    Hp = np.zeros((ncol, ncol), dtype=np.complex128)
    Mp = np.zeros_like(Hp)
    ctx.Project_Hamiltonian_kpt(d["kpts"][1], Y, HY, Hp, Mp)
    HYo = (H @ Y.T).T
    assert rel(HY, HYo) < 1e-12
    # column-major C arrays: element (m, n) of Hp sits at [n, m]
    assert rel(Hp.T, Y.conj() @ HYo.T) < 1e-12
    assert rel(Mp.T, Y.conj() @ Y.T) < 1e-12
    lam = np.zeros(ncol)
    Q = Hp.copy()
    ctx.Solve_Generalized_EigenProblem_kpt(Q, Mp.copy(), lam)
    Hpo, Mpo = Y.conj() @ HYo.T, Y.conj() @ Y.T
    lo = sl.eigh(0.5 * (Hpo + Hpo.conj().T), Mpo, eigvals_only=True)
    assert np.abs(lam - lo).max() < 1e-10 * np.abs(lo).max()
    X = np.zeros_like(Y)
    ctx.Subspace_Rotation_kpt(Y, Q, X)
    # X[:, n] = sum_k Y[:, k] Q[k, n]; Q column-major: Q.T is the matrix
    assert rel(X, (Y.T @ Q.T).T) < 1e-12


@pytest.mark.parametrize("precision,tol", [(sg.SGPU_PREC_FP64, 1e-8),
                                           (sg.SGPU_PREC_FP32, 1e-4)])
def test_batched_chefsi_converges_to_dense_eigenvalues(gpu_available, si2k, precision, tol):
    import torch
    d, ctx, dense, Nd = si2k
    ncol, want = 12, 8
    cdt = torch.complex128 if precision == sg.SGPU_PREC_FP64 else torch.complex64
    gen = torch.Generator(device="cuda")
    gen.manual_seed(11)
    blocks = []
    for slot in (0, 1):
        _, ev = dense[slot]
        X = torch.complex(torch.rand((ncol, Nd), generator=gen, device="cuda", dtype=torch.float64),
                          torch.rand((ncol, Nd), generator=gen, device="cuda", dtype=torch.float64)
                          ).to(cdt) - (0.5 + 0.5j)
        blocks.append(dict(spin=0, k=list(d["kpts"][slot]), X=X, Y=torch.empty_like(X),
                           a=float(ev[ncol]) + 0.05, b=float(ev[-1]) * 1.01,
                           a0=float(ev[0]) - 0.1))
    for _ in range(14):
        lam = ctx.CheFSI_batched(blocks, 12, precision=precision)
    for slot in (0, 1):
        _, ev = dense[slot]
        assert np.abs(lam[slot][:want] - ev[:want]).max() < tol, (slot, lam[slot][:want] - ev[:want])


@pytest.mark.parametrize("precision,tol", [(sg.SGPU_PREC_FP64, 1e-11),
                                           (sg.SGPU_PREC_FP32, 2e-5)])
def test_batched_rayleigh_ritz_matches_per_block(gpu_available, si2k, precision, tol):
    """The batched Rayleigh-Ritz step (batched products, batched Cholesky reduction, one
    batched Hermitian eigensolve) against one zhegvd per block, on the same filtered blocks:
    the same Ritz values and the same Ritz subspaces (projector difference)."""
    import torch
    d, ctx, dense, Nd = si2k
    ncol = 10
    cdt = torch.complex128 if precision == sg.SGPU_PREC_FP64 else torch.complex64
    gen = torch.Generator(device="cuda")
    gen.manual_seed(23)
    X0 = [torch.complex(torch.rand((ncol, Nd), generator=gen, device="cuda", dtype=torch.float64),
                        torch.rand((ncol, Nd), generator=gen, device="cuda", dtype=torch.float64)
                        ).to(cdt) - (0.5 + 0.5j) for _ in range(3)]
    res = {}
    for mode in (1, 0):
        ctx.set_rr_batched(mode)
        blocks = []
        for b, slot in enumerate((0, 1, 0)):
            _, ev = dense[slot]
            blocks.append(dict(spin=0, k=list(d["kpts"][slot]), X=X0[b].clone(),
                               Y=torch.empty_like(X0[b]), a=float(ev[ncol]) + 0.05,
                               b=float(ev[-1]) * 1.01, a0=float(ev[0]) - 0.1))
        lam = ctx.CheFSI_batched(blocks, 9, precision=precision)
        res[mode] = (lam, [bl["X"].to(torch.complex128).cpu().numpy() for bl in blocks])
    ctx.set_rr_batched(1)
    for b in range(3):
        la, lb = res[1][0][b], res[0][0][b]
        assert np.abs(la - lb).max() < tol * max(1.0, np.abs(lb).max())
        # the Ritz vectors agree up to phases (and rotations inside degenerate groups): the
        # principal angles between the two spans are zero
        Qa, _ = np.linalg.qr(res[1][1][b].T)
        Qb, _ = np.linalg.qr(res[0][1][b].T)
        sv = np.linalg.svd(Qa.conj().T @ Qb, compute_uv=False)
        assert np.abs(1.0 - sv).max() < 100 * tol
