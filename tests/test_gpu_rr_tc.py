"""The Rayleigh-Ritz products on the library's tcgen05 kernels (split BF16 slices with exact
chunk accumulation) against numpy FP64 products of the same inputs, through the C ABI.

Reference: DP_Project_Hamiltonian (src/eigenSolver.c:1022-1033: Mp = Yᵀ Y, Hp = Yᵀ HY) and
DP_Subspace_Rotation (src/eigenSolver.c:1415: X = Y Q), both cblas_dgemm in the reference.
Tolerances: FP64-accurate products 1e-12 of |y_m| |z_n| for the Gram entries (an FP64 GEMM
differs from exact by ~1e-14 of that) and 1e-11 of (|Y| |Q|) entrywise for the rotation (six
7-bit slices keep ~43 bits; a numpy emulation of the same slicing gives 5e-13); FP32-accurate
products (three slices) 1e-5. The rotation's Q is built like the eigenvectors of
(Yᵀ HY, Yᵀ Y): its rows scale inversely to Y's column norms. The shapes are chosen so that K
is not a multiple of the 512-long exact chunk nor of the 32-long step, and the column count
is not a multiple of the 128-wide tile; the columns of Y span six decades, one is zero."""
import numpy as np
import pytest

import sparc_gb300 as sg
from sparc_gb300.synthetic import fd_d2_coeffs

pytestmark = pytest.mark.gpu

SHAPE = (44, 40, 37)  # Nd = 65120
NCOL = 150


def _ctx(rng):
    h = 0.4
    c = fd_d2_coeffs(6, h)
    ctx = sg.Context(*SHAPE, 6, c, c, c, h ** 3)
    Nd = SHAPE[0] * SHAPE[1] * SHAPE[2]
    ctx.set_veff(rng.normal(0.0, 0.5, Nd))
    return ctx, Nd


def _block(rng, ncol, Nd):
    """Columns of very different magnitudes (row scaling of the split), one zero column."""
    Y = rng.uniform(-1, 1, (ncol, Nd)) * 10.0 ** rng.uniform(-3, 3, (ncol, 1))
    Y[7] = 0.0
    return Y


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def scf_like_q(rng, Y):
    """Q whose rows scale like the inverse column norms of Y, as the eigenvectors of
    (Yᵀ HY, Yᵀ Y) do (C array: row n = column n of the column-major Q)."""
    s = np.abs(Y).max(axis=1)
    s[s == 0] = 1.0
    return rng.normal(size=(Y.shape[0], Y.shape[0])) / s[None, :]


def test_fp64_accurate_projection_and_rotation(gpu_available):
    rng = np.random.default_rng(3)
    ctx, Nd = _ctx(rng)
    ctx.set_rr_products(2)  # the tensor-core products for the plain FP64 calls too
    Y = _block(rng, NCOL, Nd)
    HY = np.zeros_like(Y)
    Hp = np.zeros((NCOL, NCOL))
    Mp = np.zeros((NCOL, NCOL))
    ctx.Project_Hamiltonian(Y, HY, Hp, Mp)
    assert ctx.kernel_status() == 0
    ny = np.linalg.norm(Y, axis=1)
    nh = np.linalg.norm(HY, axis=1)
    scale = np.outer(ny, ny)
    nz = scale > 0
    assert np.all(Mp[~nz] == 0)
    assert float((np.abs(Mp - Y @ Y.T)[nz] / scale[nz]).max()) < 1e-12
    # column-major Hp(m, n) = y_m . hy_n is computed for m <= n and mirrored (the eigensolver
    # reads one triangle); in the C array that is Hp[n, m], n >= m, against (HY Yᵀ)[n, m]
    lo = np.tril_indices(NCOL)
    sc = np.outer(nh, ny)[lo]
    nz = sc > 0
    err = np.abs(Hp[lo] - (HY @ Y.T)[lo])[nz] / sc[nz]
    assert float(err.max()) < 1e-12
    assert np.array_equal(Hp, Hp.T) and np.array_equal(Mp, Mp.T)
    # the same inputs give the same bits (fixed split, fixed reduction order)
    Hp2, Mp2 = np.zeros_like(Hp), np.zeros_like(Mp)
    ctx.Project_Hamiltonian(Y, HY, Hp2, Mp2)
    assert np.array_equal(Mp, Mp2) and np.array_equal(Hp, Hp2)
    Q = scf_like_q(rng, Y)
    X = np.zeros_like(Y)
    ctx.Subspace_Rotation(Y, Q, X)
    # Q column-major: row n of the C array holds column n, so row n of X is sum_k Q[n, k] Y[k]
    Xo = Q @ Y
    bound = np.abs(Q) @ np.abs(Y)
    assert float((np.abs(X - Xo) / bound).max()) < 1e-11
    assert rel(X, Xo) < 1e-11
    assert ctx.kernel_status() == 0
    ctx.close()


def test_fp32_accurate_products_on_fp32_blocks(gpu_available):
    import torch
    rng = np.random.default_rng(4)
    ctx, Nd = _ctx(rng)
    ctx.set_rr_products(1)
    y = _block(rng, NCOL, Nd).astype(np.float32)
    Yd = torch.from_numpy(y).cuda()
    HYd = torch.zeros_like(Yd)
    Hp = np.zeros((NCOL, NCOL))
    Mp = np.zeros((NCOL, NCOL))
    ctx.Project_Hamiltonian_f32(Yd, HYd, Hp, Mp)
    y64 = y.astype(np.float64)
    hy64 = HYd.cpu().numpy().astype(np.float64)
    assert rel(Mp, y64 @ y64.T) < 1e-5
    lo = np.tril_indices(NCOL)
    assert rel(Hp[lo], (hy64 @ y64.T)[lo]) < 1e-5
    Q = scf_like_q(rng, y64)
    Xd = torch.zeros_like(Yd)
    ctx.Subspace_Rotation_f32(Yd, Q, Xd)
    assert rel(Xd.cpu().numpy().astype(np.float64), Q @ y64) < 1e-5
    assert ctx.kernel_status() == 0
    ctx.close()


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_generalized_eigensolver_modes(gpu_available, mode):
    """sgpu_Solve_Generalized_EigenProblem in each solver mode (dsygvd; Cholesky reduction with
    dsyevd; with Jacobi dsyevj) against scipy's eigh on an SPD pencil like the subspace's:
    eigenvalues 1e-10 of the largest, Mp-orthonormal eigenvectors with residual 1e-9."""
    import scipy.linalg as sl
    rng = np.random.default_rng(9 + mode)
    ctx, Nd = _ctx(rng)
    ctx.set_eig_solver(mode)
    n = 90
    A = rng.normal(size=(n, n))
    H = A + A.T
    B = rng.normal(size=(n, n)) / n
    M = B @ B.T + np.eye(n)
    Hp, Mp, lam = H.copy(), M.copy(), np.zeros(n)
    ctx.Solve_Generalized_EigenProblem(Hp, Mp, lam)
    lo = sl.eigh(H, M, eigvals_only=True)
    assert np.abs(lam - lo).max() < 1e-10 * np.abs(lo).max()
    Q = Hp.T  # C array rows are the column-major eigenvectors
    assert np.abs(H @ Q - M @ Q * lam[None, :]).max() < 1e-9 * np.abs(lo).max()
    assert np.abs(Q.T @ M @ Q - np.eye(n)).max() < 1e-9
    ctx.close()
