"""The CPU oracle against golden vectors produced by the reference SPARC program itself
(tests/golden/*.npz, see tests/golden/make_golden.py). CPU only."""
import numpy as np
import pytest

from golden_io import CASES, load, rel_err
from oracle.oracle import Oracle, fd_d2_weights

TOL = 1e-13  # FP64 restatement of the same arithmetic: differences are rounding only


@pytest.mark.parametrize("case", CASES)
def test_fd_weights(case):
    d, grid, _ = load(case)
    w = fd_d2_weights(grid["FDn"], float(d["h"][0]))
    assert rel_err(w, d["cx"]) < 1e-14


@pytest.mark.parametrize("case", CASES)
def test_stencil_bit_exact(case):
    d, grid, nl = load(case)
    o = Oracle(grid, nl)
    # Lap_plus_diag_vec_mult_orth with and without the diagonal term: same operation order
    np.testing.assert_array_equal(o.lap_plus_diag(-0.5, 1.0, 0.3, d["veff"], d["x"]),
                                  d["lap_plus_diag"])
    np.testing.assert_array_equal(o.lap_plus_diag(1.0, 0.0, 0.0, None, d["x"][:1]), d["lap"])
    np.testing.assert_array_equal(o.poisson_residual(0.0, d["x"][0], d["b"]),
                                  d["poisson_residual"])


@pytest.mark.parametrize("case", CASES)
def test_nonlocal_hamiltonian_filter(case):
    d, grid, nl = load(case)
    o = Oracle(grid, nl)
    assert rel_err(o.vnl(d["x"]), d["vnl"]) < TOL
    assert rel_err(o.hamiltonian(d["veff"], -1.2, d["x"]), d["hamiltonian"]) < TOL
    b = d["cheb_bounds"]
    X, Y = o.chebyshev(d["veff"], int(d["cheb_m"]), b[0], b[1], b[2], d["x"])
    assert rel_err(Y, d["cheb_Y"]) < 1e-12
    assert rel_err(X, d["cheb_X"]) < 1e-12


def test_oracle_detects_planted_error():
    """A mistake planted in the oracle's inputs must be caught by the golden comparison."""
    d, grid, nl = load("si2_small")
    cx = d["cx"].copy()
    cx[3] *= 1.0 + 1e-9
    o = Oracle(dict(grid, cx=cx), nl)
    assert rel_err(o.lap_plus_diag(1.0, 0.0, 0.0, None, d["x"][:1]), d["lap"]) > 1e-12


@pytest.mark.parametrize("lmax", [0, 1, 2, 3])
def test_synthetic_projector_sets_are_consistent(lmax):
    """The synthetic nonlocal sets used by the kernel tests hold exactly sum(ndc) x nproj Chi
    values and in-range grid positions (the kernels and the oracle read them as such)."""
    import numpy as np
    from sparc_gb300.synthetic import synthetic_nonlocal
    rng = np.random.default_rng(lmax)
    N = (20, 18, 16)
    nl = synthetic_nonlocal(rng, N, 0.4, natom=5, rc=2.0, lmax=lmax)
    nproj = (lmax + 1) ** 2
    assert np.all(np.diff(nl["ip_displ"]) == nproj)
    assert len(nl["gamma"]) == 5 * nproj
    assert len(nl["chi"]) == int(np.sum(nl["img_ndc"])) * nproj
    assert len(nl["grid_pos"]) == int(np.sum(nl["img_ndc"]))
    assert nl["grid_pos"].min() >= 0 and nl["grid_pos"].max() < np.prod(N)
    assert np.all(np.isfinite(nl["chi"]))
