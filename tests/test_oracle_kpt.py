"""The k-point (complex, Bloch-phase) oracle against the reference program's own k-point
kernels (tests/golden/si2_kpt_kernels.npz, from Lap_plus_diag_vec_mult_orth_kpt,
Vnl_vec_mult_kpt, Hamiltonian_vectors_mult_kpt and ChebyshevFiltering_kpt). CPU only."""
import numpy as np
import pytest

from golden_io import rel_err
from oracle.oracle import Oracle

import os
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_kpt():
    f = np.load(os.path.join(GOLDEN, "si2_kpt_kernels.npz"))
    d = {k: f[k] for k in f.files}
    grid = dict(Nx=int(d["Nx"]), Ny=int(d["Ny"]), Nz=int(d["Nz"]), FDn=int(d["FDn"]),
                cx=d["cx"], cy=d["cy"], cz=d["cz"], dV=float(d["dV"]))
    nl = {k[3:]: v for k, v in d.items() if k.startswith("nl_")}
    return d, grid, nl


@pytest.mark.parametrize("slot", [0, 1])
def test_kpt_oracle_matches_reference(slot):
    d, grid, nl = load_kpt()
    o = Oracle(grid, nl)
    k, L, ic = d["kpts"][slot], d["L"], d["img_coords"]
    assert rel_err(o.lap_plus_diag_kpt(k, L, -0.5, 1.0, 0.3, d["veff"], d["x"]),
                   d[f"lap_plus_diag_{slot}"]) < 1e-14
    assert rel_err(o.vnl_kpt(k, L, ic, d["x"]), d[f"vnl_{slot}"]) < 1e-13
    assert rel_err(o.hamiltonian_kpt(k, L, ic, d["veff"], -1.2, d["x"]),
                   d[f"hamiltonian_{slot}"]) < 1e-13
    b = d["cheb_bounds"]
    X, Y = o.chebyshev_kpt(k, L, ic, d["veff"], int(d["cheb_m"]), b[0], b[1], b[2], d["x"])
    assert rel_err(Y, d[f"cheb_Y_{slot}"]) < 1e-12
    assert rel_err(X, d[f"cheb_X_{slot}"]) < 1e-12


def test_kpt_phases_matter():
    """A k-point with nonzero phases gives a different result from Gamma (the fixture would
    not catch a dropped phase otherwise)."""
    d, grid, nl = load_kpt()
    o = Oracle(grid, nl)
    assert np.abs(d["kpts"][0]).min() > 0.1
    g = o.lap_plus_diag_kpt(np.zeros(3), d["L"], -0.5, 1.0, 0.3, d["veff"], d["x"])
    assert rel_err(g, d["lap_plus_diag_0"]) > 1e-3
