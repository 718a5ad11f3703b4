"""The SCF-side oracle (oracle/scf_oracle.py) against the reference program's own outputs for
the Si8 system (tests/golden/Si8_c1_scf.npz). CPU only."""
import numpy as np

from oracle import scf_oracle as so
from oracle.oracle import Oracle
from scf_io import load_scf


def test_lda_pw_matches_reference():
    d, grid, nl, ref = load_scf()
    vxc, exc = so.lda_pw(d["rho0"], d["rho_core"] if int(d["nlcc"]) else None,
                         ref["params"]["xc_rhotol"])
    assert np.abs(vxc - d["vxc0"]).max() <= 1e-13 * np.abs(d["vxc0"]).max()
    assert np.abs(exc - d["exc0"]).max() <= 1e-13 * np.abs(d["exc0"]).max()


def test_poisson_matches_reference():
    d, grid, nl, ref = load_scf()
    o = Oracle(grid, nl)
    phi, it = so.poisson(o, d["rho0"], d["b"], np.zeros_like(d["b"]),
                         ref["params"]["TOL_POISSON"])
    # both solves stop at ||r|| <= 1e-8 ||rhs||; the solutions agree to that level
    assert np.abs(phi - d["phi0"]).max() < 1e-6 * np.abs(d["phi0"]).max()
    assert 10 < it < 3000


def test_mixer_keeps_charge_and_positivity():
    d, grid, nl, ref = load_scf()
    o = Oracle(grid, nl)
    neg = -float(d["Nelectron"])
    mx = so.PulayMixer(o, d["rho0"], neg, grid["dV"],
                       precond_tol=ref["params"]["TOL_PRECOND"])
    rng = np.random.default_rng(0)
    g = d["rho0"] * (1.0 + 0.05 * rng.standard_normal(d["rho0"].size))
    for it in range(3):
        x = mx.step(it, g)
        assert x.min() >= 0.0
        assert abs(x.sum() * grid["dV"] + neg) < 1e-9
        g = 0.5 * (g + x)
