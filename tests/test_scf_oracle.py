"""The SCF-side oracle (oracle/scf_oracle.py) against the reference program's own outputs for
the Si8 system (tests/golden/Si8_c1_scf.npz) and against the reference's own mixing, Kerker
and AAR routines called through oracle/ref/ref_harness.c (tests/golden/Si8_c1_mixing.npz,
written by tests/golden/make_golden.py --only mixing). CPU only."""
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


def _mixing_fixture():
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    return np.load(os.path.join(here, "golden", "Si8_c1_mixing.npz"))


def test_pulay_mixer_matches_reference_mixing():
    """PulayMixer against the reference's own Mixing_periodic_pulay (src/mixing.c:213, through
    oracle/ref/ref_harness.c) over nine SCF iterations of seeded output densities on the Si8
    set-up: past the history of seven, with Kerker preconditioning."""
    d, grid, nl, ref = load_scf()
    m = _mixing_fixture()
    assert np.array_equal(m["rho0"], d["rho0"])
    o = Oracle(grid, nl)
    mx = so.PulayMixer(o, m["rho0"], -float(d["Nelectron"]), grid["dV"],
                       precond_tol=ref["params"]["TOL_PRECOND"])
    for it, g in enumerate(m["outputs"]):
        x = mx.step(it, g.copy())
        assert np.abs(x - m["mixed"][it]).max() <= 1e-10 * np.abs(m["mixed"][it]).max(), it


def test_kerker_and_aar_match_reference():
    """kerker and aar against the reference's Kerker_precond (src/mixing.c:462) and AAR
    (src/linearSolver.c:37, Poisson settings, Jacobi preconditioner) on the Si8 grid."""
    d, grid, nl, ref = load_scf()
    m = _mixing_fixture()
    o = Oracle(grid, nl)
    f = m["kerker_f"]
    Pf = so.kerker(o, f, float(m["kerker_a"]), 1.0, 0.1, ref["params"]["TOL_PRECOND"],
                   np.zeros_like(f))
    assert np.abs(Pf - m["kerker_Pf"]).max() <= 1e-12 * np.abs(m["kerker_Pf"]).max()
    b = m["aar_b"]
    x0, _ = so.aar(o, 0.0, np.zeros_like(b), b - b.mean(), tol=float(m["aar_tol"]))
    x1, _ = so.aar(o, -1.0, np.zeros_like(b), b, tol=float(m["aar_tol"]))
    assert np.abs(x0 - m["aar_x_c0"]).max() <= 1e-12 * np.abs(m["aar_x_c0"]).max()
    assert np.abs(x1 - m["aar_x_c1"]).max() <= 1e-12 * np.abs(m["aar_x_c1"]).max()
