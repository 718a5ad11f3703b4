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


def test_lsda_matches_reference():
    """lsda_pw against the reference's own spin Calculate_Vxc (slater_spin + pw_spin with the
    core density split between the spins) on the Al4 spin start density."""
    d, grid, nl, ref = load_scf("Al4_spin_kpt")
    rho3 = d["rho3_0"]
    assert np.allclose(rho3[1] + rho3[2], rho3[0]) and np.allclose(rho3[1] - rho3[2], d["mag0"])
    vxc, exc = so.lsda_pw(rho3[1], rho3[2], d["rho_core"], ref["params"]["xc_rhotol"])
    assert np.abs(vxc - d["vxc0_spin"]).max() <= 1e-12 * np.abs(d["vxc0_spin"]).max()
    assert np.abs(exc - d["exc0_spin"]).max() <= 1e-12 * np.abs(d["exc0_spin"]).max()
    # unpolarised limit: equal spin densities give the LDA potential on both spins
    vu, eu = so.lsda_pw(0.5 * rho3[0], 0.5 * rho3[0], d["rho_core"], ref["params"]["xc_rhotol"])
    vl, el = so.lda_pw(rho3[0], d["rho_core"], ref["params"]["xc_rhotol"])
    assert np.abs(vu[0] - vl).max() < 1e-9 and np.abs(eu - el).max() < 1e-9


def test_spin_mixer_matches_reference_mixing():
    """PulayMixer with nspden = 2 ([rho, magz]) against the reference's Mixing_periodic_pulay
    on the Al4 spin set-up over nine iterations of seeded output densities and
    magnetizations (Kerker on rho, plain amix_mag on magz, integral-preserving shifts)."""
    d, grid, nl, ref = load_scf("Al4_spin_kpt")
    p = ref["params"]
    assert p["MixingPrecondMag"] == 0
    o = Oracle(grid, nl)
    x0 = np.concatenate([d["rho3_0"][0], d["mag0"]])
    mx = so.PulayMixer(o, x0, -float(d["Nelectron"]), grid["dV"], m=int(p["MixingHistory"]),
                       beta=p["MixingParameter"], omega=p["MixingParameterSimple"],
                       kerker_on=int(p["MixingPrecond"] == 1), kTF=p["precond_kerker_kTF"],
                       idiemac=p["precond_kerker_thresh"], precond_tol=p["TOL_PRECOND"],
                       nspden=2, beta_mag=p["MixingParameterMag"],
                       omega_mag=p["MixingParameterSimpleMag"])
    nd = d["rho3_0"].shape[1]
    for it, (g, gm) in enumerate(zip(d["mix_outputs"], d["mix_mag_outputs"])):
        x = mx.step(it, np.concatenate([g, gm]))
        r_ref, m_ref = d["mix_rho"][it], d["mix_mag"][it]
        assert np.abs(x[:nd] - r_ref).max() <= 1e-10 * np.abs(r_ref).max(), it
        assert np.abs(x[nd:] - m_ref).max() <= 1e-10 * np.abs(m_ref).max(), it
