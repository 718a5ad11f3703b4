"""CPU oracle for the SCF-side rows of the CheFSI path (numpy over the C stencil of
sparc_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker for tests/ and bench.py's CPU baseline; never imported
by the GPU library. Each function restates the reference routine it names (file:line in the
reference SPARC sources); parity with the reference program itself is pinned by
tests/golden/*_scf.npz (reference Calculate_Vxc / Calculate_elecstPotential outputs) and by
the reference SCF run in tests/golden/*_scf_ref.json.
"""
import math

import numpy as np


def density(psi, occ, occfac, dV):
    """rho = (1/dV) sum_n occfac occ_n psi_n^2 (CalculateDensity_psi,
    src/electronDensity.c:104-205, Gamma point, one spin). psi: (ncol, Nd)."""
    w = occfac * np.asarray(occ)
    return (w[:, None] * psi * psi).sum(axis=0) / dV


def lda_pw(rho, rho_core, rhotol):
    """Slater exchange + PW92 correlation on max(rho + rho_core, rhotol): returns (vxc, exc).
    Restates slater (src/exchangeCorrelation.c:459), pw (:475) and add_rho_core (:1254)."""
    r = rho + (rho_core if rho_core is not None else 0.0)
    r = np.maximum(r, rhotol)
    C2, C3, C31 = 0.738558766382022, 0.9847450218426965, 0.6203504908993999
    A, a1 = 0.031091, 0.21370
    b1, b2, b3, b4 = 7.5957, 3.5876, 1.6382, 0.49294
    rc = np.cbrt(r)
    ex, vx = -C2 * rc, -C3 * rc
    rs = C31 / rc
    rsq = np.sqrt(rs)
    G2 = 2.0 * A * (b1 * rsq + b2 * rs + b3 * rs * rsq + b4 * rs * rs)
    G1 = np.log(1.0 + 1.0 / G2)
    ec = -2.0 * A * (1.0 + a1 * rs) * G1
    vc = ec - (rs / 3.0) * (-2.0 * A * a1 * G1 + (2.0 * A * (1.0 + a1 * rs) *
                                                   (A * (b1 / rsq + 2.0 * b2 + 3.0 * b3 * rsq + 4.0 * b4 * rs)))
                            / (G2 * (G2 + 1.0)))
    return vx + vc, ex + ec


def _pw92_g(rs, A, a1, b1, b2, b3, b4):
    """PW92 G(rs) for one parameter set and its rs derivative (PRB 45, 13244, eq. 10)."""
    rsq = np.sqrt(rs)
    q1 = 2.0 * A * (b1 * rsq + b2 * rs + b3 * rs * rsq + b4 * rs * rs)
    dq1 = A * (b1 / rsq + 2.0 * b2 + 3.0 * b3 * rsq + 4.0 * b4 * rs)
    lg = np.log(1.0 + 1.0 / q1)
    q0 = -2.0 * A * (1.0 + a1 * rs)
    return q0 * lg, -2.0 * A * a1 * lg - q0 * dq1 / (q1 * (q1 + 1.0))


def lsda_pw(up, dn, rho_core, rhotol):
    """Spin-polarised Slater exchange + PW92 correlation (collinear spin): each spin density
    plus half the core density, clamped at rhotol; returns (vxc (2, Nd), exc). Restates
    slater_spin (src/exchangeCorrelation.c:759), pw_spin (:787) with its zeta scaling by
    1 - 1e-6, and add_rho_core with three columns (:1254)."""
    hc = 0.5 * rho_core if rho_core is not None else 0.0
    ru = np.maximum(up + hc, rhotol)
    rd = np.maximum(dn + hc, rhotol)
    r = ru + rd
    kx = 0.75 * (6.0 / math.pi) ** (1.0 / 3.0)
    exu, exd = -kx * np.cbrt(ru), -kx * np.cbrt(rd)
    ex = (exu * ru + exd * rd) / r
    rs = (3.0 / (4.0 * math.pi)) ** (1.0 / 3.0) / np.cbrt(r)
    e0, de0 = _pw92_g(rs, 0.031091, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294)
    e1, de1 = _pw92_g(rs, 0.015545, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517)
    am, dam = _pw92_g(rs, 0.016887, 0.11125, 10.357, 3.6231, 0.88026, 0.49671)  # -alpha_c
    az, fpp0 = 1.0 - 1e-6, 1.709921
    fden = 1.0 / (2.0 ** (4.0 / 3.0) - 2.0)
    z = (ru - rd) / r
    zp, zm = 1.0 + az * z, 1.0 - az * z
    f = (zp ** (4.0 / 3.0) + zm ** (4.0 / 3.0) - 2.0) * fden
    df = (4.0 / 3.0) * az * (np.cbrt(zp) - np.cbrt(zm)) * fden
    z4 = z ** 4
    ec = e0 - am / fpp0 * f * (1.0 - z4) + (e1 - e0) * f * z4
    dec_drs = de0 - dam / fpp0 * f * (1.0 - z4) + (de1 - de0) * f * z4
    dec_dz = -am / fpp0 * (df * (1.0 - z4) - 4.0 * z ** 3 * f) + (e1 - e0) * (df * z4 + 4.0 * z ** 3 * f)
    base = ec - rs / 3.0 * dec_drs - z * dec_dz
    vxc = np.stack([4.0 / 3.0 * exu + base + dec_dz, 4.0 / 3.0 * exd + base - dec_dz])
    return vxc, ex + ec


def _lstsq_min_norm(A, b):
    """Minimum-norm least squares as LAPACK dgelsd with rcond = -1 (machine epsilon)."""
    return np.linalg.lstsq(A, b, rcond=np.finfo(float).eps)[0]


def aar(orc, c, x, b, omega=0.6, beta=0.6, m=7, p=6, tol=1e-8, max_iter=3000):
    """AAR for b + (Lap + c) x = 0 with the Jacobi preconditioner, restating AAR
    (src/linearSolver.c:37-165), poisson_residual (src/lapVecRoutines.c:69) and
    Jacobi_preconditioner (src/electrostatics.c:1682). Returns (x, iterations)."""
    N = x.size
    x = x.copy()
    X = np.zeros((m, N))
    F = np.zeros((m, N))
    minv = orc.g.cx[0] + orc.g.cy[0] + orc.g.cz[0] + c
    if abs(minv) < 1e-14:
        minv = 1.0
    minv = -1.0 / minv

    def res(xx):
        return orc.poisson_residual(c, xx, b)

    x_old = x.copy()
    f_old = np.zeros(N)
    r = res(x)
    tol = tol * np.linalg.norm(b)
    rnorm = tol + 1.0
    it = 0
    while rnorm > tol and it < max_iter:
        f = minv * r
        if it > 0:
            h = (it - 1) % m
            X[h] = x - x_old
            F[h] = f - f_old
        x_old = x.copy()
        f_old = f.copy()
        if (it + 1) % p == 0 and it > 0:
            gam = _lstsq_min_norm(F @ F.T, F @ f)
            x = x_old - gam @ X + beta * (f - gam @ F)
            r = res(x)
            rnorm = np.linalg.norm(r)
        else:
            x = x_old + omega * f
            r = res(x)
        it += 1
    return x, it


def poisson(orc, rho, b, phi0, tol, max_iter=3000):
    """-Lap phi = 4 pi (b + rho), zero mean (Calculate_elecstPotential,
    src/electrostatics.c:1593-1680 with poisson_RHS :1494)."""
    phi, it = aar(orc, 0.0, phi0, 4.0 * math.pi * (b + rho), tol=tol, max_iter=max_iter)
    return phi - phi.mean(), it


def kerker(orc, f, a, kTF, idiemac, tol, Pf0):
    """Pf = a (L - kTF^2)^-1 (L - idiemac kTF^2) f via AAR (Kerker_precond,
    src/mixing.c:462-528)."""
    Lf = orc.lap_plus_diag(1.0, 0.0, -kTF * kTF * idiemac, None, f)[0]
    Pf, _ = aar(orc, -kTF * kTF, Pf0, Lf, tol=tol, max_iter=1000)
    if abs(kTF) < 1e-14:
        Pf = Pf - Pf.mean()
    return -a * Pf


class PulayMixer:
    """Periodic-Pulay density mixing with Kerker preconditioning, restating
    Mixing_periodic_pulay (src/mixing.c:213-455) and AndersonExtrapWtdAvg (:77). With
    nspden = 2 (collinear spin) x is [rho, magz]: the magnetization residual is scaled by
    beta_mag / omega_mag alone (MixingPrecondMag = 0), both preconditioned parts are shifted
    to their residual's integral (:376-385), and only rho is clamped and rescaled."""

    def __init__(self, orc, x0, neg_charge, dV, m=7, p=1, beta=0.3, omega=0.3, kerker_on=1,
                 kTF=1.0, idiemac=0.1, precond_tol=1e-4, nspden=1, beta_mag=None,
                 omega_mag=None):
        self.orc, self.m, self.p, self.beta, self.omega = orc, m, p, beta, omega
        self.kerker, self.kTF, self.idiemac, self.tol = kerker_on, kTF, idiemac, precond_tol
        self.neg_charge, self.dV = neg_charge, dV
        self.nspden = nspden
        self.beta_mag = beta if beta_mag is None else beta_mag
        self.omega_mag = self.beta_mag if omega_mag is None else omega_mag
        N = x0.size
        self.x_k = x0.copy()
        self.x_km1 = np.zeros(N)
        self.f_k = np.zeros(N)
        self.f_km1 = np.zeros(N)
        self.R = np.zeros((m, N))
        self.F = np.zeros((m, N))
        self.Pf = np.zeros(N)

    def step(self, it, g):
        pulay = ((it + 1) % self.p == 0) and it > 0
        amix = self.beta if pulay else self.omega
        if it > 0:
            self.f_km1 = self.f_k.copy()
        self.f_k = g - self.x_k
        if it > 0:
            h = (it - 1) % self.m
            self.R[h] = self.x_k - self.x_km1
            self.F[h] = self.f_k - self.f_km1
        if pulay:
            gam = _lstsq_min_norm(self.F @ self.F.T, self.F @ self.f_k)
            xw = self.x_k - gam @ self.R
            fw = self.f_k - gam @ self.F
        else:
            xw, fw = self.x_k.copy(), self.f_k.copy()
        nd = g.size // self.nspden
        Pf = self.Pf.copy()
        if self.kerker:
            Pf[:nd] = kerker(self.orc, fw[:nd], amix, self.kTF, self.idiemac, self.tol, Pf[:nd])
        else:
            Pf[:nd] = amix * fw[:nd]
        if self.nspden == 2:
            Pf[nd:] = (self.beta_mag if pulay else self.omega_mag) * fw[nd:]
            for c in range(2):
                seg = slice(c * nd, (c + 1) * nd)
                Pf[seg] += (fw[seg].sum() - Pf[seg].sum()) / nd
        self.Pf = Pf
        x = xw + Pf
        x[:nd][x[:nd] < 0.0] = 0.0
        x[:nd] *= -self.neg_charge / (x[:nd].sum() * self.dV)
        self.x_km1 = self.x_k
        self.x_k = x.copy()
        return x


def scf_error(rho_out, rho_in):
    """Evaluate_scf_error (src/electronicGroundState.c:1160-1195)."""
    return math.sqrt(((rho_out - rho_in) ** 2).sum() / (rho_out ** 2).sum())


def smearing(beta, lam, ef, typ=0):
    """smearing_function (src/occupation.c:31)."""
    if typ:
        return 0.5 * (1.0 - np.vectorize(math.erf)(beta * (lam - ef)))
    return 1.0 / (1.0 + np.exp(beta * (lam - ef)))
