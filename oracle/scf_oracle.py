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
    Mixing_periodic_pulay (src/mixing.c:213-455) and AndersonExtrapWtdAvg (:77)."""

    def __init__(self, orc, x0, neg_charge, dV, m=7, p=1, beta=0.3, omega=0.3, kerker_on=1,
                 kTF=1.0, idiemac=0.1, precond_tol=1e-4):
        self.orc, self.m, self.p, self.beta, self.omega = orc, m, p, beta, omega
        self.kerker, self.kTF, self.idiemac, self.tol = kerker_on, kTF, idiemac, precond_tol
        self.neg_charge, self.dV = neg_charge, dV
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
        if self.kerker:
            self.Pf = kerker(self.orc, fw, amix, self.kTF, self.idiemac, self.tol, self.Pf)
        else:
            self.Pf = amix * fw
        x = xw + self.Pf
        x[x < 0.0] = 0.0
        x *= -self.neg_charge / (x.sum() * self.dV)
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
