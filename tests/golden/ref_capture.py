"""Capture set-up data and kernel outputs from the reference SPARC objects.

Runs only where the reference was compiled (oracle/_ref/libsparc_ref.so, built by
oracle/ref/Makefile). Each capture runs in its own process because the reference keeps one
SPARC_OBJ per process. Used by make_golden.py to write the committed fixtures.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(HERE, "..", "..", "oracle", "_ref", "libsparc_ref.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


class RefSystem:
    """The reference's own set-up of one .inpt/.ion system, with its kernels callable."""

    def __init__(self, base):
        self.lib = ctypes.CDLL(os.path.abspath(REF_LIB))
        cwd = os.getcwd()
        os.chdir(os.path.dirname(base))
        try:
            self.lib.ref_init(os.path.basename(base).encode())
        finally:
            os.chdir(cwd)
        dims = np.zeros(10, dtype=np.int32)
        self.lib.ref_dims(_i(dims))
        self.Nx, self.Ny, self.Nz, self.Nd, self.order, self.n_atom, self.Ntypes, \
            self.Nstates, self.nproj_total, self.cell_typ = [int(v) for v in dims]
        g = np.zeros(7)
        self.lib.ref_grid(_d(g))
        self.h = g[0:3].copy()
        self.dV = float(g[3])
        self.L = g[4:7].copy()
        fdn = self.order // 2
        self.cx, self.cy, self.cz = (np.zeros(fdn + 1) for _ in range(3))
        self.lib.ref_d2coeffs(_d(self.cx), _d(self.cy), _d(self.cz))

    def nonlocal_data(self):
        """Per atom image: (type, atom_index, grid_pos, Chi[ndc x nproj] column-major)."""
        types = []
        images = []
        for t in range(self.Ntypes):
            ints = np.zeros(16, dtype=np.int32)
            gam = np.zeros(64)
            self.lib.ref_psd(t, _i(ints), _d(gam))
            lmax, lloc, nproj, nat = (int(v) for v in ints[:4])
            ppl = ints[4:4 + lmax + 1].copy()
            types.append(dict(lmax=lmax, lloc=lloc, nproj=nproj, natom=nat, ppl=ppl,
                              gamma=gam[:int(ppl.sum())].copy()))
            for iat in range(self.lib.ref_nloc_natom(t)):
                info = np.zeros(2, dtype=np.int32)
                self.lib.ref_nloc_atom(t, iat, _i(info))
                ndc = int(info[0])
                gp = np.zeros(ndc, dtype=np.int32)
                chi = np.zeros(ndc * max(nproj, 1))
                self.lib.ref_nloc_copy(t, iat, _i(gp), _d(chi))
                images.append(dict(type=t, atom_index=int(info[1]), grid_pos=gp,
                                   chi=chi[:ndc * nproj].reshape(nproj, ndc).T.copy()))
        return types, images

    def setup_fields(self):
        b, bref, rho0 = (np.zeros(self.Nd) for _ in range(3))
        sc = np.zeros(4)
        self.lib.ref_setup_fields(_d(b), _d(bref), _d(rho0), _d(sc))
        return dict(b=b, bref=bref, rho0=rho0, Esc=sc[0], PosCharge=sc[1], NegCharge=sc[2],
                    Nelectron=sc[3])

    def setup_fields2(self):
        bref, rho_at = np.zeros(self.Nd), np.zeros(self.Nd)
        self.lib.ref_setup_fields2(_d(bref), _d(rho_at))
        return dict(b_ref=bref, rho_at=rho_at)

    def core_density(self):
        core = np.zeros(self.Nd)
        self.lib.ref_core_density(_d(core))
        return core

    def psd_tables(self, ityp):
        """The reference's parsed pseudopotential tables of one type (PSD_OBJ)."""
        ints = np.zeros(16, dtype=np.int32)
        sc = np.zeros(16)
        self.lib.ref_psd_tables(ityp, _i(ints), _d(sc), None, None, None, None, None, None)
        n, lmax = int(ints[0]), int(ints[1])
        ppl = ints[5:6 + lmax].copy()
        tot = int(ppl.sum())
        g, u, rv, ri, rc, ga = (np.zeros(n), np.zeros(n * tot), np.zeros(n), np.zeros(n),
                                np.zeros(n), np.zeros(tot))
        self.lib.ref_psd_tables(ityp, _i(ints), _d(sc), _d(g), _d(u), _d(rv), _d(ri), _d(rc),
                                _d(ga))
        return dict(size=n, lmax=lmax, lloc=int(ints[2]), is_r_uniform=int(ints[3]),
                    Znucl=int(ints[4]), ppl=ppl, Vloc_0=sc[0], fchrg=sc[1],
                    rc=sc[2:3 + lmax].copy(), RadialGrid=g, UdV=u.reshape(tot, n), rVloc=rv,
                    rhoIsoAtom=ri, rho_c_table=rc, Gamma=ga)

    def cutoff(self, ityp):
        out = np.zeros(8)
        self.lib.ref_cutoff(ityp, _d(out))
        return dict(cutoff=out[:3].copy(), natom=int(out[3]), tol=out[4], ref_cutoff=out[5],
                    net_charge=int(out[6]))

    def atom_positions(self):
        xyz = np.zeros(3 * self.n_atom)
        self.lib.ref_atom_positions(_d(xyz))
        return xyz.reshape(-1, 3)

    # ---- kernels (x, y column-major: shape (ncol, Nd) C-contiguous == Nd x ncol col-major)
    def lap_plus_diag(self, a, b, c, v, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        vv = np.ascontiguousarray(v, dtype=np.float64) if v is not None else None
        self.lib.ref_lap_plus_diag(ctypes.c_int(x.shape[0]), ctypes.c_double(a),
                                   ctypes.c_double(b), ctypes.c_double(c),
                                   _d(vv) if vv is not None else None, _d(x), _d(y))
        return y

    def vnl(self, x, hx0=None):
        x = np.ascontiguousarray(x, dtype=np.float64)
        hx = np.zeros_like(x) if hx0 is None else np.array(hx0, dtype=np.float64)
        self.lib.ref_vnl(ctypes.c_int(x.shape[0]), _d(x), _d(hx))
        return hx

    def hamiltonian(self, veff, c, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        hx = np.zeros_like(x)
        veff = np.ascontiguousarray(veff, dtype=np.float64)
        self.lib.ref_hamiltonian(ctypes.c_int(x.shape[0]), _d(veff), ctypes.c_double(c),
                                 _d(x), _d(hx))
        return hx

    def chebyshev(self, veff, m, a, b, a0, X):
        X = np.array(X, dtype=np.float64, order="C")
        Y = np.zeros_like(X)
        veff = np.ascontiguousarray(veff, dtype=np.float64)
        self.lib.ref_chebyshev(_d(veff), ctypes.c_int(X.shape[0]), ctypes.c_int(m),
                               ctypes.c_double(a), ctypes.c_double(b), ctypes.c_double(a0),
                               _d(X), _d(Y))
        return X, Y

    def poisson_residual(self, c, x, b):
        x = np.ascontiguousarray(x, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        r = np.zeros_like(x)
        self.lib.ref_poisson_residual(ctypes.c_double(c), _d(x), _d(b), _d(r))
        return r

    def aar(self, c, x0, b, tol, max_iter=3000):
        """The reference's AAR (Poisson settings) on b + (Lap + c) x = 0 from x0."""
        x = np.array(x0, dtype=np.float64)
        b = np.array(b, dtype=np.float64)
        self.lib.ref_aar(ctypes.c_double(c), _d(x), _d(b), ctypes.c_double(tol),
                         ctypes.c_int(max_iter))
        return x

    def kerker(self, f, a):
        """The reference's Kerker_precond of f with mixing parameter a."""
        f = np.array(f, dtype=np.float64)
        Pf = np.zeros_like(f)
        self.lib.ref_kerker(_d(f), ctypes.c_double(a), _d(Pf))
        return Pf

    def mix(self, rho0, outputs):
        """The reference's periodic Pulay mixing over a sequence of output densities: the
        mixed density after each SCF iteration."""
        r0 = np.ascontiguousarray(rho0, dtype=np.float64)
        self.lib.ref_mix_init(_d(r0))
        mixed = []
        for it, g in enumerate(outputs):
            g = np.array(g, dtype=np.float64)
            self.lib.ref_mix_step(ctypes.c_int(it), _d(g))
            mixed.append(g)
        return np.array(mixed)


def spin_fields(r):
    """Collinear-spin set-up of RefSystem r: (spin_typ, [total, up, down] initial density,
    initial magnetization, magnetization mixing parameters)."""
    rho3 = np.zeros(3 * r.Nd)
    mag = np.zeros(r.Nd)
    prm = np.zeros(3)
    st = r.lib.ref_spin_fields(_d(rho3), _d(mag), _d(prm))
    return int(st), rho3.reshape(3, r.Nd), mag, dict(MixingParameterMag=float(prm[0]),
                                                       MixingParameterSimpleMag=float(prm[1]),
                                                       MixingPrecondMag=float(prm[2]))


def vxc_spin(r, rho3):
    """The reference's spin Vxc (2 x Nd) and e_xc (Nd) for [total, up, down] rho3."""
    rho3 = np.ascontiguousarray(rho3, dtype=np.float64).reshape(-1)
    vxc = np.zeros(2 * r.Nd)
    exc = np.zeros(r.Nd)
    r.lib.ref_vxc_spin(_d(rho3), _d(vxc), _d(exc))
    return vxc.reshape(2, r.Nd), exc


def mix_spin(r, rho0, mag0, outputs, mag_outputs):
    """The reference's collinear-spin periodic Pulay mixing: (mixed densities, mixed
    magnetizations) after each SCF iteration."""
    r.lib.ref_mix_init_spin(_d(np.ascontiguousarray(rho0, dtype=np.float64)),
                            _d(np.ascontiguousarray(mag0, dtype=np.float64)))
    rho_m, mag_m = [], []
    for it, (g, gm) in enumerate(zip(outputs, mag_outputs)):
        g = np.array(g, dtype=np.float64)
        gm = np.array(gm, dtype=np.float64)
        r.lib.ref_mix_step_spin(ctypes.c_int(it), _d(g), _d(gm))
        rho_m.append(g)
        mag_m.append(gm)
    return np.array(rho_m), np.array(mag_m)


class RefKpt:
    """k-point (complex) kernels of a RefSystem built from a system with a k-point grid.
    Complex blocks are numpy complex128 arrays of shape (ncol, Nd)."""

    def __init__(self, r):
        self.r = r
        self.lib = r.lib
        self.lib.ref_nloc_copy_kpt.restype = ctypes.c_double
        k = np.zeros(3 * 4096)
        w = np.zeros(4096)
        nk = self.lib.ref_kpoints(_d(k), _d(w))
        self.kpts = k[:3 * nk].reshape(nk, 3).copy()
        self.wts = w[:nk].copy()

    def images(self):
        """Per image: atom index, grid_pos, real Chi (ndc x nproj) and image coordinates."""
        types = []
        out = []
        for t in range(self.r.Ntypes):
            ints = np.zeros(16, dtype=np.int32)
            gam = np.zeros(64)
            self.lib.ref_psd(t, _i(ints), _d(gam))
            lmax, lloc, np_, nat = (int(v) for v in ints[:4])
            ppl = ints[4:4 + lmax + 1].copy()
            types.append(dict(lmax=lmax, lloc=lloc, nproj=np_, natom=nat, ppl=ppl,
                              gamma=gam[:int(ppl.sum())].copy()))
            for iat in range(self.lib.ref_nloc_natom(t)):
                info = np.zeros(2, dtype=np.int32)
                self.lib.ref_nloc_atom(t, iat, _i(info))
                ndc = int(info[0])
                gp = np.zeros(ndc, dtype=np.int32)
                chi = np.zeros(max(ndc * np_, 1))
                mi = self.lib.ref_nloc_copy_kpt(t, iat, _i(gp), _d(chi))
                assert mi == 0.0, "complex projectors are expected to be real-valued"
                xyz = np.zeros(3)
                self.lib.ref_nloc_image_coords(t, iat, _d(xyz))
                out.append(dict(atom_index=int(info[1]), grid_pos=gp,
                                chi=chi[:ndc * np_].reshape(np_, ndc).T.copy(), coords=xyz))
        return types, out

    def lap_plus_diag(self, kpt, a, b, c, v, x):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.zeros_like(x)
        vv = np.ascontiguousarray(v, dtype=np.float64) if v is not None else None
        self.lib.ref_lap_plus_diag_kpt(ctypes.c_int(kpt), ctypes.c_int(x.shape[0]),
                                       ctypes.c_double(a), ctypes.c_double(b),
                                       ctypes.c_double(c), _d(vv) if vv is not None else None,
                                       _d(x.view(np.float64)), _d(y.view(np.float64)))
        return y

    def vnl(self, kpt, x):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        hx = np.zeros_like(x)
        self.lib.ref_vnl_kpt(ctypes.c_int(kpt), ctypes.c_int(x.shape[0]),
                             _d(x.view(np.float64)), _d(hx.view(np.float64)))
        return hx

    def hamiltonian(self, kpt, veff, c, x):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        hx = np.zeros_like(x)
        veff = np.ascontiguousarray(veff, dtype=np.float64)
        self.lib.ref_hamiltonian_kpt(ctypes.c_int(kpt), ctypes.c_int(x.shape[0]), _d(veff),
                                     ctypes.c_double(c), _d(x.view(np.float64)),
                                     _d(hx.view(np.float64)))
        return hx

    def chebyshev(self, kpt, veff, m, a, b, a0, X):
        X = np.array(X, dtype=np.complex128, order="C")
        Y = np.zeros_like(X)
        veff = np.ascontiguousarray(veff, dtype=np.float64)
        self.lib.ref_chebyshev_kpt(ctypes.c_int(kpt), _d(veff), ctypes.c_int(X.shape[0]),
                                   ctypes.c_int(m), ctypes.c_double(a), ctypes.c_double(b),
                                   ctypes.c_double(a0), _d(X.view(np.float64)),
                                   _d(Y.view(np.float64)))
        return X, Y


def scf_setup(r):
    """SCF inputs from the reference set-up of system r (a RefSystem), plus the reference's
    own Vxc and electrostatic potential for the initial density."""
    Nd = r.Nd
    f = r.setup_fields()
    core = np.zeros(Nd)
    nlcc = r.lib.ref_core_density(_d(core))
    prm = np.zeros(20)
    r.lib.ref_scf_params(_d(prm))
    vxc, exc = np.zeros(Nd), np.zeros(Nd)
    r.lib.ref_vxc(_d(f["rho0"]), _d(vxc), _d(exc))
    phi = np.zeros(Nd)
    r.lib.ref_poisson(_d(f["rho0"]), _d(phi))
    keys = ["Beta", "TOL_SCF", "TOL_POISSON", "TOL_PRECOND", "TOL_LANCZOS", "xc_rhotol",
            "ChebDegree", "rhoTrigger", "MixingParameter", "MixingParameterSimple",
            "MixingHistory", "PulayFrequency", "MixingPrecond", "precond_kerker_kTF",
            "precond_kerker_thresh", "MAXIT_POISSON", "MINIT_SCF", "MAXIT_SCF", "elec_T_type",
            "Nchefsi"]
    params = {k: float(v) for k, v in zip(keys, prm)}
    return dict(b=f["b"], rho0=f["rho0"], rho_core=core, nlcc=int(nlcc), Esc=f["Esc"],
                NegCharge=f["NegCharge"], Nelectron=f["Nelectron"], vxc0=vxc, exc0=exc,
                phi0=phi), params


def parse_reference_outputs(base):
    """Energies, SCF count, eigenvalues/occupations and forces from a reference run."""
    out = {}
    with open(base + ".out") as fh:
        for line in fh:
            if line.startswith("Free energy per atom"):
                out["Etot_per_atom"] = float(line.split(":")[1].split()[0])
            elif line.startswith("Total free energy"):
                out["Etot"] = float(line.split(":")[1].split()[0])
            elif line.startswith("Total number of SCF"):
                out["scf_iters"] = int(line.split(":")[1])
            elif line.startswith("Fermi level"):
                out["Efermi"] = float(line.split(":")[1].split()[0])
            elif line.startswith("Total walltime"):
                out["walltime_s"] = float(line.split(":")[1].split()[0])
            elif line.startswith("Band structure energy"):
                out["Eband"] = float(line.split(":")[1].split()[0])
            elif line.startswith("Exchange correlation energy"):
                out["Exc"] = float(line.split(":")[1].split()[0])
            elif line.startswith("Self and correction energy"):
                out["Esc"] = float(line.split(":")[1].split()[0])
            elif line.startswith("-Entropy*kb*T"):
                out["Entropy"] = float(line.split(":")[1].split()[0])
    lam, occ = [], []
    lam_dn, occ_dn = [], []  # collinear spin: the second pair of columns
    with open(base + ".eigen") as fh:
        for line in fh:
            p = line.split()
            if len(p) in (3, 5) and p[0].isdigit():
                lam.append(float(p[1]))
                occ.append(float(p[2]))
                if len(p) == 5:
                    lam_dn.append(float(p[3]))
                    occ_dn.append(float(p[4]))
    # spin-major as the reference's lambda array (n + k Ns + spin Nk Ns); occupations as
    # printed (occ * 2 / (Nspin Nspinor))
    out["lambda"] = lam + lam_dn
    out["occ"] = occ + occ_dn
    with open(base + ".out") as fh:
        for line in fh:
            if line.startswith("Net magnetization"):
                out["net_mag"] = float(line.split(":")[1].split()[0])
    forces = []
    with open(base + ".static") as fh:
        lines = fh.read().splitlines()
    for i, line in enumerate(lines):
        if line.startswith("Atomic forces"):
            for l2 in lines[i + 1:]:
                p = l2.split()
                if len(p) != 3:
                    break
                forces.append([float(v) for v in p])
    out["forces"] = forces
    return out
