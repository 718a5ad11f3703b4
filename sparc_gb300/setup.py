"""Host side of the per-geometry set-up for a periodic orthogonal cell: the grid and FD
weights, the defaults the reference derives from its input, and the device set-up calls.

Mirrors the parts of the reference's Initialize (src/initialization.c) that the CheFSI SCF
reads: the grid from MESH_SPACING (numIntervals = max(ceil(L/mesh), FDn), :1935-1938), the
second-derivative FD weights (:2112-2146), TOL_PSEUDOCHARGE = 1e-3 TOL_SCF (:2607),
TOL_POISSON = 1e-2 TOL_SCF (:2595), TOL_PRECOND = h^2 1e-3 (:2578), REFERENCE_CUTOFF = 0.5
(:745), rhoTrigger = 4 (:2263), and the SCF defaults of :726-814; then the set-up entry points
of the library (pseudocharge cut-offs, pseudocharge and initial densities, projectors).
Atom coordinates are taken as the reference reads them from a .ion file written with 12
decimals, so that both programs see the same numbers.
"""
import math

import numpy as np

from . import Context, ScfParams, SGPU_PREC_FP64
from .synthetic import fd_d2_coeffs


def grid_from_mesh(L, mesh_spacing, FDn=6):
    """Grid points per direction of a periodic cell for a target mesh spacing."""
    return tuple(max(int(math.ceil(Li / mesh_spacing)), FDn) for Li in L)


def ion_coordinates(pos, L=None, exact=False):
    """Coordinates as a 12-decimal .ion file carries them (exact: as given, e.g. fractional
    coordinates already multiplied by the cell lengths, as the reader does for COORD_FRAC,
    src/readfiles.c:1665-1670); with the cell lengths L, mapped into [0, L) per direction as
    the reference does for periodic directions (src/initialization.c:2013-2023:
    x = fmod(x, L) + (x < 0) L when x < 0 or x >= L)."""
    if exact:
        out = np.array(pos, dtype=np.float64).copy()
    else:
        out = np.array([[float(f"{v:.12f}") for v in p] for p in np.asarray(pos)],
                       dtype=np.float64)
    if L is not None:
        for d in range(3):
            for i in range(out.shape[0]):
                x = out[i, d]
                if x < 0 or x >= L[d]:
                    x = math.fmod(x, L[d])
                    out[i, d] = x + (L[d] if x < 0.0 else 0.0)
    return out


class CellSystem:
    """A periodic orthogonal cell with its atoms on the device: the library context (grid,
    FD weights, nonlocal projectors) and the set-up fields an SCF starts from."""

    def __init__(self, L, N, species, tables, tol_scf=1e-6, ref_cutoff=0.5, net_charge=0,
                 FDn=6, device=0, exact_coords=False):
        """species: list of (symbol, positions (n, 3) Bohr); tables: {symbol: read_psp8
        dict}. Atoms are ordered type by type, as the reference orders them. Positions are
        taken as a 12-decimal Cartesian .ion file carries them, or as given with exact_coords
        (fractional coordinates times the cell lengths)."""
        self.exact_coords = exact_coords
        self.N = tuple(int(n) for n in N)
        self.FDn = FDn
        self.tables = [tables[s] for s, _ in species]
        self.tol_scf = tol_scf
        self.ref_cutoff = ref_cutoff
        self.net_charge = net_charge
        self.nlcc = any(float(t["fchrg"]) > 1e-12 for t in self.tables)
        self._grid(L)
        self.ctx = Context(*self.N, FDn, self.cx, self.cy, self.cz, self.dV, device=device)
        self.ctx.set_psd(self.tables)
        self.set_geometry(L, species)

    def _grid(self, L):
        self.L = np.asarray(L, dtype=np.float64)
        self.h = self.L / np.array(self.N)
        self.dV = float(np.prod(self.h))
        self.cx, self.cy, self.cz = (fd_d2_coeffs(self.FDn, hh) for hh in self.h)

    def set_geometry(self, L, species):
        """New cell lengths (same grid) and atom positions (same species and counts): the FD
        weights, pseudocharge cut-offs, set-up fields and projectors are rebuilt on the
        existing context."""
        if np.any(np.asarray(L, dtype=np.float64) != getattr(self, "L", None)):
            self._grid(L)
            self.ctx.set_grid_coeffs(self.cx, self.cy, self.cz, self.dV)
        self.nAtomv = np.array([len(p) for _, p in species], dtype=np.int32)
        self.n_atom = int(self.nAtomv.sum())
        self.atom_pos = np.concatenate([ion_coordinates(p, self.L, self.exact_coords)
                                        for _, p in species], axis=0)
        self.Nelectron = float(sum(int(t["Znucl"]) * n for t, n in zip(self.tables,
                                                                       self.nAtomv))) - self.net_charge
        self.cutoff = self.ctx.Calculate_PseudochargeCutoff(self.L, 1e-3 * self.tol_scf)
        self.fields = self.ctx.Generate_PseudoChargeDensity(
            self.L, self.nAtomv, self.atom_pos, ref_cutoff=self.ref_cutoff,
            net_charge=self.net_charge)
        self.ctx.CalculateNonlocalProjectors(self.L, self.nAtomv, self.atom_pos)

    def scf_params(self, Nstates, cheb_degree, smearing=1e-3, precision=SGPU_PREC_FP64,
                   fp64_switch_error=1e-4, graded_tail=0, tail_fp64_degrees=0, seed=1,
                   verbose=0, maxit_scf=100, elec_T_type=0):
        """sgpu_scf_params with the reference's defaults for this cell (smearing in Ha,
        Fermi-Dirac (elec_T_type 0) or Gaussian (1), density mixing with Kerker
        preconditioning, Pulay history 7)."""
        h_eff = float(self.h[0]) if np.ptp(self.h) < 1e-12 else \
            math.sqrt(3.0 / float(np.sum(1.0 / self.h ** 2)))
        p = ScfParams()
        p.Nstates = int(Nstates)
        p.n_atom = self.n_atom
        p.Nelectron = self.Nelectron
        p.Beta = 1.0 / smearing
        p.elec_T_type = int(elec_T_type)
        p.cheb_degree = int(cheb_degree)
        p.rho_trigger = 4
        p.nchefsi = 1
        p.tol_scf = self.tol_scf
        p.tol_poisson = 0.01 * self.tol_scf
        p.tol_precond = h_eff * h_eff * 1e-3
        p.tol_lanczos = 1e-2
        p.maxit_scf = maxit_scf
        p.minit_scf = 2
        p.maxit_poisson = 3000
        p.mixing_history = 7
        p.pulay_freq = 1
        p.pulay_restart = 0
        p.mixing_param = 0.3
        p.mixing_param_simple = 0.3
        p.kerker = 1
        p.kerker_kTF = 1.0
        p.kerker_idiemac = 0.1
        p.xc_rhotol = 1e-14
        p.Esc = self.fields["Esc"]
        p.precision = precision
        p.fp64_switch_error = fp64_switch_error
        p.graded_tail = int(graded_tail)
        p.tail_fp64_degrees = int(tail_fp64_degrees)
        p.seed = seed
        p.verbose = verbose
        return p

    def scf(self, params, rho_init=None, fields=None):
        """Run the SCF from the superposition of atomic densities (or from rho_init); with
        fields a dict, also return the final orbitals and potentials there (Context.scf)."""
        f = self.fields
        r0 = f["rho_at"] if rho_init is None else rho_init
        return self.ctx.scf(params, f["b"], r0, f["rho_core"] if self.nlcc else None,
                            fields=fields)

    def initial_magnetization(self, atom_spin_z):
        """The reference's initial magnetization for per-atom spins (type-major, as the
        atoms): sum over atoms of spin / Znucl times the isolated-atom density."""
        return self.ctx.Generate_InitialMagnetization(self.L, self.nAtomv, self.atom_pos,
                                                      atom_spin_z)

    def scf_kpt(self, params, kpts, kpt_wts, atom_spin_z=None, rho_init=None, fields=None):
        """k-point SCF (Context.scf_kpt) from the superposition of atomic densities (or
        rho_init); with atom_spin_z, collinear spin from the reference's initial
        magnetization of those moments."""
        f = self.fields
        r0 = f["rho_at"] if rho_init is None else rho_init
        mag = None if atom_spin_z is None else self.initial_magnetization(atom_spin_z)
        return self.ctx.scf_kpt(params, kpts, kpt_wts, f["b"], r0,
                                f["rho_core"] if self.nlcc else None, fields=fields,
                                mag_init=mag)

    def forces(self, fields, occ, occfac=2.0):
        """Atomic forces (n_atom, 3) in Ha/Bohr after an SCF that filled fields (psi, phi,
        vxc) and returned occ: local + nonlocal (+ core correction) with the mean removed, as
        Calculate_EGS_Forces (src/forces.c:49) assembles them."""
        F = self.ctx.Calculate_local_forces(self.L, self.nAtomv, self.atom_pos, fields["phi"],
                                            ref_cutoff=self.ref_cutoff)
        F = F + self.ctx.Calculate_nonlocal_forces(self.L, fields["psi"], occ, occfac)
        if self.nlcc:
            F = F + self.ctx.Calculate_forces_xc(self.L, self.nAtomv, self.atom_pos, fields["vxc"])
        return F - F.mean(axis=0)

    def close(self):
        self.ctx.close()
