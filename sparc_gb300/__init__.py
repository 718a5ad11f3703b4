"""Python host layer over libsparc_gpu.so, the GB300 CheFSI hot-path library.

This mirrors the C ABI in include/sparc_gpu.h one to one (names follow the reference SPARC
functions they replace) so that tests and benchmarks read like calls into the reference.
There is no CPU fallback: if the CUDA library is missing, importing `lib()` raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsparc_gpu.so")

SGPU_OK = 0
SGPU_PREC_FP64 = 64
SGPU_PREC_FP32 = 32
STENCIL_VARIANTS = 11  # SGPU_STENCIL_VARIANTS

# every entry point declared in include/sparc_gpu.h
EXPORTED = [
    "sgpu_last_error", "sgpu_version", "sgpu_create", "sgpu_destroy", "sgpu_set_veff",
    "sgpu_set_nonlocal", "sgpu_Lap_plus_diag_vec_mult_orth", "sgpu_Lap_vec_mult",
    "sgpu_Vnl_vec_mult", "sgpu_Hamiltonian_vectors_mult", "sgpu_ChebyshevFiltering",
    "sgpu_poisson_residual", "sgpu_last_filter_ms", "sgpu_profile_enable", "sgpu_profile_read",
    "sgpu_ChebyshevFiltering_f32", "sgpu_get_stream", "sgpu_Project_Hamiltonian",
    "sgpu_Solve_Generalized_EigenProblem", "sgpu_Subspace_Rotation", "sgpu_Lanczos",
    "sgpu_CalculateDensity_psi", "sgpu_Calculate_Vxc_LDA_PW", "sgpu_AAR",
    "sgpu_Calculate_elecstPotential", "sgpu_Mixing_init", "sgpu_Mixing_periodic_pulay",
    "sgpu_Evaluate_scf_error", "sgpu_scf", "sgpu_scf_kpt", "sgpu_Vnl_vec_mult_noalloc",
    "sgpu_Calculate_Vxc_LSDA_PW", "sgpu_Mixing_init_spin", "sgpu_Mixing_periodic_pulay_spin",
    "sgpu_Generate_InitialMagnetization", "sgpu_set_zstencil_pairs", "sgpu_set_rr_batched",
    "sgpu_set_kpoint_geometry", "sgpu_Lap_plus_diag_vec_mult_orth_kpt", "sgpu_Vnl_vec_mult_kpt",
    "sgpu_Hamiltonian_vectors_mult_kpt", "sgpu_ChebyshevFiltering_kpt", "sgpu_set_psd",
    "sgpu_Calculate_PseudochargeCutoff", "sgpu_Generate_PseudoChargeDensity",
    "sgpu_CalculateNonlocalProjectors", "sgpu_autotune", "sgpu_set_stencil_variant",
    "sgpu_ChebyshevFiltering_batched", "sgpu_set_grid_coeffs", "sgpu_density_descriptors",
    "sgpu_mlp_create", "sgpu_mlp_destroy", "sgpu_mlp_nparam", "sgpu_mlp_get", "sgpu_mlp_set",
    "sgpu_mlp_forward", "sgpu_mlp_loss_grad", "sgpu_mlp_zero_grad", "sgpu_mlp_adam_step",
    "sgpu_Project_Hamiltonian_std", "sgpu_Solve_Standard_EigenProblem",
    "sgpu_set_nonlocal_apply_variant", "sgpu_set_nonlocal_project_variant", "sgpu_get_variants",
    "sgpu_get_tuning", "sgpu_Calculate_local_forces", "sgpu_Calculate_nonlocal_forces",
    "sgpu_Calculate_forces_xc", "sgpu_Gradient_vectors_dir", "sgpu_Symmetrize_forces",
    "sgpu_kernel_status", "sgpu_check_wait_bound", "sgpu_set_nonlocal_fuse",
    "sgpu_get_nonlocal_fuse", "sgpu_get_nonlocal_fuse_tc", "sgpu_ChebyshevFiltering_y", "sgpu_Project_Hamiltonian_f32",
    "sgpu_Subspace_Rotation_f32", "sgpu_set_gemm_emulation", "sgpu_measure_fp64_rate",
    "sgpu_set_rr_products", "sgpu_set_eig_solver", "sgpu_Project_Hamiltonian_kpt",
    "sgpu_Solve_Generalized_EigenProblem_kpt", "sgpu_Subspace_Rotation_kpt", "sgpu_CheFSI_batched",
]


class FilterBlock(ctypes.Structure):
    """sgpu_filter_block (include/sparc_gpu.h)."""
    _fields_ = [("spin", ctypes.c_int), ("k", ctypes.c_double * 3), ("X", ctypes.c_void_p),
                ("ldi", ctypes.c_int), ("Y", ctypes.c_void_p), ("ldo", ctypes.c_int),
                ("ncol", ctypes.c_int), ("a", ctypes.c_double), ("b", ctypes.c_double),
                ("a0", ctypes.c_double)]


class Psd(ctypes.Structure):
    """sgpu_psd (include/sparc_gpu.h): one atom type's radial tables."""
    _fields_ = [("size", ctypes.c_int), ("lmax", ctypes.c_int), ("lloc", ctypes.c_int),
                ("Znucl", ctypes.c_int), ("ppl", ctypes.c_void_p), ("rc", ctypes.c_void_p),
                ("Vloc_0", ctypes.c_double), ("fchrg", ctypes.c_double),
                ("RadialGrid", ctypes.c_void_p), ("UdV", ctypes.c_void_p),
                ("rVloc", ctypes.c_void_p), ("rhoIsoAtom", ctypes.c_void_p),
                ("rho_c_table", ctypes.c_void_p), ("Gamma", ctypes.c_void_p)]

SGPU_ERR_NOT_CONVERGED = 5


class ScfParams(ctypes.Structure):
    """sgpu_scf_params (include/sparc_gpu.h)."""
    _fields_ = [("Nstates", ctypes.c_int), ("n_atom", ctypes.c_int),
                ("Nelectron", ctypes.c_double), ("Beta", ctypes.c_double),
                ("elec_T_type", ctypes.c_int), ("cheb_degree", ctypes.c_int),
                ("rho_trigger", ctypes.c_int), ("nchefsi", ctypes.c_int),
                ("tol_scf", ctypes.c_double), ("tol_poisson", ctypes.c_double),
                ("tol_precond", ctypes.c_double), ("tol_lanczos", ctypes.c_double),
                ("maxit_scf", ctypes.c_int), ("minit_scf", ctypes.c_int),
                ("maxit_poisson", ctypes.c_int), ("mixing_history", ctypes.c_int),
                ("pulay_freq", ctypes.c_int), ("pulay_restart", ctypes.c_int),
                ("mixing_param", ctypes.c_double), ("mixing_param_simple", ctypes.c_double),
                ("kerker", ctypes.c_int), ("kerker_kTF", ctypes.c_double),
                ("kerker_idiemac", ctypes.c_double), ("xc_rhotol", ctypes.c_double),
                ("Esc", ctypes.c_double), ("precision", ctypes.c_int),
                ("fp64_switch_error", ctypes.c_double), ("graded_tail", ctypes.c_int),
                ("tail_fp64_degrees", ctypes.c_int), ("seed", ctypes.c_ulonglong),
                ("verbose", ctypes.c_int), ("history", ctypes.c_void_p),
                ("psi_out", ctypes.c_void_p), ("phi_out", ctypes.c_void_p),
                ("vxc_out", ctypes.c_void_p), ("spin_typ", ctypes.c_int),
                ("mag_init", ctypes.c_void_p), ("mixing_param_mag", ctypes.c_double),
                ("mixing_param_simple_mag", ctypes.c_double), ("mag_out", ctypes.c_void_p)]


class ScfResult(ctypes.Structure):
    """sgpu_scf_result (include/sparc_gpu.h)."""
    _fields_ = [("scf_iters", ctypes.c_int), ("converged", ctypes.c_int),
                ("fp64_switch_iter", ctypes.c_int), ("Etot", ctypes.c_double),
                ("Eband", ctypes.c_double), ("E1", ctypes.c_double), ("E2", ctypes.c_double),
                ("E3", ctypes.c_double), ("Exc", ctypes.c_double), ("Esc", ctypes.c_double),
                ("Entropy", ctypes.c_double), ("Efermi", ctypes.c_double),
                ("scf_error", ctypes.c_double), ("time_s", ctypes.c_double),
                ("filter_ms", ctypes.c_double), ("net_mag", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}

KERNEL_STENCIL, KERNEL_NL_PROJECT, KERNEL_NL_APPLY, KERNEL_OTHER, KERNEL_KINDS = range(5)

_lib = None
_vp = ctypes.c_void_p


class SgpuError(RuntimeError):
    pass


def lib():
    """Load libsparc_gpu.so (built by sparc_gb300/build.py); raise if it is absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise SgpuError(f"{LIB_PATH} is missing: run sparc_gb300/build.py (no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        L.sgpu_last_error.restype = ctypes.c_char_p
        for name in EXPORTED:
            if name != "sgpu_last_error":
                getattr(L, name).restype = ctypes.c_int
        _lib = L
    return _lib


def _check(rc):
    if rc != SGPU_OK:
        raise SgpuError(f"status {rc}: {lib().sgpu_last_error().decode()}")


def _ptr(a):
    """Raw pointer of a numpy array or a torch tensor (host or device). The library runs on
    its own CUDA stream, so work torch queued on a device tensor's current stream is waited
    for first: the call then reads the finished tensor (each call synchronises its own stream
    before returning, so its results are ready for torch afterwards)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return _vp(a.ctypes.data)
    if getattr(a, "is_cuda", False):
        import torch
        torch.cuda.current_stream(a.device).synchronize()
    return _vp(a.data_ptr())


class Context:
    """Device-resident state the reference reads from SPARC_OBJ (grid, FD weights, Veff,
    nonlocal projectors), behind an sgpu_ctx."""

    def __init__(self, Nx, Ny, Nz, FDn, cx, cy, cz, dV, device=0):
        self.Nx, self.Ny, self.Nz = int(Nx), int(Ny), int(Nz)
        self.Nd = self.Nx * self.Ny * self.Nz
        self._h = _vp()
        cx, cy, cz = (np.ascontiguousarray(c, dtype=np.float64) for c in (cx, cy, cz))
        _check(lib().sgpu_create(ctypes.byref(self._h), int(device), self.Nx, self.Ny, self.Nz,
                                 int(FDn), _ptr(cx), _ptr(cy), _ptr(cz), ctypes.c_double(dV)))

    def close(self):
        if self._h:
            lib().sgpu_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- set-up
    def set_veff(self, veff, nspin=1):
        v = np.ascontiguousarray(veff, dtype=np.float64) if isinstance(veff, np.ndarray) else veff
        _check(lib().sgpu_set_veff(self._h, int(nspin), _ptr(v)))

    def set_nonlocal(self, ip_displ, gamma, img_atom, img_ndc, grid_pos, chi):
        arrs = [np.ascontiguousarray(ip_displ, dtype=np.int32),
                np.ascontiguousarray(gamma, dtype=np.float64),
                np.ascontiguousarray(img_atom, dtype=np.int32),
                np.ascontiguousarray(img_ndc, dtype=np.int32),
                np.ascontiguousarray(grid_pos, dtype=np.int32),
                np.ascontiguousarray(chi, dtype=np.float64)]
        _check(lib().sgpu_set_nonlocal(self._h, len(arrs[0]) - 1, _ptr(arrs[0]), _ptr(arrs[1]),
                                       len(arrs[2]), _ptr(arrs[2]), _ptr(arrs[3]), _ptr(arrs[4]),
                                       _ptr(arrs[5])))
        self._natom_nl = len(arrs[0]) - 1

    def set_grid_coeffs(self, cx, cy, cz, dV):
        cx, cy, cz = (np.ascontiguousarray(c, dtype=np.float64) for c in (cx, cy, cz))
        _check(lib().sgpu_set_grid_coeffs(self._h, _ptr(cx), _ptr(cy), _ptr(cz),
                                          ctypes.c_double(dV)))

    def density_descriptors(self, cell, atom_pos, desc, rcut=6.0, width=0.5):
        """24 descriptors per grid point into desc (device float32 tensor, Nd x 24)."""
        cell = np.ascontiguousarray(cell, dtype=np.float64)
        pos = np.ascontiguousarray(atom_pos, dtype=np.float64).reshape(-1)
        _check(lib().sgpu_density_descriptors(self._h, _ptr(cell), int(pos.size // 3), _ptr(pos),
                                              ctypes.c_double(rcut), ctypes.c_double(width),
                                              _ptr(desc)))

    # ---- per-geometry set-up (pseudopotential tables from sparc_gb300.psp8.read_psp8)
    def set_psd(self, tables):
        """Store the radial tables of each atom type (a list of read_psp8 dicts)."""
        keep, structs = [], []
        for t in tables:
            arrs = dict(ppl=np.ascontiguousarray(t["ppl"], dtype=np.int32))
            for k in ("rc", "RadialGrid", "UdV", "rVloc", "rhoIsoAtom", "rho_c_table", "Gamma"):
                arrs[k] = np.ascontiguousarray(t[k], dtype=np.float64)
            keep.append(arrs)
            structs.append(Psd(int(t["size"]), int(t["lmax"]), int(t["lloc"]), int(t["Znucl"]),
                               arrs["ppl"].ctypes.data, arrs["rc"].ctypes.data,
                               float(t["Vloc_0"]), float(t["fchrg"]),
                               *(arrs[k].ctypes.data for k in ("RadialGrid", "UdV", "rVloc",
                                                               "rhoIsoAtom", "rho_c_table",
                                                               "Gamma"))))
        arr = (Psd * len(structs))(*structs)
        _check(lib().sgpu_set_psd(self._h, len(structs), arr))
        self._psd_keep = keep

    def Calculate_PseudochargeCutoff(self, cell, tol):
        cell = np.ascontiguousarray(cell, dtype=np.float64)
        out = np.zeros(3 * len(self._psd_keep))
        _check(lib().sgpu_Calculate_PseudochargeCutoff(self._h, _ptr(cell), ctypes.c_double(tol),
                                                       _ptr(out)))
        return out.reshape(-1, 3)

    def Generate_PseudoChargeDensity(self, cell, nAtomv, atom_pos, ref_cutoff=0.5,
                                     net_charge=0, cutoff=None, want_bref=False):
        """Returns dict(b, b_ref, rho_at, rho_core, Esc, PosCharge, NegCharge) (host arrays)."""
        cell = np.ascontiguousarray(cell, dtype=np.float64)
        nat = np.ascontiguousarray(nAtomv, dtype=np.int32)
        pos = np.ascontiguousarray(atom_pos, dtype=np.float64).reshape(-1)
        cut = None if cutoff is None else np.ascontiguousarray(cutoff, dtype=np.float64)
        b, rho, core = (np.zeros(self.Nd) for _ in range(3))
        bref = np.zeros(self.Nd) if want_bref else None
        sc = np.zeros(3)
        _check(lib().sgpu_Generate_PseudoChargeDensity(
            self._h, _ptr(cell), _ptr(nat), _ptr(pos), _ptr(cut), ctypes.c_double(ref_cutoff),
            int(net_charge), _ptr(b), _ptr(bref), _ptr(rho), _ptr(core), _ptr(sc)))
        return dict(b=b, b_ref=bref, rho_at=rho, rho_core=core, Esc=float(sc[0]),
                    PosCharge=float(sc[1]), NegCharge=float(sc[2]))

    def Generate_InitialMagnetization(self, cell, nAtomv, atom_pos, atom_spin_z, cutoff=None):
        """Initial magnetization density (Nd) of a collinear-spin run from per-atom spins."""
        cell = np.ascontiguousarray(cell, dtype=np.float64)
        nat = np.ascontiguousarray(nAtomv, dtype=np.int32)
        pos = np.ascontiguousarray(atom_pos, dtype=np.float64).reshape(-1)
        sp = np.ascontiguousarray(atom_spin_z, dtype=np.float64).reshape(-1)
        cut = None if cutoff is None else np.ascontiguousarray(cutoff, dtype=np.float64)
        mag = np.zeros(self.Nd)
        _check(lib().sgpu_Generate_InitialMagnetization(self._h, _ptr(cell), _ptr(nat), _ptr(pos),
                                                        _ptr(cut), _ptr(sp), _ptr(mag)))
        return mag

    def CalculateNonlocalProjectors(self, cell, nAtomv, atom_pos):
        cell = np.ascontiguousarray(cell, dtype=np.float64)
        nat = np.ascontiguousarray(nAtomv, dtype=np.int32)
        pos = np.ascontiguousarray(atom_pos, dtype=np.float64).reshape(-1)
        _check(lib().sgpu_CalculateNonlocalProjectors(self._h, _ptr(cell), _ptr(nat), _ptr(pos)))
        self._natom_nl = int(nat.sum())

    # ---- forces (src/forces.c)
    def Calculate_local_forces(self, cell, nAtomv, atom_pos, phi, ref_cutoff=0.5, cutoff=None):
        """Local force components, (n_atom, 3)."""
        cell = np.ascontiguousarray(cell, dtype=np.float64)
        nat = np.ascontiguousarray(nAtomv, dtype=np.int32)
        pos = np.ascontiguousarray(atom_pos, dtype=np.float64).reshape(-1)
        cut = None if cutoff is None else np.ascontiguousarray(cutoff, dtype=np.float64)
        f = np.zeros(3 * int(nat.sum()))
        _check(lib().sgpu_Calculate_local_forces(
            self._h, _ptr(cell), _ptr(nat), _ptr(pos), _ptr(cut), ctypes.c_double(ref_cutoff),
            _ptr(np.ascontiguousarray(phi, dtype=np.float64)), _ptr(f)))
        return f.reshape(-1, 3)

    def Calculate_nonlocal_forces(self, cell, X, occ, occfac=2.0):
        """Nonlocal force components of the projector atoms from orbitals X (ncol, Nd)."""
        cell = np.ascontiguousarray(cell, dtype=np.float64)
        ncol, ld = self._ncol_ld(X)
        occ = np.ascontiguousarray(occ, dtype=np.float64)
        f = np.zeros(3 * self._nl_natom())
        _check(lib().sgpu_Calculate_nonlocal_forces(self._h, ncol, _ptr(X), ld, _ptr(occ),
                                                    ctypes.c_double(occfac), _ptr(cell), _ptr(f)))
        return f.reshape(-1, 3)

    def Calculate_forces_xc(self, cell, nAtomv, atom_pos, vxc, cutoff=None):
        """Core-correction (NLCC) force components, (n_atom, 3)."""
        cell = np.ascontiguousarray(cell, dtype=np.float64)
        nat = np.ascontiguousarray(nAtomv, dtype=np.int32)
        pos = np.ascontiguousarray(atom_pos, dtype=np.float64).reshape(-1)
        cut = None if cutoff is None else np.ascontiguousarray(cutoff, dtype=np.float64)
        f = np.zeros(3 * int(nat.sum()))
        _check(lib().sgpu_Calculate_forces_xc(self._h, _ptr(cell), _ptr(nat), _ptr(pos), _ptr(cut),
                                              _ptr(np.ascontiguousarray(vxc, dtype=np.float64)),
                                              _ptr(f)))
        return f.reshape(-1, 3)

    def Gradient_vectors_dir(self, cell, x, dx, direction):
        cell = np.ascontiguousarray(cell, dtype=np.float64)
        ncol, ld = self._ncol_ld(x)
        _, ldo = self._ncol_ld(dx)
        _check(lib().sgpu_Gradient_vectors_dir(self._h, ncol, _ptr(cell), _ptr(x), ld, _ptr(dx),
                                               ldo, int(direction)))

    def _nl_natom(self):
        if getattr(self, "_natom_nl", None) is None:
            raise SgpuError("the number of projector atoms is not known: call set_nonlocal or "
                            "CalculateNonlocalProjectors first")
        return self._natom_nl

    # ---- hot path (x, y: (ncol, Nd) C-contiguous == Nd x ncol column-major, ld = Nd)
    def _ncol_ld(self, x):
        if x.ndim == 1:
            return 1, self.Nd
        return int(x.shape[0]), int(x.shape[1]) if isinstance(x, np.ndarray) else int(x.stride(0))

    def Lap_plus_diag_vec_mult_orth(self, a, b, c, v, x, y):
        ncol, ld = self._ncol_ld(x)
        _check(lib().sgpu_Lap_plus_diag_vec_mult_orth(
            self._h, ncol, ctypes.c_double(a), ctypes.c_double(b), ctypes.c_double(c), _ptr(v),
            _ptr(x), ld, _ptr(y), ld))
        return y

    def Lap_vec_mult(self, c, x, y):
        ncol, ld = self._ncol_ld(x)
        _check(lib().sgpu_Lap_vec_mult(self._h, ncol, ctypes.c_double(c), _ptr(x), ld, _ptr(y),
                                       ld))
        return y

    def Vnl_vec_mult(self, x, hx):
        ncol, ld = self._ncol_ld(x)
        _check(lib().sgpu_Vnl_vec_mult(self._h, ncol, _ptr(x), ld, _ptr(hx), ld))
        return hx

    def Hamiltonian_vectors_mult(self, c, x, hx, spin=0):
        ncol, ld = self._ncol_ld(x)
        _check(lib().sgpu_Hamiltonian_vectors_mult(self._h, int(spin), ncol, ctypes.c_double(c),
                                                   _ptr(x), ld, _ptr(hx), ld))
        return hx

    def ChebyshevFiltering(self, X, Y, m, a, b, a0, spin=0, precision=SGPU_PREC_FP64):
        ncol, ld = self._ncol_ld(X)
        _check(lib().sgpu_ChebyshevFiltering(self._h, int(spin), _ptr(X), ld, _ptr(Y), ld, ncol,
                                             int(m), ctypes.c_double(a), ctypes.c_double(b),
                                             ctypes.c_double(a0), int(precision)))
        return X, Y

    def ChebyshevFiltering_y(self, X, Y, m, a, b, a0, spin=0, precision=SGPU_PREC_FP64):
        """The filter with the host block X as input only (left unchanged); Y gets the result."""
        ncol, ld = self._ncol_ld(X)
        _check(lib().sgpu_ChebyshevFiltering_y(self._h, int(spin), _ptr(X), ld, _ptr(Y), ld,
                                               ncol, int(m), ctypes.c_double(a),
                                               ctypes.c_double(b), ctypes.c_double(a0),
                                               int(precision)))
        return Y

    def set_gemm_emulation(self, mode):
        """FP32-block products: 0 cuBLAS FP32 GEMM (BF16x9 emulation where cuBLAS expects a
        gain), 1 the same with eager emulation, 2 three-part BF16 split on the tensor cores."""
        _check(lib().sgpu_set_gemm_emulation(self._h, int(mode)))

    def Project_Hamiltonian_f32(self, Y, HY, Hp, Mp, spin=0):
        """FP32 device blocks Y, HY (ncol, Nd); Hp, Mp (ncol, ncol) FP64."""
        ncol, ld = self._ncol_ld(Y)
        _check(lib().sgpu_Project_Hamiltonian_f32(self._h, int(spin), _ptr(Y), ld, _ptr(HY), ld,
                                                  ncol, _ptr(Hp), _ptr(Mp)))
        return Hp, Mp

    def Subspace_Rotation_f32(self, Y, Q, X):
        """X = Y Q on FP32 device blocks (ncol, Nd); Q (ncol, ncol) FP64."""
        ncol, ld = self._ncol_ld(Y)
        _check(lib().sgpu_Subspace_Rotation_f32(self._h, _ptr(Y), ld, _ptr(Q), ncol, _ptr(X), ld))
        return X

    def ChebyshevFiltering_f32(self, X, Y, m, a, b, a0, spin=0):
        ncol, ld = self._ncol_ld(X)
        _check(lib().sgpu_ChebyshevFiltering_f32(self._h, int(spin), _ptr(X), ld, _ptr(Y), ld,
                                                 ncol, int(m), ctypes.c_double(a),
                                                 ctypes.c_double(b), ctypes.c_double(a0)))
        return X, Y

    def stream(self):
        """The context's cudaStream_t as an integer handle."""
        s = _vp()
        _check(lib().sgpu_get_stream(self._h, ctypes.byref(s)))
        return int(s.value or 0)

    def poisson_residual(self, c, x, b, r):
        _check(lib().sgpu_poisson_residual(self._h, ctypes.c_double(c), _ptr(x), _ptr(b),
                                           _ptr(r)))
        return r

    # ---- k-point rows (complex128 numpy arrays (ncol, Nd) or complex torch tensors)
    def set_kpoint_geometry(self, L, img_coords):
        ic = np.ascontiguousarray(img_coords, dtype=np.float64).reshape(-1)
        _check(lib().sgpu_set_kpoint_geometry(self._h, ctypes.c_double(L[0]),
                                              ctypes.c_double(L[1]), ctypes.c_double(L[2]),
                                              int(ic.size // 3), _ptr(ic)))

    @staticmethod
    def _kvec(k):
        return np.ascontiguousarray(k, dtype=np.float64)

    def Lap_plus_diag_vec_mult_orth_kpt(self, k, a, b, c, v, x, y):
        ncol, ld = self._ncol_ld(x)
        kv = self._kvec(k)
        _check(lib().sgpu_Lap_plus_diag_vec_mult_orth_kpt(
            self._h, _ptr(kv), ncol, ctypes.c_double(a), ctypes.c_double(b), ctypes.c_double(c),
            _ptr(v), _ptr(x), ld, _ptr(y), ld))
        return y

    def Vnl_vec_mult_kpt(self, k, x, hx):
        ncol, ld = self._ncol_ld(x)
        kv = self._kvec(k)
        _check(lib().sgpu_Vnl_vec_mult_kpt(self._h, _ptr(kv), ncol, _ptr(x), ld, _ptr(hx), ld))
        return hx

    def Hamiltonian_vectors_mult_kpt(self, k, c, x, hx, spin=0):
        ncol, ld = self._ncol_ld(x)
        kv = self._kvec(k)
        _check(lib().sgpu_Hamiltonian_vectors_mult_kpt(self._h, int(spin), _ptr(kv), ncol,
                                                       ctypes.c_double(c), _ptr(x), ld, _ptr(hx),
                                                       ld))
        return hx

    def ChebyshevFiltering_kpt(self, k, X, Y, m, a, b, a0, spin=0, precision=SGPU_PREC_FP64):
        ncol, ld = self._ncol_ld(X)
        kv = self._kvec(k)
        _check(lib().sgpu_ChebyshevFiltering_kpt(self._h, int(spin), _ptr(kv), _ptr(X), ld,
                                                 _ptr(Y), ld, ncol, int(m), ctypes.c_double(a),
                                                 ctypes.c_double(b), ctypes.c_double(a0),
                                                 int(precision)))
        return X, Y

    def ChebyshevFiltering_batched(self, blocks, m, precision=SGPU_PREC_FP64):
        """Filter several (k-point, spin) blocks in one call. blocks: list of dicts with spin,
        k (3), X, Y (device torch tensors of shape (ncol, Nd), complex128 for FP64 or
        complex64 for FP32) and the bounds a, b, a0."""
        arr = self._blocks(blocks)
        _check(lib().sgpu_ChebyshevFiltering_batched(self._h, len(blocks), arr, int(m),
                                                     int(precision)))

    def _blocks(self, blocks):
        arr = (FilterBlock * len(blocks))()
        for i, b in enumerate(blocks):
            X, Y = b["X"], b["Y"]
            ncol = int(X.shape[0]) if X.dim() == 2 else 1
            arr[i] = FilterBlock(int(b.get("spin", 0)), (ctypes.c_double * 3)(*b["k"]),
                                 _ptr(X).value, self.Nd, _ptr(Y).value, self.Nd, ncol,
                                 float(b["a"]), float(b["b"]), float(b["a0"]))
        return arr

    def CheFSI_batched(self, blocks, m, precision=SGPU_PREC_FP64):
        """One CheFSI pass over (k-point, spin) blocks (as ChebyshevFiltering_batched): the
        filter, then per block H Y, the projection, the generalized eigensolve and the
        rotation into X. Returns the Ritz values of every block (list of arrays)."""
        arr = self._blocks(blocks)
        ncols = [int(b["X"].shape[0]) if b["X"].dim() == 2 else 1 for b in blocks]
        lam = np.zeros(max(1, sum(ncols)))
        _check(lib().sgpu_CheFSI_batched(self._h, len(blocks), arr, int(m), int(precision),
                                         _ptr(lam)))
        out, off = [], 0
        for n in ncols:
            out.append(lam[off:off + n].copy())
            off += n
        return out

    def Project_Hamiltonian_kpt(self, k, Y, HY, Hp, Mp, spin=0):
        """Complex128 blocks (ncol, Nd) and Ns x Ns matrices (column-major C arrays)."""
        ncol, ld = self._ncol_ld(Y)
        kv = self._kvec(k)
        _check(lib().sgpu_Project_Hamiltonian_kpt(self._h, int(spin), _ptr(kv), _ptr(Y), ld,
                                                  _ptr(HY), ld, ncol, _ptr(Hp), _ptr(Mp)))
        return Hp, Mp

    def Solve_Generalized_EigenProblem_kpt(self, Hp, Mp, lam):
        _check(lib().sgpu_Solve_Generalized_EigenProblem_kpt(self._h, int(Hp.shape[0]),
                                                             _ptr(Hp), _ptr(Mp), _ptr(lam)))
        return Hp, lam

    def Subspace_Rotation_kpt(self, Y, Q, X):
        ncol, ld = self._ncol_ld(Y)
        _check(lib().sgpu_Subspace_Rotation_kpt(self._h, _ptr(Y), ld, _ptr(Q), ncol, _ptr(X),
                                                ld))
        return X

    # ---- Rayleigh-Ritz
    def Project_Hamiltonian(self, Y, HY, Hp, Mp, spin=0):
        ncol, ld = self._ncol_ld(Y)
        _check(lib().sgpu_Project_Hamiltonian(self._h, int(spin), _ptr(Y), ld, _ptr(HY), ld,
                                              ncol, _ptr(Hp), _ptr(Mp)))
        return Hp, Mp

    def Solve_Generalized_EigenProblem(self, Hp, Mp, lam):
        _check(lib().sgpu_Solve_Generalized_EigenProblem(self._h, int(Hp.shape[0]), _ptr(Hp),
                                                         _ptr(Mp), _ptr(lam)))
        return Hp, lam

    def Project_Hamiltonian_std(self, Y, HY, Hp, spin=0):
        """Y is overwritten by its Cholesky-orthonormalised block."""
        ncol, ld = self._ncol_ld(Y)
        _check(lib().sgpu_Project_Hamiltonian_std(self._h, int(spin), _ptr(Y), ld, _ptr(HY),
                                                  ld, ncol, _ptr(Hp)))
        return Y, HY, Hp

    def Solve_Standard_EigenProblem(self, Hp, lam):
        _check(lib().sgpu_Solve_Standard_EigenProblem(self._h, int(Hp.shape[0]), _ptr(Hp),
                                                      _ptr(lam)))
        return Hp, lam

    def Subspace_Rotation(self, Y, Q, X):
        ncol, ld = self._ncol_ld(Y)
        _check(lib().sgpu_Subspace_Rotation(self._h, _ptr(Y), ld, _ptr(Q), ncol, _ptr(X), ld))
        return X

    def Lanczos(self, x0, tol=1e-2, maxit=1000, spin=0):
        lo, hi = ctypes.c_double(), ctypes.c_double()
        x0 = np.ascontiguousarray(x0, dtype=np.float64)
        _check(lib().sgpu_Lanczos(self._h, int(spin), _ptr(x0), ctypes.c_double(tol),
                                  int(maxit), ctypes.byref(lo), ctypes.byref(hi)))
        return lo.value, hi.value

    # ---- SCF-side rows
    def CalculateDensity_psi(self, psi, occ, occfac, rho):
        ncol, ld = self._ncol_ld(psi)
        occ = np.ascontiguousarray(occ, dtype=np.float64)
        _check(lib().sgpu_CalculateDensity_psi(self._h, _ptr(psi), ld, ncol, _ptr(occ),
                                               ctypes.c_double(occfac), _ptr(rho)))
        return rho

    def Calculate_Vxc_LDA_PW(self, rho, rho_core, xc_rhotol, vxc, exc):
        _check(lib().sgpu_Calculate_Vxc_LDA_PW(self._h, _ptr(rho), _ptr(rho_core),
                                               ctypes.c_double(xc_rhotol), _ptr(vxc), _ptr(exc)))
        return vxc, exc

    def AAR(self, c, x, b, omega=0.6, beta=0.6, m=7, p=6, tol=1e-8, max_iter=3000):
        it = ctypes.c_int()
        rc = lib().sgpu_AAR(self._h, ctypes.c_double(c), _ptr(x), _ptr(b),
                            ctypes.c_double(omega), ctypes.c_double(beta), int(m), int(p),
                            ctypes.c_double(tol), int(max_iter), ctypes.byref(it))
        if rc not in (SGPU_OK, SGPU_ERR_NOT_CONVERGED):
            _check(rc)
        return it.value, rc == SGPU_OK

    def Calculate_elecstPotential(self, rho, b, phi, tol, max_iter=3000):
        it = ctypes.c_int()
        _check(lib().sgpu_Calculate_elecstPotential(self._h, _ptr(rho), _ptr(b), _ptr(phi),
                                                    ctypes.c_double(tol), int(max_iter),
                                                    ctypes.byref(it)))
        return it.value

    def Mixing_init(self, rho_in, neg_charge, history=7, pulay_frequency=1, pulay_restart=0,
                    mixing_parameter=0.3, mixing_parameter_simple=0.3, kerker=1, kTF=1.0,
                    idiemac=0.1, tol_precond=1e-4):
        _check(lib().sgpu_Mixing_init(self._h, int(history), int(pulay_frequency),
                                      int(pulay_restart), ctypes.c_double(mixing_parameter),
                                      ctypes.c_double(mixing_parameter_simple), int(kerker),
                                      ctypes.c_double(kTF), ctypes.c_double(idiemac),
                                      ctypes.c_double(tol_precond), ctypes.c_double(neg_charge),
                                      _ptr(rho_in)))

    def Calculate_Vxc_LSDA_PW(self, rho_up, rho_dn, rho_core, xc_rhotol, vxc, exc):
        """vxc: 2 x Nd (up, down); exc: Nd."""
        _check(lib().sgpu_Calculate_Vxc_LSDA_PW(self._h, _ptr(rho_up), _ptr(rho_dn),
                                                _ptr(rho_core), ctypes.c_double(xc_rhotol),
                                                _ptr(vxc), _ptr(exc)))
        return vxc, exc

    def Mixing_init_spin(self, rho_in, mag_in, neg_charge, history=7, pulay_frequency=1,
                         pulay_restart=0, mixing_parameter=0.3, mixing_parameter_simple=0.3,
                         mixing_parameter_mag=0.3, mixing_parameter_simple_mag=0.3, kerker=1,
                         kTF=1.0, idiemac=0.1, tol_precond=1e-4):
        _check(lib().sgpu_Mixing_init_spin(
            self._h, int(history), int(pulay_frequency), int(pulay_restart),
            ctypes.c_double(mixing_parameter), ctypes.c_double(mixing_parameter_simple),
            ctypes.c_double(mixing_parameter_mag), ctypes.c_double(mixing_parameter_simple_mag),
            int(kerker), ctypes.c_double(kTF), ctypes.c_double(idiemac),
            ctypes.c_double(tol_precond), ctypes.c_double(neg_charge), _ptr(rho_in),
            _ptr(mag_in)))

    def Mixing_periodic_pulay_spin(self, iter_count, rho, mag):
        _check(lib().sgpu_Mixing_periodic_pulay_spin(self._h, int(iter_count), _ptr(rho),
                                                     _ptr(mag)))
        return rho, mag

    def Mixing_periodic_pulay(self, iter_count, rho):
        _check(lib().sgpu_Mixing_periodic_pulay(self._h, int(iter_count), _ptr(rho)))
        return rho

    def Evaluate_scf_error(self, rho_out, rho_in):
        e = ctypes.c_double()
        _check(lib().sgpu_Evaluate_scf_error(self._h, _ptr(rho_out), _ptr(rho_in),
                                             ctypes.byref(e)))
        return e.value

    def scf(self, params, b, rho_init, rho_core=None, Nstates=None, fields=None):
        """Run sgpu_scf; returns (result dict, final density, eigenvalues, occupations). With
        fields a dict, it also receives the final orbitals ("psi", Nstates x Nd), the
        electrostatic potential ("phi") and the exchange-correlation potential ("vxc")."""
        Ns = params.Nstates
        rho = np.zeros(self.Nd)
        lam = np.zeros(Ns)
        occ = np.zeros(Ns)
        res = ScfResult()
        b = np.ascontiguousarray(b, dtype=np.float64)
        r0 = np.ascontiguousarray(rho_init, dtype=np.float64)
        rc_ = None if rho_core is None else np.ascontiguousarray(rho_core, dtype=np.float64)
        hist = np.full(3 * max(1, params.maxit_scf), np.nan)
        params.history = hist.ctypes.data
        if fields is not None:
            fields["psi"] = np.zeros((Ns, self.Nd))
            fields["phi"] = np.zeros(self.Nd)
            fields["vxc"] = np.zeros(self.Nd)
            params.psi_out = fields["psi"].ctypes.data
            params.phi_out = fields["phi"].ctypes.data
            params.vxc_out = fields["vxc"].ctypes.data
        try:
            _check(lib().sgpu_scf(self._h, ctypes.byref(params), _ptr(b), _ptr(r0), _ptr(rc_),
                                  _ptr(rho), _ptr(lam), _ptr(occ), ctypes.byref(res)))
        finally:
            params.history = None
            params.psi_out = params.phi_out = params.vxc_out = None
        out = res.as_dict()
        h = hist.reshape(-1, 3)[:out["scf_iters"]]
        out["history"] = {"Etot": h[:, 0].tolist(), "scf_error": h[:, 1].tolist(),
                          "time_s": h[:, 2].tolist()}
        return out, rho, lam, occ

    def scf_kpt(self, params, kpts, kpt_wts, b, rho_init, rho_core=None, fields=None,
                mag_init=None):
        """Run sgpu_scf_kpt on the k-points kpts (nkpt x 3, Cartesian 1/Bohr) with weights
        kpt_wts (as the reference's kptWts_loc); returns (result dict, final density,
        eigenvalues nblk x Nstates, occupations nblk x Nstates), nblk = nkpt, or 2 nkpt with
        collinear spin (mag_init given: the initial magnetization; blocks spin-major). With
        fields a dict, it also receives the final orbitals ("psi", nblk x Nstates x Nd
        complex128), "phi", "vxc" (nspin x Nd) and, with spin, the magnetization "mag"."""
        Ns = params.Nstates
        kp = np.ascontiguousarray(kpts, dtype=np.float64).reshape(-1, 3)
        wt = np.ascontiguousarray(kpt_wts, dtype=np.float64).reshape(-1)
        nk = kp.shape[0]
        if wt.shape[0] != nk:
            raise ValueError("one weight per k-point")
        mag0 = None if mag_init is None else np.ascontiguousarray(mag_init, dtype=np.float64)
        nspin = 1 if mag0 is None else 2
        rho = np.zeros(self.Nd)
        lam = np.zeros((nspin * nk, Ns))
        occ = np.zeros((nspin * nk, Ns))
        res = ScfResult()
        b = np.ascontiguousarray(b, dtype=np.float64)
        r0 = np.ascontiguousarray(rho_init, dtype=np.float64)
        rc_ = None if rho_core is None else np.ascontiguousarray(rho_core, dtype=np.float64)
        hist = np.full(3 * max(1, params.maxit_scf), np.nan)
        params.history = hist.ctypes.data
        params.spin_typ = nspin - 1
        params.mag_init = None if mag0 is None else mag0.ctypes.data
        if fields is not None:
            fields["psi"] = np.zeros((nspin * nk, Ns, self.Nd), dtype=np.complex128)
            fields["phi"] = np.zeros(self.Nd)
            fields["vxc"] = np.zeros((nspin, self.Nd))
            params.psi_out = fields["psi"].ctypes.data
            params.phi_out = fields["phi"].ctypes.data
            params.vxc_out = fields["vxc"].ctypes.data
            if nspin == 2:
                fields["mag"] = np.zeros(self.Nd)
                params.mag_out = fields["mag"].ctypes.data
        try:
            _check(lib().sgpu_scf_kpt(self._h, ctypes.byref(params), int(nk), _ptr(kp), _ptr(wt),
                                      _ptr(b), _ptr(r0), _ptr(rc_), _ptr(rho), _ptr(lam),
                                      _ptr(occ), ctypes.byref(res)))
        finally:
            params.history = None
            params.psi_out = params.phi_out = params.vxc_out = params.mag_out = None
            params.mag_init = None
        out = res.as_dict()
        h = hist.reshape(-1, 3)[:out["scf_iters"]]
        out["history"] = {"Etot": h[:, 0].tolist(), "scf_error": h[:, 1].tolist(),
                          "time_s": h[:, 2].tolist()}
        return out, rho, lam, occ

    def autotune(self, ncol=64):
        """Time the FP32 stencil variants; returns (chosen variant, per-variant ms)."""
        v = ctypes.c_int()
        ms = np.zeros(STENCIL_VARIANTS)
        _check(lib().sgpu_autotune(self._h, int(ncol), ctypes.byref(v), _ptr(ms)))
        return int(v.value), ms

    def set_stencil_variant(self, variant):
        _check(lib().sgpu_set_stencil_variant(self._h, int(variant)))

    def set_rr_batched(self, on):
        _check(lib().sgpu_set_rr_batched(self._h, int(bool(on))))

    def set_zstencil_pairs(self, on):
        _check(lib().sgpu_set_zstencil_pairs(self._h, int(bool(on))))

    def set_nonlocal_apply_variant(self, variant):
        _check(lib().sgpu_set_nonlocal_apply_variant(self._h, int(variant)))

    def set_nonlocal_project_variant(self, variant):
        _check(lib().sgpu_set_nonlocal_project_variant(self._h, int(variant)))

    def variants(self):
        """The kernel forms in use: dict(stencil, nl_apply, nl_project)."""
        s, a, p = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(lib().sgpu_get_variants(self._h, ctypes.byref(s), ctypes.byref(a), ctypes.byref(p)))
        return dict(stencil=s.value, nl_apply=a.value, nl_project=p.value)

    def tuning(self):
        """Per-form milliseconds of the last autotune: dict(nl_apply=[5], nl_project=[2])."""
        a, p = np.zeros(5), np.zeros(2)
        _check(lib().sgpu_get_tuning(self._h, _ptr(a), _ptr(p)))
        return dict(nl_apply=a.tolist(), nl_project=p.tolist())

    def profile_enable(self, on=True):
        _check(lib().sgpu_profile_enable(self._h, int(bool(on))))

    def profile_read(self, kind):
        """(total device ms, launches) of one kernel kind since the last profile reset;
        kind == KERNEL_KINDS gives (0, kernels launched)."""
        ms = ctypes.c_double()
        n = ctypes.c_long()
        _check(lib().sgpu_profile_read(self._h, int(kind), ctypes.byref(ms), ctypes.byref(n)))
        return float(ms.value), int(n.value)

    def kernel_status(self):
        """Read and clear the kernel status word: 0 when no bounded wait of a kernel ran out
        (otherwise the call raises, the results since the last check being invalid)."""
        st = ctypes.c_int()
        _check(lib().sgpu_kernel_status(self._h, ctypes.byref(st)))
        return int(st.value)

    def set_nonlocal_fuse(self, on, cpl=None):
        """Carry the nonlocal projections across filter degrees (fused range apply) or not;
        cpl = 2 or 4 fixes the CUDA-core kernel's columns per thread, cpl = 3 selects the
        tensor-core kernel."""
        mode = 0 if not on else (int(cpl) if cpl else 1)
        _check(lib().sgpu_set_nonlocal_fuse(self._h, mode))

    def nonlocal_fuse_tc(self):
        """(whether the tensor-core fused form is available, ms of one launch at the last
        tuning)."""
        av = ctypes.c_int()
        ms = ctypes.c_double()
        _check(lib().sgpu_get_nonlocal_fuse_tc(self._h, ctypes.byref(av), ctypes.byref(ms)))
        return bool(av.value), float(ms.value)

    def nonlocal_fuse(self):
        """(on, columns per thread of the fused form or 0, [ms of one fused launch with 2 and
        4 columns per thread at the last tuning])."""
        mode = ctypes.c_int()
        ms = (ctypes.c_double * 2)()
        _check(lib().sgpu_get_nonlocal_fuse(self._h, ctypes.byref(mode), ms))
        return mode.value != 0, int(mode.value), [float(ms[0]), float(ms[1])]

    def set_rr_products(self, mode):
        """Rayleigh-Ritz products: 1 tensor-core split slices for FP32 blocks and the mixed
        SCF's FP64 phase, 2 also for plain FP64 calls, 0 cuBLAS (sgpu_set_rr_products)."""
        _check(lib().sgpu_set_rr_products(self._h, int(mode)))

    def set_eig_solver(self, mode):
        """Subspace eigensolver: 0 dsygvd, 1 Cholesky reduction + dsyevd, 2 reduction +
        Jacobi dsyevj (sgpu_set_eig_solver)."""
        _check(lib().sgpu_set_eig_solver(self._h, int(mode)))

    def measure_fp64_rate(self):
        """This GPU's FP64 FMA rate in TFLOP/s (sgpu_measure_fp64_rate)."""
        t = ctypes.c_double()
        _check(lib().sgpu_measure_fp64_rate(self._h, ctypes.byref(t)))
        return float(t.value)

    def check_wait_bound(self):
        """Run the bounded-wait diagnostic; returns the status word it left (2 when a wait
        that nothing completes runs out as it should)."""
        st = ctypes.c_int()
        _check(lib().sgpu_check_wait_bound(self._h, ctypes.byref(st)))
        return int(st.value)

    def last_filter_ms(self):
        ms = ctypes.c_float()
        _check(lib().sgpu_last_filter_ms(self._h, ctypes.byref(ms)))
        return float(ms.value)
