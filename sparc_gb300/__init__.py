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

# every entry point declared in include/sparc_gpu.h
EXPORTED = [
    "sgpu_last_error", "sgpu_version", "sgpu_create", "sgpu_destroy", "sgpu_set_veff",
    "sgpu_set_nonlocal", "sgpu_Lap_plus_diag_vec_mult_orth", "sgpu_Lap_vec_mult",
    "sgpu_Vnl_vec_mult", "sgpu_Hamiltonian_vectors_mult", "sgpu_ChebyshevFiltering",
    "sgpu_poisson_residual", "sgpu_last_filter_ms", "sgpu_profile_enable", "sgpu_profile_read",
    "sgpu_ChebyshevFiltering_f32", "sgpu_get_stream",
]

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
    """Raw pointer of a numpy array or a torch tensor (host or device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return _vp(a.ctypes.data)
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

    def profile_enable(self, on=True):
        _check(lib().sgpu_profile_enable(self._h, int(bool(on))))

    def profile_read(self, kind):
        """(total device ms, launches) of one kernel kind since the last profile reset;
        kind == KERNEL_KINDS gives (0, kernels launched)."""
        ms = ctypes.c_double()
        n = ctypes.c_long()
        _check(lib().sgpu_profile_read(self._h, int(kind), ctypes.byref(ms), ctypes.byref(n)))
        return float(ms.value), int(n.value)

    def last_filter_ms(self):
        ms = ctypes.c_float()
        _check(lib().sgpu_last_filter_ms(self._h, ctypes.byref(ms)))
        return float(ms.value)
