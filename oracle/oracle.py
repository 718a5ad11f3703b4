"""ctypes binding of the CPU oracle (oracle/sparc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg as the checker. The GPU library never imports or calls this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "sparc_oracle.c")
LIB = os.path.join(HERE, "liboracle.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_long)


def build():
    """Compile liboracle.so with gcc (OpenMP over columns)."""
    deps = [SRC, os.path.join(HERE, "sparc_oracle.h")]
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    tmp = LIB + ".tmp"
    subprocess.run(["gcc", "-O2", "-fopenmp", "-shared", "-fPIC", "-std=gnu99", SRC, "-o", tmp,
                    "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


class _Grid(ctypes.Structure):
    _fields_ = [("Nx", ctypes.c_int), ("Ny", ctypes.c_int), ("Nz", ctypes.c_int),
                ("FDn", ctypes.c_int), ("cx", _dp), ("cy", _dp), ("cz", _dp),
                ("dV", ctypes.c_double)]


class _Nonlocal(ctypes.Structure):
    _fields_ = [("natom", ctypes.c_int), ("ip_displ", _ip), ("gamma", _dp),
                ("nimg", ctypes.c_int), ("img_atom", _ip), ("img_ndc", _ip),
                ("img_off", _lp), ("img_chi_off", _lp), ("grid_pos", _ip), ("chi", _dp)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


class Oracle:
    """CPU restatement of the reference kernels for one grid and nonlocal set.

    grid: dict with Nx, Ny, Nz, FDn, cx, cy, cz, dV. nloc: dict with the flattened
    projector arrays (ip_displ, gamma, img_atom, img_ndc, grid_pos, chi) or None.
    """

    def __init__(self, grid, nloc=None):
        self.lib = lib()
        self.Nx, self.Ny, self.Nz = int(grid["Nx"]), int(grid["Ny"]), int(grid["Nz"])
        self.Nd = self.Nx * self.Ny * self.Nz
        self.FDn = int(grid["FDn"])
        self._keep = []
        cx, cy, cz = (np.ascontiguousarray(grid[k], dtype=np.float64) for k in ("cx", "cy", "cz"))
        self._keep += [cx, cy, cz]
        self.g = _Grid(self.Nx, self.Ny, self.Nz, self.FDn, _d(cx), _d(cy), _d(cz),
                       float(grid["dV"]))
        self.nl = None
        if nloc is not None and len(nloc["img_atom"]) > 0:
            ip = np.ascontiguousarray(nloc["ip_displ"], dtype=np.int32)
            gam = np.ascontiguousarray(nloc["gamma"], dtype=np.float64)
            ia = np.ascontiguousarray(nloc["img_atom"], dtype=np.int32)
            nd = np.ascontiguousarray(nloc["img_ndc"], dtype=np.int32)
            gp = np.ascontiguousarray(nloc["grid_pos"], dtype=np.int32)
            chi = np.ascontiguousarray(nloc["chi"], dtype=np.float64)
            npa = ip[1:] - ip[:-1]
            off = np.concatenate([[0], np.cumsum(nd)[:-1]]).astype(np.int64)
            choff = np.concatenate([[0], np.cumsum(nd.astype(np.int64) * npa[ia])[:-1]]).astype(np.int64)
            self._keep += [ip, gam, ia, nd, gp, chi, off, choff]
            self.nl = _Nonlocal(len(ip) - 1, ip.ctypes.data_as(_ip), _d(gam), len(ia),
                                ia.ctypes.data_as(_ip), nd.ctypes.data_as(_ip),
                                off.ctypes.data_as(_lp), choff.ctypes.data_as(_lp),
                                gp.ctypes.data_as(_ip), _d(chi))

    def _nlp(self):
        return ctypes.byref(self.nl) if self.nl is not None else None

    @staticmethod
    def _blk(x):
        x = np.array(x, dtype=np.float64, order="C", copy=True)
        return x.reshape(1, -1) if x.ndim == 1 else x

    def lap_plus_diag(self, a, b, c, v, x):
        x = self._blk(x)
        y = np.zeros_like(x)
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        self.lib.orc_lap_plus_diag_orth(
            self.Nx, self.Ny, self.Nz, self.FDn, self.g.cx, self.g.cy, self.g.cz,
            ctypes.c_int(x.shape[0]), ctypes.c_double(a), ctypes.c_double(b), ctypes.c_double(c),
            _d(vv) if vv is not None else None, _d(x), ctypes.c_long(self.Nd), _d(y),
            ctypes.c_long(self.Nd))
        return y

    def vnl(self, x, hx=None):
        x = self._blk(x)
        out = np.zeros_like(x) if hx is None else self._blk(hx)
        if self.nl is not None:
            self.lib.orc_vnl_vec_mult(self._nlp(), ctypes.c_double(self.g.dV),
                                      ctypes.c_int(x.shape[0]), _d(x), ctypes.c_long(self.Nd),
                                      _d(out), ctypes.c_long(self.Nd))
        return out

    def hamiltonian(self, veff, c, x):
        x = self._blk(x)
        hx = np.zeros_like(x)
        veff = np.ascontiguousarray(veff, dtype=np.float64)
        self.lib.orc_hamiltonian(ctypes.byref(self.g), self._nlp(), _d(veff),
                                 ctypes.c_int(x.shape[0]), ctypes.c_double(c), _d(x),
                                 ctypes.c_long(self.Nd), _d(hx), ctypes.c_long(self.Nd))
        return hx

    def chebyshev(self, veff, m, a, b, a0, X):
        X = self._blk(X)
        Y = np.zeros_like(X)
        veff = np.ascontiguousarray(veff, dtype=np.float64)
        self.lib.orc_chebyshev_filter(ctypes.byref(self.g), self._nlp(), _d(veff), _d(X),
                                      ctypes.c_long(self.Nd), _d(Y), ctypes.c_long(self.Nd),
                                      ctypes.c_int(X.shape[0]), ctypes.c_int(m),
                                      ctypes.c_double(a), ctypes.c_double(b), ctypes.c_double(a0))
        return X, Y

    def poisson_residual(self, c, x, b):
        x = np.ascontiguousarray(x, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        r = np.zeros_like(x)
        self.lib.orc_poisson_residual(ctypes.byref(self.g), ctypes.c_double(c), _d(x), _d(b), _d(r))
        return r

    # ---- k-point twins: complex blocks (ncol, Nd) complex128; k (3,), L (3,) in Bohr units;
    # img_coords (nimg, 3) image coordinates of the nonlocal set
    @staticmethod
    def _cblk(x):
        x = np.array(x, dtype=np.complex128, order="C", copy=True)
        return x.reshape(1, -1) if x.ndim == 1 else x

    def lap_plus_diag_kpt(self, k, L, a, b, c, v, x):
        x = self._cblk(x)
        y = np.zeros_like(x)
        k = np.ascontiguousarray(k, dtype=np.float64)
        L = np.ascontiguousarray(L, dtype=np.float64)
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        self.lib.orc_lap_plus_diag_orth_kpt(
            self.Nx, self.Ny, self.Nz, self.FDn, self.g.cx, self.g.cy, self.g.cz, _d(k), _d(L),
            ctypes.c_int(x.shape[0]), ctypes.c_double(a), ctypes.c_double(b), ctypes.c_double(c),
            _d(vv) if vv is not None else None, _d(x.view(np.float64)), ctypes.c_long(self.Nd),
            _d(y.view(np.float64)), ctypes.c_long(self.Nd))
        return y

    def _kargs(self, k, L, img_coords):
        k = np.ascontiguousarray(k, dtype=np.float64)
        L = np.ascontiguousarray(L, dtype=np.float64)
        ic = np.ascontiguousarray(img_coords, dtype=np.float64).reshape(-1)
        self._keep += [k, L, ic]
        return k, L, ic

    def vnl_kpt(self, k, L, img_coords, x):
        x = self._cblk(x)
        out = np.zeros_like(x)
        k, L, ic = self._kargs(k, L, img_coords)
        if self.nl is not None:
            self.lib.orc_vnl_vec_mult_kpt(self._nlp(), _d(ic), _d(k), _d(L),
                                          ctypes.c_double(self.g.dV), ctypes.c_int(x.shape[0]),
                                          _d(x.view(np.float64)), ctypes.c_long(self.Nd),
                                          _d(out.view(np.float64)), ctypes.c_long(self.Nd))
        return out

    def hamiltonian_kpt(self, k, L, img_coords, veff, c, x):
        x = self._cblk(x)
        hx = np.zeros_like(x)
        k, L, ic = self._kargs(k, L, img_coords)
        veff = np.ascontiguousarray(veff, dtype=np.float64)
        self.lib.orc_hamiltonian_kpt(ctypes.byref(self.g), self._nlp(), _d(ic), _d(k), _d(L),
                                     _d(veff), ctypes.c_int(x.shape[0]), ctypes.c_double(c),
                                     _d(x.view(np.float64)), ctypes.c_long(self.Nd),
                                     _d(hx.view(np.float64)), ctypes.c_long(self.Nd))
        return hx

    def chebyshev_kpt(self, k, L, img_coords, veff, m, a, b, a0, X):
        X = self._cblk(X)
        Y = np.zeros_like(X)
        k, L, ic = self._kargs(k, L, img_coords)
        veff = np.ascontiguousarray(veff, dtype=np.float64)
        self.lib.orc_chebyshev_filter_kpt(ctypes.byref(self.g), self._nlp(), _d(ic), _d(k),
                                          _d(L), _d(veff), _d(X.view(np.float64)),
                                          ctypes.c_long(self.Nd), _d(Y.view(np.float64)),
                                          ctypes.c_long(self.Nd), ctypes.c_int(X.shape[0]),
                                          ctypes.c_int(m), ctypes.c_double(a),
                                          ctypes.c_double(b), ctypes.c_double(a0))
        return X, Y

    def set_threads(self, n):
        self.lib.orc_set_num_threads(ctypes.c_int(n))

    def threads(self):
        return int(self.lib.orc_num_threads())


def fd_d2_weights(FDn, h):
    w = np.zeros(FDn + 1)
    lib().orc_fd_d2_weights(ctypes.c_int(FDn), ctypes.c_double(h), _d(w))
    return w
