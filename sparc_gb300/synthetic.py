"""Seeded synthetic inputs for the stencil / Chebyshev-filter microbenchmark and the tests.

The microbenchmark workload: a periodic orthogonal grid (96^3 at h = 0.35 Bohr), FD order 12,
random orbital blocks i.i.d. U[-1, 1], a local potential made of 64 seeded Gaussians
(amplitude -2 Ha, width 1.5 Bohr), and a nonlocal part of 64 atoms with 9 projectors each
(l = 0, 1, 2, one radial function per l) on 6 Bohr spheres, built as seeded radial values
times real spherical harmonics, with seeded Kleinman-Bylander energies Gamma_l.

The nonlocal set is returned in the library's flattened layout (include/sparc_gpu.h,
sgpu_set_nonlocal): one image per atom whose sphere is wrapped periodically into the cell.
"""
import math

import numpy as np


def fd_d2_coeffs(FDn, h):
    """Central second-derivative weights of half-order FDn divided by h^2, following the
    reference's FDweights_D2 (src/initialization.c:2112-2121, fract at src/tools.c:725)."""
    def fract(n, k):
        return math.prod(range(n - k + 1, n + 1)) / math.prod(range(n + 1, n + k + 1))
    w = np.zeros(FDn + 1)
    for p in range(1, FDn + 1):
        w[0] -= 2.0 / (p * p)
        w[p] = 2.0 * (-1.0) ** (p + 1) * fract(FDn, p) / (p * p)
    return w / (h * h)


def _grid_coords(N, h):
    return (np.arange(N, dtype=np.float64)) * h


def gaussian_potential(rng, N, h, ncenters=64, amp=-2.0, width=1.5):
    """Sum of periodic Gaussians on an N^3 grid of spacing h (x fastest)."""
    Nx, Ny, Nz = N
    L = np.array([Nx * h, Ny * h, Nz * h])
    centers = rng.uniform(0.0, 1.0, size=(ncenters, 3)) * L
    x, y, z = _grid_coords(Nx, h), _grid_coords(Ny, h), _grid_coords(Nz, h)
    v = np.zeros((Nz, Ny, Nx))
    for c in centers:
        dx = np.abs(x - c[0]); dx = np.minimum(dx, L[0] - dx)
        dy = np.abs(y - c[1]); dy = np.minimum(dy, L[1] - dy)
        dz = np.abs(z - c[2]); dz = np.minimum(dz, L[2] - dz)
        gx = np.exp(-dx ** 2 / (2 * width ** 2))
        gy = np.exp(-dy ** 2 / (2 * width ** 2))
        gz = np.exp(-dz ** 2 / (2 * width ** 2))
        v += amp * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
    return v.reshape(-1)


def real_ylm(l, dx, dy, dz, r):
    """Real spherical harmonics for l <= 3, in the order m = -l..l (unit-normalised): 2l+1
    functions."""
    rs = np.where(r > 1e-12, r, 1.0)
    X, Y, Z = dx / rs, dy / rs, dz / rs
    if l == 0:
        return [np.full_like(r, 0.5 / math.sqrt(math.pi))]
    if l == 1:
        c = math.sqrt(3.0 / (4.0 * math.pi))
        return [c * Y, c * Z, c * X]
    if l == 2:
        c1 = 0.5 * math.sqrt(15.0 / math.pi)
        c2 = 0.25 * math.sqrt(5.0 / math.pi)
        c3 = 0.25 * math.sqrt(15.0 / math.pi)
        return [c1 * X * Y, c1 * Y * Z, c2 * (3 * Z * Z - 1), c1 * X * Z, c3 * (X * X - Y * Y)]
    if l == 3:
        a = 0.25 * math.sqrt(35.0 / (2.0 * math.pi))
        b = 0.5 * math.sqrt(105.0 / math.pi)
        c = 0.25 * math.sqrt(21.0 / (2.0 * math.pi))
        d = 0.25 * math.sqrt(7.0 / math.pi)
        e = 0.25 * math.sqrt(105.0 / math.pi)
        return [a * (3 * X * X - Y * Y) * Y, b * X * Y * Z, c * Y * (5 * Z * Z - 1),
                d * Z * (5 * Z * Z - 3), c * X * (5 * Z * Z - 1), e * (X * X - Y * Y) * Z,
                a * (X * X - 3 * Y * Y) * X]
    raise ValueError("real_ylm: l <= 3 only")


def synthetic_nonlocal(rng, N, h, natom=64, rc=6.0, lmax=2):
    """64 atoms x (1+3+5) projectors on rc-spheres, flattened for sgpu_set_nonlocal."""
    Nx, Ny, Nz = N
    L = np.array([Nx * h, Ny * h, Nz * h])
    pos = rng.uniform(0.0, 1.0, size=(natom, 3)) * L
    nr = int(math.ceil(rc / h))
    off = np.arange(-nr, nr + 1)
    OZ, OY, OX = np.meshgrid(off, off, off, indexing="ij")
    OX, OY, OZ = OX.reshape(-1), OY.reshape(-1), OZ.reshape(-1)
    nproj = sum(2 * l + 1 for l in range(lmax + 1))
    gam_l = rng.uniform(-2.0, 4.0, size=lmax + 1)
    gamma = np.concatenate([[gam_l[l]] * (2 * l + 1) for l in range(lmax + 1)])
    img_ndc, grid_pos, chi = [], [], []
    for a in range(natom):
        ci = np.floor(pos[a] / h).astype(int)
        gi, gj, gk = ci[0] + OX, ci[1] + OY, ci[2] + OZ
        dx, dy, dz = gi * h - pos[a, 0], gj * h - pos[a, 1], gk * h - pos[a, 2]
        r = np.sqrt(dx * dx + dy * dy + dz * dz)
        m = r <= rc
        dx, dy, dz, r = dx[m], dy[m], dz[m], r[m]
        gi, gj, gk = gi[m] % Nx, gj[m] % Ny, gk[m] % Nz
        p = gi + gj * Nx + gk * Nx * Ny
        order = np.argsort(p, kind="stable")
        p, dx, dy, dz, r = p[order], dx[order], dy[order], dz[order], r[order]
        cols = []
        for l in range(lmax + 1):
            # seeded smooth radial function vanishing at rc
            c = rng.uniform(0.5, 1.5, size=3)
            u = (c[0] + c[1] * (r / rc) + c[2] * (r / rc) ** 2) * np.cos(0.5 * math.pi * r / rc) ** 2
            u *= (r / rc) ** l
            for y in real_ylm(l, dx, dy, dz, r):
                cols.append(u * y)
        img_ndc.append(len(p))
        grid_pos.append(p.astype(np.int32))
        chi.append(np.stack(cols, axis=1).T.reshape(-1))  # column-major ndc x nproj
    return dict(
        ip_displ=(np.arange(natom + 1) * nproj).astype(np.int32),
        gamma=np.tile(gamma, natom),
        img_atom=np.arange(natom, dtype=np.int32),
        img_ndc=np.array(img_ndc, dtype=np.int32),
        grid_pos=np.concatenate(grid_pos),
        chi=np.concatenate(chi),
    )


def microbench_workload(N=(96, 96, 96), h=0.35, ncol=512, natom=64, rc=6.0, seed=2026,
                        with_vectors=True):
    """The stencil/filter microbenchmark inputs (see module docstring)."""
    rng = np.random.default_rng(seed)
    c = fd_d2_coeffs(6, h)
    grid = dict(Nx=N[0], Ny=N[1], Nz=N[2], FDn=6, cx=c, cy=c.copy(), cz=c.copy(), dV=h ** 3)
    veff = gaussian_potential(rng, N, h)
    nl = synthetic_nonlocal(rng, N, h, natom=natom, rc=rc) if natom > 0 else None
    X = rng.uniform(-1.0, 1.0, size=(ncol, N[0] * N[1] * N[2])) if with_vectors else None
    return dict(grid=grid, veff=veff, nl=nl, X=X, m=20, a=0.5, b=50.0, a0=-1.0)


def filter_bytes(Nd, ncol, m, elem_bytes):
    """Algorithmic HBM bytes of one degree-m filter over an Nd x ncol block: the first step
    reads X and writes Y, each later degree reads Y and X and writes the new iterate."""
    return Nd * ncol * elem_bytes * (3 * m - 1)
