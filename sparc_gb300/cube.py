"""Cube files of grid densities, the bridge that lets a density from this library (a learned
initial density, or a converged one) enter an unmodified SPARC run through its
INPUT_DENS_FILE / READ_INIT_DENS input keywords.

The layout is the one SPARC writes and reads (printDens_cube, src/printing.c:138;
readDens_cube and read_vec_cube, src/readfiles.c:1250, :1423): a title line; a
"Cell length: Lx Ly Lz, boundary condition: P P P." line; the atom count and the origin; one
line per direction with the point count and the step vector; one line per atom (atomic
number, valence charge, position in Bohr); then the values with x outermost and z innermost,
six per line, the grid index being i + j*Nx + k*Nx*Ny as everywhere in the library. SPARC
checks that N times the step vector matches the cell within 1e-4 Bohr and that the point
counts match its grid.
"""
import time

import numpy as np


def write_cube(path, rho, N, L, atoms=(), title="Electron density"):
    """Write rho (Nx*Ny*Nz, index i + j*Nx + k*Nx*Ny) of an orthogonal periodic cell with
    lengths L on the N grid; atoms: iterable of (Z, valence, (x, y, z))."""
    Nx, Ny, Nz = (int(n) for n in N)
    rho = np.asarray(rho, dtype=np.float64).reshape(Nz, Ny, Nx)
    atoms = list(atoms)
    h = [float(L[d]) / int(N[d]) for d in range(3)]
    with open(path, "w") as f:
        f.write(f"{title} in Cube format (written {time.strftime('%a %b %d %H:%M:%S %Y')})\n")
        f.write(f"Cell length: {L[0]:.6f} {L[1]:.6f} {L[2]:.6f}, boundary condition: P P P.\n")
        f.write(f"{len(atoms):5d} {0.0:11.6f}  {0.0:11.6f}  {0.0:11.6f}\n")
        f.write(f"{Nx:5d} {h[0]:11.6f}  {0.0:11.6f}  {0.0:11.6f}\n")
        f.write(f"{Ny:5d} {0.0:11.6f}  {h[1]:11.6f}  {0.0:11.6f}\n")
        f.write(f"{Nz:5d} {0.0:11.6f}  {0.0:11.6f}  {h[2]:11.6f}\n")
        for Z, zion, pos in atoms:
            f.write(f"{int(Z):5d} {float(zion):11.6f} {pos[0]:11.6f}  {pos[1]:11.6f}  "
                    f"{pos[2]:11.6f}\n")
        # x outermost, z innermost; rows of Nz values broken every six
        block = rho.transpose(2, 1, 0).reshape(Nx * Ny, Nz)
        for row in block:
            for k0 in range(0, Nz, 6):
                f.write("".join(f"  {v:.10E}" for v in row[k0:k0 + 6]))
                f.write("\n")


def read_cube(path):
    """Read a cube file: returns (rho (Nd, index i + j*Nx + k*Nx*Ny), N, step vectors (3, 3),
    atoms [(Z, valence, (x, y, z))])."""
    with open(path) as f:
        lines = f.read().split("\n")
    head = lines[2].split()
    n_atom = int(head[0])
    N, steps = [], []
    for d in range(3):
        p = lines[3 + d].split()
        N.append(int(p[0]))
        steps.append([float(v) for v in p[1:4]])
    atoms = []
    for a in range(n_atom):
        p = lines[6 + a].split()
        atoms.append((int(p[0]), float(p[1]), tuple(float(v) for v in p[2:5])))
    vals = np.array(" ".join(lines[6 + n_atom:]).split(), dtype=np.float64)
    Nx, Ny, Nz = N
    if vals.size != Nx * Ny * Nz:
        raise ValueError(f"{path}: {vals.size} values for a {Nx}x{Ny}x{Nz} grid")
    rho = vals.reshape(Nx, Ny, Nz).transpose(2, 1, 0).reshape(-1)
    return rho, tuple(N), np.array(steps), atoms
