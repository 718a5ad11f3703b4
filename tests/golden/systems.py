"""Seeded test systems, written as SPARC input files (.inpt/.ion).

The same generator feeds the reference program (to produce golden outputs) and the GPU path
(through fixtures exported from the reference set-up), so both see identical geometry.

Input keywords follow the reference's .inpt/.ion format (src/readfiles.c:132 read_input,
src/readfiles.c:1462 read_ion).
"""
import os

import numpy as np

DIAMOND_FRAC = np.array([
    [0.00, 0.00, 0.00], [0.00, 0.50, 0.50], [0.50, 0.00, 0.50], [0.50, 0.50, 0.00],
    [0.25, 0.25, 0.25], [0.25, 0.75, 0.75], [0.75, 0.25, 0.75], [0.75, 0.75, 0.25],
])


def diamond_supercell(a, reps):
    """Cartesian positions (Bohr) of a reps^3 supercell of the 8-atom diamond cubic cell."""
    pos = []
    for i in range(reps):
        for j in range(reps):
            for k in range(reps):
                pos.append((DIAMOND_FRAC + np.array([i, j, k])) * a)
    return np.concatenate(pos, axis=0)


def si8_c1(seed=20261203):
    """8-atom diamond-cubic Si, a=10.26 Bohr, displacements N(0, 0.05^2) Bohr per component."""
    a = 10.26
    rng = np.random.default_rng(seed)
    pos = diamond_supercell(a, 1) + rng.normal(0.0, 0.05, size=(8, 3))
    return dict(
        name="Si8_c1", L=(a, a, a), species=[("Si", pos)],
        keys=dict(MESH_SPACING="0.40", FD_ORDER="12", EXCHANGE_CORRELATION="LDA_PW",
                  ELEC_TEMP_TYPE="fermi-dirac", SMEARING="0.001", NSTATES="32",
                  CHEB_DEGREE="20", MIXING_VARIABLE="density", MIXING_HISTORY="7",
                  TOL_SCF="1e-6", PRINT_FORCES="1", PRINT_EIGEN="1"),
    )


def si216_c4(seed=20261204):
    """216-atom diamond Si (3x3x3 cells, a = 30.78 Bohr), displacements N(0, 0.1^2) Bohr,
    h = 0.40 (77^3 grid), LDA_PW, 520 states, Chebyshev degree 24, Gamma point."""
    a = 10.26
    rng = np.random.default_rng(seed)
    pos = diamond_supercell(a, 3) + rng.normal(0.0, 0.1, size=(216, 3))
    L = 3 * a
    return dict(
        name="Si216_c4", L=(L, L, L), species=[("Si", pos)],
        keys=dict(MESH_SPACING="0.40", FD_ORDER="12", EXCHANGE_CORRELATION="LDA_PW",
                  ELEC_TEMP_TYPE="fermi-dirac", SMEARING="0.001", NSTATES="520",
                  CHEB_DEGREE="24", MIXING_VARIABLE="density", MIXING_HISTORY="7",
                  TOL_SCF="1e-6", PRINT_FORCES="1", PRINT_EIGEN="1"),
    )


def si2_small(seed=7):
    """2-atom Si in a 7.0 Bohr cubic box at h=0.5 (14^3 grid): a fast kernel-level case."""
    a = 7.0
    rng = np.random.default_rng(seed)
    pos = np.array([[0.3, 0.2, 0.1], [1.9, 1.7, 1.8]]) + rng.normal(0.0, 0.05, size=(2, 3))
    return dict(
        name="Si2_small", L=(a, a, a), species=[("Si", pos)],
        keys=dict(MESH_SPACING="0.50", FD_ORDER="12", EXCHANGE_CORRELATION="LDA_PW",
                  ELEC_TEMP_TYPE="fermi-dirac", SMEARING="0.001", NSTATES="8",
                  CHEB_DEGREE="16", MIXING_VARIABLE="density", MIXING_HISTORY="7",
                  TOL_SCF="1e-6", PRINT_FORCES="1", PRINT_EIGEN="1"),
    )


def al4_small(seed=9):
    """4-atom FCC Al conventional cell, a = 7.65 Bohr, displacements N(0, 0.05^2) Bohr,
    h = 0.5 (16^3 grid): a second species for the set-up checks (its psp8 carries a model
    core charge and a different projector radius per l)."""
    a = 7.65
    rng = np.random.default_rng(seed)
    fcc = np.array([[0.0, 0.0, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0]])
    pos = fcc * a + rng.normal(0.0, 0.05, size=(4, 3))
    return dict(
        name="Al4_small", L=(a, a, a), species=[("Al", pos)],
        keys=dict(MESH_SPACING="0.50", FD_ORDER="12", EXCHANGE_CORRELATION="LDA_PW",
                  ELEC_TEMP_TYPE="fermi-dirac", SMEARING="0.001", NSTATES="12",
                  CHEB_DEGREE="16", MIXING_VARIABLE="density", MIXING_HISTORY="7",
                  TOL_SCF="1e-6", PRINT_FORCES="1", PRINT_EIGEN="1"),
    )


def si2_kpt(seed=8):
    """The 2-atom Si box with a 3x3x3 k-point grid (complex Bloch orbitals): a fast case for
    the k-point kernels (Bloch phases at the periodic faces and on atom images)."""
    d = si2_small(seed)
    d["name"] = "Si2_kpt"
    d["kpoint_grid"] = (3, 3, 3)
    return d


def al4_spin_kpt(seed=10):
    """The Al4 FCC cell with a 2x2x2 k-point grid, spin-polarised (collinear) from seeded
    initial moments of +-0.2 per atom: a small case of the batched k-point/spin SCF."""
    d = al4_small(seed)
    rng = np.random.default_rng(seed + 1)
    d["name"] = "Al4_spin_kpt"
    d["kpoint_grid"] = (2, 2, 2)
    d["spins"] = {"Al": rng.choice([-0.2, 0.2], size=4) + rng.normal(0.0, 0.02, size=4)}
    d["keys"] = dict(d["keys"], SPIN_TYP="1", NSTATES="16", SMEARING="0.003", MESH_SPACING="0.45")
    return d


def write_system(sysd, outdir, psp_dir):
    """Write <name>.inpt and <name>.ion for the system into outdir."""
    os.makedirs(outdir, exist_ok=True)
    name = sysd["name"]
    L = sysd["L"]
    lines = [f"LATVEC_SCALE: {L[0]:.10f} {L[1]:.10f} {L[2]:.10f}",
             "LATVEC:", "1 0 0", "0 1 0", "0 0 1",
             "BC: P P P", "KPOINT_GRID: %d %d %d" % tuple(sysd.get("kpoint_grid", (1, 1, 1)))]
    for k, v in sysd["keys"].items():
        lines.append(f"{k}: {v}")
    with open(os.path.join(outdir, name + ".inpt"), "w") as f:
        f.write("\n".join(lines) + "\n")
    psp = {"Si": "14_Si_4_1.9_1.9_pbe_n_v1.0.psp8", "Al": "13_Al_3_1.9_1.9_pbe_n_v1.0.psp8"}
    ion = []
    for sym, pos in sysd["species"]:
        ion += [f"ATOM_TYPE: {sym}", f"N_TYPE_ATOM: {len(pos)}",
                f"PSEUDO_POT: {os.path.join(psp_dir, psp[sym])}", "COORD:"]
        ion += [f"  {p[0]:.12f} {p[1]:.12f} {p[2]:.12f}" for p in pos]
        if sym in sysd.get("spins", {}):
            ion += ["SPIN:"] + [f"  {v:.12f}" for v in sysd["spins"][sym]]
        ion.append("")
    with open(os.path.join(outdir, name + ".ion"), "w") as f:
        f.write("\n".join(ion) + "\n")
    return os.path.join(outdir, name)
