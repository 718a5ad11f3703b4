"""C4 at full size: the 216-atom Si cell (3x3x3 diamond cells, a = 30.78 Bohr, 77^3 grid,
520 states, degree 24, LDA, TOL_SCF 1e-6), set up on the device from the Si psp8 tables, in
plain FP64 and in the mixed-precision mode (FP32 filter and FP32-accurate tensor-core
products, then the graded FP64 tail with FP64-accurate tensor-core products), against the
reference program's own run of the same input (tests/golden/Si216_c4_scf_ref.json).

Parity bars (written here as in the configuration): free energy within 1e-5 Ha/atom, occupied
eigenvalues within 1e-5 Ha, forces within 1e-4 Ha/Bohr, SCF convergence. Reference functions:
the SCF of src/electronicGroundState.c:607, forces src/forces.c:49."""
import json
import os
import sys

import numpy as np
import pytest

from sparc_gb300.psp8 import load_tables
from sparc_gb300.setup import CellSystem, grid_from_mesh

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def si216():
    sys.path.insert(0, GOLDEN)
    import systems
    sysd = systems.si216_c4()
    N = grid_from_mesh(sysd["L"], float(sysd["keys"]["MESH_SPACING"]))
    assert tuple(N) == (77, 77, 77)
    cs = CellSystem(sysd["L"], N, sysd["species"],
                    {"Si": load_tables(os.path.join(GOLDEN, "psp_Si.npz"))})
    with open(os.path.join(GOLDEN, "Si216_c4_scf_ref.json")) as fh:
        ref = json.load(fh)
    yield cs, ref
    cs.close()


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_si216_matches_reference_program(gpu_available, si216, mode):
    cs, ref = si216
    kw = dict(precision=64) if mode == "fp64" else dict(
        precision=32, fp64_switch_error=1e-4, graded_tail=1, tail_fp64_degrees=0)
    fields = {}
    res, rho, lam, occ = cs.scf(cs.scf_params(Nstates=520, cheb_degree=24, **kw),
                                fields=fields)
    assert res["converged"] == 1
    assert abs(res["Etot"] / cs.n_atom - ref["Etot_per_atom"]) < 1e-5
    occupied = np.array(ref["occ"]) > 1e-3
    assert np.abs(lam[occupied] - np.array(ref["lambda"])[occupied]).max() < 1e-5
    F = cs.forces(fields, occ)
    Fref = np.array(ref["forces"])
    assert F.shape == Fref.shape == (216, 3)
    assert np.abs(F - Fref).max() < 1e-4, np.abs(F - Fref).max()
