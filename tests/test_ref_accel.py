"""The drop-in boundary, end to end: the unmodified reference program compiled with its own
accelerator hooks on (-DSPARCX_ACCEL -DACCEL, src/eigenSolver.c:314-321, :953-958, :1267-1300,
src/forces.c:726-729) and linked through sparc_gb300/shim against libsparc_gpu.so
(oracle/ref/Makefile, target accel).

CPU: the accelerated program compiles and links against the library (where the reference
sources, or their staged copy, are present). GPU: the linked program runs the Si8 system
(C1: 26^3 grid, 32 states, LDA, TOL_SCF 1e-6) with its CheFSI filter, H Y, subspace
eigensolver and nonlocal forces on the GPU, and its own output must match the reference
program's CPU run (tests/golden/Si8_c1_scf_ref.json): free energy within 1e-5 Ha/atom, forces
within 1e-4 Ha/Bohr, occupied eigenvalues within 1e-5 Ha, SCF iteration count within 2.
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

from oracle.refpath import psps_dir, reference_present, reference_root

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
ACCEL = os.path.join(ROOT, "oracle", "_ref", "sparc_accel")
LIB = os.path.join(ROOT, "sparc_gb300", "libsparc_gpu.so")

needs_ref = pytest.mark.skipif(not reference_present(), reason="reference sources not present")


def _make_accel():
    if not os.path.exists(LIB):
        from sparc_gb300 import build
        build.build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"),
                    f"REF={reference_root()}", f"-j{os.cpu_count() or 4}", "accel"],
                   check=True)


@needs_ref
def test_accelerated_reference_compiles_and_links():
    _make_accel()
    assert os.path.exists(ACCEL)
    out = subprocess.run(["ldd", ACCEL], capture_output=True, text=True).stdout
    assert "libsparc_gpu.so" in out, out
    # the hooks resolve to the shim, the shim to the library
    syms = subprocess.run(["nm", ACCEL], capture_output=True, text=True).stdout
    for name in ("gb300_ChebyshevFiltering", "gb300_dsygv", "gb300_nonlocal_forces_linear"):
        assert f" T {name}" in syms, name
    assert "U sgpu_ChebyshevFiltering_y" in syms


@needs_ref
@pytest.mark.gpu
def test_accelerated_reference_runs_si8_on_the_gpu(gpu_available):
    _make_accel()
    sys.path.insert(0, GOLDEN)
    import systems
    from ref_capture import parse_reference_outputs
    with open(os.path.join(GOLDEN, "Si8_c1_scf_ref.json")) as fh:
        ref = json.load(fh)
    tmp = tempfile.mkdtemp(prefix="sparc_accel_")
    base = systems.write_system(systems.si8_c1(), tmp, psps_dir())
    env = dict(os.environ, OMP_NUM_THREADS="4")
    run = subprocess.run([ACCEL, "-name", os.path.basename(base)], cwd=tmp, env=env,
                         capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, run.stdout[-3000:] + run.stderr[-2000:]
    assert "Hardware acceleration is ENABLED" in run.stdout
    assert "libsparc_gpu: CheFSI filter" in run.stdout
    got = parse_reference_outputs(base)
    assert abs(got["Etot_per_atom"] - ref["Etot_per_atom"]) < 1e-5
    assert abs(got["scf_iters"] - ref["scf_iters"]) <= 2
    occ = np.array(ref["occ"]) > 1e-3
    lam = np.array(got["lambda"])
    assert np.abs(lam[occ] - np.array(ref["lambda"])[occ]).max() < 1e-5
    F = np.array(got["forces"])
    assert F.shape == (8, 3)
    assert np.abs(F - np.array(ref["forces"])).max() < 1e-4
