"""The library's psp8 reader and set-up defaults against the reference (CPU only).

The reference's parsed tables (PSD_OBJ after read_pseudopotential_PSP, src/readfiles.c:1957)
are stored in tests/golden/<system>_setup.npz; tests/golden/psp_<El>.npz are the library
reader's output for the same files. Both must agree exactly.
"""
import os

import numpy as np
import pytest

from oracle.refpath import psps_dir
from sparc_gb300.psp8 import Psp8Error, load_tables, read_psp8
from sparc_gb300.setup import grid_from_mesh, ion_coordinates
from sparc_gb300.synthetic import fd_d2_coeffs

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REF_PSPS = psps_dir()
FIELDS = ("RadialGrid", "UdV", "rVloc", "rhoIsoAtom", "rho_c_table", "Gamma", "rc", "ppl")
CASES = [("Si2_small", "Si"), ("Si8_c1", "Si"), ("Al4_small", "Al")]


def ref_tables(system):
    d = np.load(os.path.join(GOLDEN, f"{system}_setup.npz"))
    return {k[3:]: d[k] for k in d.files if k.startswith("t0_")}, d


@pytest.mark.parametrize("system,el", CASES)
def test_reader_tables_equal_reference(system, el):
    ref, _ = ref_tables(system)
    mine = load_tables(os.path.join(GOLDEN, f"psp_{el}.npz"))
    for k in FIELDS:
        np.testing.assert_array_equal(np.asarray(mine[k]).reshape(-1),
                                      np.asarray(ref[k]).reshape(-1), err_msg=k)
    for k in ("size", "lmax", "lloc", "Znucl", "is_r_uniform"):
        assert int(mine[k]) == int(ref[k]), k
    assert mine["Vloc_0"] == float(ref["Vloc_0"])
    assert mine["fchrg"] == float(ref["fchrg"])


@pytest.mark.skipif(not os.path.isdir(REF_PSPS), reason="reference pseudopotentials absent")
@pytest.mark.parametrize("el,fn", [("Si", "14_Si_4_1.9_1.9_pbe_n_v1.0.psp8"),
                                   ("Al", "13_Al_3_1.9_1.9_pbe_n_v1.0.psp8")])
def test_reader_on_psp8_file(el, fn):
    mine = read_psp8(os.path.join(REF_PSPS, fn), el)
    stored = load_tables(os.path.join(GOLDEN, f"psp_{el}.npz"))
    for k in FIELDS:
        np.testing.assert_array_equal(np.asarray(mine[k]), np.asarray(stored[k]), err_msg=k)


def test_reader_rejects_wrong_element(tmp_path):
    if not os.path.isdir(REF_PSPS):
        pytest.skip("reference pseudopotentials absent")
    with pytest.raises(Psp8Error):
        read_psp8(os.path.join(REF_PSPS, "14_Si_4_1.9_1.9_pbe_n_v1.0.psp8"), "Al")


def test_reader_rejects_truncated_file(tmp_path):
    p = tmp_path / "bad.psp8"
    p.write_text("Si  test\n 14.0 4.0 0\n 8 11 2 4 600 0\n")
    with pytest.raises(Psp8Error):
        read_psp8(str(p))


@pytest.mark.parametrize("system,el", CASES)
def test_grid_and_fd_weights_equal_reference(system, el):
    _, d = ref_tables(system)
    L = d["L"]
    mesh = {"Si2_small": 0.5, "Si8_c1": 0.4, "Al4_small": 0.5}[system]
    assert grid_from_mesh(L, mesh) == (int(d["Nx"]), int(d["Ny"]), int(d["Nz"]))
    h = L / np.array([int(d["Nx"]), int(d["Ny"]), int(d["Nz"])])
    np.testing.assert_allclose(h, d["h"], rtol=0, atol=1e-15)
    for c, hh in zip(("cx", "cy", "cz"), h):
        np.testing.assert_allclose(fd_d2_coeffs(6, hh), d[c], rtol=1e-14, atol=0)


@pytest.mark.parametrize("system", ["Si2_small", "Si8_c1", "Al4_small"])
def test_ion_coordinates_match_reference_read(system):
    import sys
    sys.path.insert(0, GOLDEN)
    import systems
    _, d = ref_tables(system)
    sysd = getattr(systems, system.lower())()
    pos = ion_coordinates(sysd["species"][0][1], sysd["L"])
    np.testing.assert_array_equal(pos, d["atom_pos"])
