"""Cube-file bridge (sparc_gb300/cube.py): round trip, and the files this library writes parsed
by the reference program's own reader (readDens_cube, src/readfiles.c:1250) where the reference
was compiled into oracle/_ref (the build container; skipped elsewhere). CPU only."""
import ctypes
import os

import numpy as np
import pytest

from sparc_gb300.cube import read_cube, write_cube

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libsparc_ref.so")

CELLS = [((26, 26, 26), (10.26, 10.26, 10.26)), ((13, 17, 11), (5.2, 7.1, 4.4)),
         ((52, 52, 52), (20.52, 19.9, 21.1))]


def _density(N, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(0.0, 0.2, int(np.prod(N)))


@pytest.mark.parametrize("N,L", CELLS)
def test_round_trip(tmp_path, N, L):
    rho = _density(N, sum(N))
    atoms = [(14, 4.0, (0.1, 0.2, 0.3)), (14, 4.0, (2.6, 2.5, 2.7))]
    path = str(tmp_path / "rho.cube")
    write_cube(path, rho, N, L, atoms, title="Learned initial density")
    r2, N2, steps, atoms2 = read_cube(path)
    assert N2 == tuple(N)
    np.testing.assert_allclose(np.diag(steps) * np.array(N), L, atol=1e-4)
    assert [a[0] for a in atoms2] == [14, 14]
    np.testing.assert_allclose([a[2] for a in atoms2], [a[2] for a in atoms], atol=1e-6)
    np.testing.assert_allclose(r2, rho, rtol=1e-10, atol=0)


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference not compiled here")
@pytest.mark.parametrize("N,L", CELLS)
def test_reference_reader_parses_our_files(tmp_path, N, L):
    lib = ctypes.CDLL(REF_LIB)
    lib.readDens_cube.restype = ctypes.POINTER(ctypes.c_double)
    rho = _density(N, 7 + sum(N))
    path = str(tmp_path / "rho.cube")
    write_cube(path, rho, N, L, [(14, 4.0, (1.0, 2.0, 3.0))])
    gs = (ctypes.c_int * 3)()
    lv = (ctypes.c_double * 9)()
    p = lib.readDens_cube(path.encode(), gs, lv)
    assert tuple(gs) == tuple(N)
    # the reference compares N x step with its lattice within 1e-4 (check_lattice_cell)
    np.testing.assert_allclose(np.array(lv).reshape(3, 3), np.diag(L), atol=1e-4)
    got = np.ctypeslib.as_array(p, shape=(int(np.prod(N)),)).copy()
    np.testing.assert_allclose(got, rho, rtol=1e-10, atol=0)
