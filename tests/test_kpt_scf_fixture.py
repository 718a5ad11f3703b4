"""The k-point SCF fixture (the reference's Si2 3x3x3 run) is what the GPU test takes it for:
the time-reversal-reduced Monkhorst-Pack points of a 3x3x3 grid with the reference's weights
(the k-point set-up of src/initialization.c), one block of Nstates eigenvalues per point."""
import numpy as np

from scf_io import load_scf


def test_kpt_fixture_is_reduced_3x3x3_grid():
    d, grid, nl, ref = load_scf("Si2_kpt")
    L = d["L"]
    k = d["kpts"]
    w = d["kpt_wts"]
    assert k.shape == (14, 3) and w.shape == (14,)
    assert w.sum() == 27.0
    frac = k * L / (2 * np.pi)                      # in units of the reciprocal vectors
    assert np.allclose(frac * 3, np.round(frac * 3), atol=1e-9)
    assert np.all(np.abs(frac) <= 1 / 3 + 1e-9)
    full = {tuple(np.round(3 * f).astype(int)) for f in frac}
    assert len(full) == 14
    for f in full:
        neg = tuple(-v for v in f)
        assert neg == f or neg not in full          # k and -k are never both kept
    self_conj = [tuple(np.round(3 * f).astype(int)) == (0, 0, 0) for f in frac]
    assert np.all(w[np.array(self_conj)] == 1.0) and np.all(w[~np.array(self_conj)] == 2.0)
    assert len(ref["lambda"]) == 14 * int(d["Nstates"])
    assert len(d["img_coords"]) == len(nl["img_atom"])
