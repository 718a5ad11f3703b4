"""Pin the oracle against the live reference program on fresh seeded inputs.

Runs only where the reference was compiled into oracle/_ref (the build container); the
committed fixtures cover the same ground elsewhere."""
import multiprocessing as mp
import os

import numpy as np
import pytest

from oracle.refpath import psps_dir

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libsparc_ref.so")
PSPS = psps_dir()

pytestmark = pytest.mark.skipif(not (os.path.exists(REF_LIB) and os.path.isdir(PSPS)),
                                reason="reference build not present")


def _worker(q, seed):
    import sys
    import tempfile
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    sys.path.insert(0, ROOT)
    import systems
    from make_golden import flatten_nonlocal
    from ref_capture import RefSystem
    from oracle.oracle import Oracle
    tmp = tempfile.mkdtemp()
    base = systems.write_system(systems.si2_small(seed=seed), tmp, PSPS)
    r = RefSystem(base)
    types, images = r.nonlocal_data()
    nl = flatten_nonlocal(types, images, r.n_atom)
    grid = dict(Nx=r.Nx, Ny=r.Ny, Nz=r.Nz, FDn=r.order // 2, cx=r.cx, cy=r.cy, cz=r.cz, dV=r.dV)
    o = Oracle(grid, nl)
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((2, r.Nd))
    v = rng.standard_normal(r.Nd)
    errs = {}
    errs["lpd"] = np.abs(o.lap_plus_diag(-0.5, 1.0, -0.7, v, x) - r.lap_plus_diag(-0.5, 1.0, -0.7, v, x)).max()
    hr = r.hamiltonian(v, 0.25, x)
    errs["ham"] = np.abs(o.hamiltonian(v, 0.25, x) - hr).max() / np.abs(hr).max()
    Xr, Yr = r.chebyshev(v, 9, 0.1, 30.0, -2.0, x)
    Xo, Yo = o.chebyshev(v, 9, 0.1, 30.0, -2.0, x)
    errs["cheb"] = np.abs(Yo - Yr).max() / np.abs(Yr).max()
    q.put(errs)


@pytest.mark.parametrize("seed", [3, 19])
def test_oracle_matches_live_reference(seed):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=_worker, args=(q, seed))
    p.start()
    errs = q.get(timeout=120)
    p.join()
    assert errs["lpd"] == 0.0
    assert errs["ham"] < 1e-13
    assert errs["cheb"] < 1e-12
