"""Load the committed golden fixtures (produced by tests/golden/make_golden.py from the
reference program) into the dictionaries the oracle and the GPU library take."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["si2_small", "si8"]


def load(name):
    f = np.load(os.path.join(GOLDEN, f"{name}_kernels.npz"))
    d = {k: f[k] for k in f.files}
    grid = dict(Nx=int(d["Nx"]), Ny=int(d["Ny"]), Nz=int(d["Nz"]), FDn=int(d["FDn"]),
                cx=d["cx"], cy=d["cy"], cz=d["cz"], dV=float(d["dV"]))
    nl = {k[3:]: v for k, v in d.items() if k.startswith("nl_")}
    return d, grid, nl


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
