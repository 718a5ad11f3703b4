"""Load the SCF golden fixture (tests/golden/<system>_scf.npz + _scf_ref.json, produced from
the reference program by tests/golden/make_golden.py) and build the SCF parameters."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_scf(name="Si8_c1"):
    f = np.load(os.path.join(GOLDEN, f"{name}_scf.npz"))
    d = {k: f[k] for k in f.files}
    with open(os.path.join(GOLDEN, f"{name}_scf_ref.json")) as fh:
        ref = json.load(fh)
    grid = dict(Nx=int(d["Nx"]), Ny=int(d["Ny"]), Nz=int(d["Nz"]), FDn=int(d["FDn"]),
                cx=d["cx"], cy=d["cy"], cz=d["cz"], dV=float(d["dV"]))
    nl = {k[3:]: v for k, v in d.items() if k.startswith("nl_")}
    return d, grid, nl, ref


def scf_params(sg, d, ref, precision=64, switch=1e-3, seed=1, verbose=0):
    """sgpu_scf_params filled with the reference's own settings for this system."""
    p = ref["params"]
    prm = sg.ScfParams()
    prm.Nstates = int(d["Nstates"])
    prm.n_atom = int(d["n_atom"])
    prm.Nelectron = float(d["Nelectron"])
    prm.Beta = p["Beta"]
    prm.elec_T_type = int(p["elec_T_type"])
    prm.cheb_degree = int(p["ChebDegree"])
    prm.rho_trigger = int(p["rhoTrigger"])
    prm.nchefsi = int(p["Nchefsi"])
    prm.tol_scf = p["TOL_SCF"]
    prm.tol_poisson = p["TOL_POISSON"]
    prm.tol_precond = p["TOL_PRECOND"]
    prm.tol_lanczos = p["TOL_LANCZOS"]
    prm.maxit_scf = int(p["MAXIT_SCF"])
    prm.minit_scf = int(p["MINIT_SCF"])
    prm.maxit_poisson = int(p["MAXIT_POISSON"])
    prm.mixing_history = int(p["MixingHistory"])
    prm.pulay_freq = int(p["PulayFrequency"])
    prm.pulay_restart = 0
    prm.mixing_param = p["MixingParameter"]
    prm.mixing_param_simple = p["MixingParameterSimple"]
    prm.kerker = 1 if int(p["MixingPrecond"]) == 1 else 0
    prm.kerker_kTF = p["precond_kerker_kTF"]
    prm.kerker_idiemac = p["precond_kerker_thresh"]
    prm.xc_rhotol = p["xc_rhotol"]
    prm.Esc = float(d["Esc"])
    prm.precision = precision
    prm.fp64_switch_error = switch
    prm.seed = seed
    prm.verbose = verbose
    return prm
