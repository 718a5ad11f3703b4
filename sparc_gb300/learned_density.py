"""Learned initial density for the CheFSI SCF.

A small network, trained on converged SCF densities that this library computes for seeded
perturbed snapshots, predicts the correction rho_SCF - rho_at to the superposition of atomic
densities at every grid point from rotation-invariant descriptors of the surrounding atoms
(sgpu_density_descriptors). The SCF then starts from

    rho_init = max(rho_at + correction, 0), rescaled to the electron count,

instead of rho_at (the reference's start, Init_electronDensity, src/orbitalElecDensInit.c:145).
The superposition start remains the fallback (rho_init is rho_at when no network is given),
and the converged SCF judges the prediction.

Descriptors, the network's forward and backward passes and the Adam step are the library's own
device kernels (sparc_gb300/csrc/mlp.cu); torch only holds device buffers and draws minibatch
indices.

The data set of the benchmark: 64-atom Si (2x2x2 diamond cells, a = 20.52 Bohr), seeded
displacements with sigma drawn from [0.1, 0.4] Bohr and an isotropic strain from [-3%, +3%], a
fixed 52^3 grid (h = L / 52, about 0.40 Bohr), 160 states, LDA.

usage (on a GPU host):
  python -m sparc_gb300.learned_density --snapshots 400 --test 50 --out result.json \
      --save sparc_gb300/data/si64_density_mlp.npz
"""
import argparse
import ctypes
import json
import math
import os
import time

import numpy as np

from . import SGPU_PREC_FP32, SgpuError, _check, _ptr, lib

NIN = 24
TSCALE = 100.0  # targets (e/Bohr^3) are scaled by this before the loss

SI_DIAMOND = np.array([[0.00, 0.00, 0.00], [0.00, 0.50, 0.50], [0.50, 0.00, 0.50],
                       [0.50, 0.50, 0.00], [0.25, 0.25, 0.25], [0.25, 0.75, 0.75],
                       [0.75, 0.25, 0.75], [0.75, 0.75, 0.25]])


def si_snapshot(index, reps=2, base_seed=4242):
    """Snapshot `index` of a Si data set of reps^3 diamond cells (a = 10.26 Bohr): seeded
    displacements with sigma from U[0.1, 0.4] Bohr and isotropic strain from U[-3%, 3%].
    Returns (cell length, positions, sigma, strain)."""
    rng = np.random.default_rng(base_seed + 7919 * index)
    sigma = rng.uniform(0.1, 0.4)
    strain = rng.uniform(-0.03, 0.03)
    a = 10.26 * (1.0 + strain)
    cells = [(SI_DIAMOND + np.array([i, j, k])) * a for i in range(reps) for j in range(reps)
             for k in range(reps)]
    pos = np.concatenate(cells, axis=0)
    pos = pos + rng.normal(0.0, sigma, size=pos.shape)
    return reps * a, pos, sigma, strain


def si64_snapshot(index):
    """Snapshot `index` of the 64-atom Si data set (2x2x2 cells)."""
    return si_snapshot(index, reps=2)


class DensityMLP:
    """The network (sgpu_mlp): 24 descriptors -> 3 x `width` SiLU -> 1, BF16 weights."""

    def __init__(self, width=128, seed=1, device=0):
        self._h = ctypes.c_void_p()
        self.width = width
        _check(lib().sgpu_mlp_create(int(device), NIN, int(width), ctypes.c_ulonglong(seed),
                                     ctypes.byref(self._h)))
        n = ctypes.c_long()
        _check(lib().sgpu_mlp_nparam(self._h, ctypes.byref(n)))
        self.nparam = int(n.value)

    def close(self):
        if self._h:
            lib().sgpu_mlp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get(self, which):
        n = self.nparam if which < 2 else NIN
        out = np.zeros(n, dtype=np.float32)
        _check(lib().sgpu_mlp_get(self._h, int(which), _ptr(out)))
        return out

    def set(self, which, values):
        v = np.ascontiguousarray(values, dtype=np.float32)
        _check(lib().sgpu_mlp_set(self._h, int(which), _ptr(v)))

    params = property(lambda self: self.get(0))
    grads = property(lambda self: self.get(1))

    def set_normalization(self, shift, scale):
        self.set(2, shift)
        self.set(3, scale)

    def forward(self, x, y):
        _check(lib().sgpu_mlp_forward(self._h, _ptr(x), int(x.shape[0]), _ptr(y)))

    def zero_grad(self):
        _check(lib().sgpu_mlp_zero_grad(self._h))

    def loss_grad(self, x, target, tscale=TSCALE):
        loss = ctypes.c_double()
        _check(lib().sgpu_mlp_loss_grad(self._h, _ptr(x), _ptr(target), int(x.shape[0]),
                                        ctypes.c_float(tscale), ctypes.byref(loss)))
        return float(loss.value)

    def adam_step(self, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        _check(lib().sgpu_mlp_adam_step(self._h, ctypes.c_float(lr), ctypes.c_float(beta1),
                                        ctypes.c_float(beta2), ctypes.c_float(eps)))

    def save(self, path, meta=None):
        np.savez_compressed(path, params=self.get(0), shift=self.get(2), scale=self.get(3),
                            width=self.width, meta=json.dumps(meta or {}))

    @classmethod
    def load(cls, path, device=0):
        d = np.load(path)
        net = cls(width=int(d["width"]), device=device)
        net.set(0, d["params"])
        net.set_normalization(d["shift"], d["scale"])
        return net


def descriptors(torch, cs, dev):
    """Descriptors of a CellSystem's current geometry as a device tensor (Nd, 24)."""
    Nd = int(np.prod(cs.N))
    desc = torch.empty((Nd, NIN), dtype=torch.float32, device=dev)
    cs.ctx.density_descriptors(cs.L, cs.atom_pos, desc)
    return desc


def initial_density(torch, cs, net, dev):
    """rho_init of the CellSystem's geometry from the network (rho_at when net is None)."""
    rho_at = cs.fields["rho_at"]
    if net is None:
        return rho_at
    desc = descriptors(torch, cs, dev)
    y = torch.empty(desc.shape[0], dtype=torch.float32, device=dev)
    net.forward(desc, y)
    rho = rho_at + y.double().cpu().numpy() / TSCALE
    np.maximum(rho, 0.0, out=rho)
    rho *= cs.Nelectron / (rho.sum() * cs.dV)
    return rho


def write_density_cube(cs, rho, path, title="Electron density"):
    """Write a density of the CellSystem's current geometry as a cube file that SPARC reads
    with INPUT_DENS_FILE: <path> and READ_INIT_DENS: 1 (sparc_gb300/cube.py)."""
    from .cube import write_cube
    atoms, a = [], 0
    for t, n in zip(cs.tables, cs.nAtomv):
        for _ in range(int(n)):
            atoms.append((int(t["Zatom"]), float(t["Znucl"]), tuple(cs.atom_pos[a])))
            a += 1
    write_cube(path, rho, cs.N, cs.L, atoms, title=title)


def scf_settings(cs, precision, Nstates=160, cheb_degree=20, rho_trigger=4):
    """SCF parameters of the data generation and the evaluation; rho_trigger is the number of
    filter passes of the first SCF iteration (the reference's rhoTrigger, default 4)."""
    kw = dict(Nstates=Nstates, cheb_degree=cheb_degree)
    if precision == 32:
        kw.update(precision=SGPU_PREC_FP32, fp64_switch_error=1e-4, graded_tail=1,
                  tail_fp64_degrees=0)
    p = cs.scf_params(**kw)
    p.rho_trigger = int(rho_trigger)
    return p


def generate(torch, cs, indices, dev, precision=32, log=None, snap=si64_snapshot, scf_kw=None):
    """Converged densities of the given snapshots (their SCF from rho_at), kept on the device
    with their descriptors: returns (desc (n, Nd, 24) float32, target (n, Nd) float32, info)."""
    Nd = int(np.prod(cs.N))
    descs = torch.empty((len(indices), Nd, NIN), dtype=torch.float32, device=dev)
    targs = torch.empty((len(indices), Nd), dtype=torch.float32, device=dev)
    info = []
    for t, idx in enumerate(indices):
        L, pos, sigma, strain = snap(idx)
        cs.set_geometry((L, L, L), [("Si", pos)])
        res, rho, _, _ = cs.scf(scf_settings(cs, precision, **(scf_kw or {})))
        if not res["converged"]:
            raise SgpuError(f"snapshot {idx}: SCF did not converge")
        descs[t] = descriptors(torch, cs, dev)
        targs[t] = torch.from_numpy(rho - cs.fields["rho_at"]).float().to(dev)
        info.append(dict(index=idx, scf_iters=res["scf_iters"], time_s=res["time_s"],
                         sigma=sigma, strain=strain))
        if log:
            log(f"snapshot {idx}: {res['scf_iters']} iterations, {res['time_s']:.2f} s")
    return descs, targs, info


def train(torch, net, descs, targs, dev, epochs=8, batch=65536, lr=2e-3, seed=0, log=None):
    """Adam on random minibatches of grid points drawn from all training snapshots."""
    n = descs.shape[0] * descs.shape[1]
    X = descs.reshape(n, NIN)
    T = targs.reshape(n)
    # input normalisation from the training set
    mu = X.mean(dim=0)
    sd = X.std(dim=0).clamp_min(1e-6)
    net.set_normalization(mu.cpu().numpy(), (1.0 / sd).cpu().numpy())
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    steps = max(1, n // batch)
    hist = []
    for ep in range(epochs):
        lr_ep = lr * 0.5 * (1 + math.cos(math.pi * ep / epochs))
        tot = 0.0
        for s in range(steps):
            idx = torch.randint(0, n, (batch,), generator=gen, device=dev)
            xb = X.index_select(0, idx).contiguous()
            tb = T.index_select(0, idx).contiguous()
            net.zero_grad()
            tot += net.loss_grad(xb, tb)
            net.adam_step(lr_ep)
        hist.append(tot / steps)
        if log:
            log(f"epoch {ep}: loss {hist[-1]:.4e}")
    return hist


def energy_reached(history, e_conv, n_atom, tol=1e-5):
    """(iterations, seconds) until the free energy per atom is within tol of e_conv and stays
    there for the rest of the SCF (None if never)."""
    e = np.asarray(history["Etot"]) / n_atom
    ok = np.abs(e - e_conv) < tol
    for i in range(len(e)):
        if ok[i:].all():
            return i + 1, float(history["time_s"][i])
    return None, None


def evaluate(torch, cs, net, indices, dev, precision=32, log=None, snap=si64_snapshot,
             scf_kw=None, energy_tol=1e-5):
    """Per snapshot and start (rho_at, learned): SCF iterations and time to TOL_SCF, and
    iterations and time until the energy is within energy_tol Ha/atom of the converged one
    (the converged energy of the rho_at start)."""
    out = []
    for idx in indices:
        L, pos, sigma, strain = snap(idx)
        cs.set_geometry((L, L, L), [("Si", pos)])
        rec = dict(index=idx)
        for tag, model in (("rho_at", None), ("learned", net)):
            t0 = time.perf_counter()
            rho0 = initial_density(torch, cs, model, dev)
            t_pred = time.perf_counter() - t0
            res, rho, _, _ = cs.scf(scf_settings(cs, precision, **(scf_kw or {})),
                                    rho_init=rho0)
            rec[tag] = dict(scf_iters=res["scf_iters"], time_s=res["time_s"] + t_pred,
                            converged=bool(res["converged"]),
                            Etot_per_atom=res["Etot"] / cs.n_atom, history=res["history"],
                            predict_s=t_pred,
                            start_error=float(np.linalg.norm(rho0 - rho) / np.linalg.norm(rho)))
        e_conv = rec["rho_at"]["Etot_per_atom"]
        for tag in ("rho_at", "learned"):
            h = rec[tag].pop("history")
            it, ts = energy_reached(h, e_conv, cs.n_atom, energy_tol)
            rec[tag]["iters_to_energy_tol"] = it
            rec[tag]["time_to_energy_tol_s"] = None if ts is None else ts + rec[tag]["predict_s"]
            # per iteration: energy error per atom against e_conv, and the SCF error
            rec[tag]["dE_per_atom"] = [float(f"{e / cs.n_atom - e_conv:.3e}") for e in h["Etot"]]
            rec[tag]["scf_error"] = [float(f"{v:.3e}") for v in h["scf_error"]]
        out.append(rec)
        if log:
            log(f"held-out {idx}: {rec['rho_at']['scf_iters']} -> {rec['learned']['scf_iters']} "
                f"iterations")
    return out


def summarize(ev, mode):
    """Means over the held-out snapshots of one evaluation mode."""
    def col(tag, key):
        return np.array([np.nan if r[tag][key] is None else r[tag][key] for r in ev], dtype=float)
    dE = np.abs(col("rho_at", "Etot_per_atom") - col("learned", "Etot_per_atom"))
    out = dict(scf_mode=mode, snapshots=len(ev))
    for tag in ("rho_at", "learned"):
        out[tag] = dict(mean_scf_iters=float(np.nanmean(col(tag, "scf_iters"))),
                        mean_time_s=float(np.nanmean(col(tag, "time_s"))),
                        mean_iters_to_energy_tol=float(np.nanmean(col(tag, "iters_to_energy_tol"))),
                        mean_time_to_energy_tol_s=float(np.nanmean(col(tag, "time_to_energy_tol_s"))),
                        mean_start_error=float(np.nanmean(col(tag, "start_error"))))
    out["max_dE_per_atom_between_starts"] = float(np.nanmax(dE))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--snapshots", type=int, default=400)
    ap.add_argument("--test", type=int, default=50)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--out", default=None)
    ap.add_argument("--save", default=None)
    ap.add_argument("--load", default=None, help="evaluate a saved network instead of training")
    ap.add_argument("--precision", type=int, default=32, help="SCF mode of the data generation")
    ap.add_argument("--eval-modes", default="32,64", help="SCF modes of the evaluation")
    ap.add_argument("--eval-count", type=int, default=None,
                    help="held-out snapshots per evaluation mode (default: all)")
    ap.add_argument("--rho-triggers", default="4",
                    help="filter passes of the first SCF iteration to evaluate (comma list)")
    ap.add_argument("--cube", default=None,
                    help="with --load: write the learned initial density of snapshot "
                         "--cube-snapshot as a cube file for SPARC's INPUT_DENS_FILE, and stop")
    ap.add_argument("--cube-snapshot", type=int, default=0)
    args = ap.parse_args()
    import torch
    from .psp8 import load_tables
    from .setup import CellSystem
    here = os.path.dirname(os.path.abspath(__file__))
    tab = {"Si": load_tables(os.path.join(here, "..", "tests", "golden", "psp_Si.npz"))}
    dev = torch.device("cuda", 0)
    L0, pos0, _, _ = si64_snapshot(0)
    cs = CellSystem((L0, L0, L0), (52, 52, 52), [("Si", pos0)], tab)
    ntrain = args.snapshots - args.test
    summary = dict(
        system="Si64 (2x2x2 diamond cells, a=20.52 Bohr +-3% strain, sigma 0.1-0.4 Bohr), "
               "52^3 grid, 160 states, LDA_PW, degree 20, TOL_SCF 1e-6",
        train_snapshots=ntrain, test_snapshots=args.test, train_points=ntrain * 52 ** 3)
    if args.load:
        net = DensityMLP.load(args.load)
        if args.cube:
            L, pos, _, _ = si64_snapshot(args.cube_snapshot)
            cs.set_geometry((L, L, L), [("Si", pos)])
            rho0 = initial_density(torch, cs, net, dev)
            write_density_cube(cs, rho0, args.cube, title="Learned initial density")
            print(json.dumps(dict(cube=args.cube, snapshot=args.cube_snapshot,
                                  electrons=float(rho0.sum() * cs.dV))))
            return
    else:
        t0 = time.perf_counter()
        descs, targs, info = generate(torch, cs, list(range(ntrain)), dev, args.precision,
                                      log=lambda s: print(s, flush=True))
        t_gen = time.perf_counter() - t0
        net = DensityMLP()
        t0 = time.perf_counter()
        hist = train(torch, net, descs, targs, dev, epochs=args.epochs,
                     log=lambda s: print(s, flush=True))
        summary.update(generation_s=round(t_gen, 1), training_s=round(time.perf_counter() - t0, 1),
                       loss_history=hist)
        del descs, targs
    held = list(range(ntrain, args.snapshots))[:args.eval_count]
    evals = {}
    triggers = [int(t) for t in args.rho_triggers.split(",")]
    for mode in (int(m) for m in args.eval_modes.split(",")):
        for rt in triggers:
            ev = evaluate(torch, cs, net, held, dev, mode, log=lambda s: print(s, flush=True),
                          scf_kw=dict(rho_trigger=rt))
            name = ("mixed" if mode == 32 else "fp64") + ("" if triggers == [4] else f"_rt{rt}")
            desc = ("mixed (FP32, then FP32 filter + FP64 Rayleigh-Ritz)" if mode == 32
                    else "FP64") + f", {rt} filter passes in the first SCF iteration"
            summary[f"eval_{name}"] = summarize(ev, desc)
            evals[name] = ev
    print(json.dumps(summary), flush=True)
    if args.out:
        with open(args.out, "w") as f:
            json.dump(dict(summary, per_snapshot=evals), f, indent=1)
    if args.save:
        net.save(args.save, meta=summary)


if __name__ == "__main__":
    main()
