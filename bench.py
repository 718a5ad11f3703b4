"""Benchmark of the CheFSI hot path: the Chebyshev filter / stencil microbenchmark.

Workload (one "step"): a degree-20 Chebyshev filter (bounds a0=-1, cutoff a=0.5, b=50 Ha)
over 512 orbital vectors on a 96^3 periodic grid (h = 0.35 Bohr, FD order 12), with a local
potential of 64 seeded Gaussians and a nonlocal part of 64 atoms x 9 projectors on 6 Bohr
spheres. Synthetic seeded inputs; the block (3.6 GB in FP64, 1.8 GB in FP32) is larger than
L2, so no flush is needed between steps.

Metric: algorithmic GB/s of the filter, N*Ns*s*(3m-1) bytes per step (the first degree reads X
and writes Y, each later one reads Y and X and writes the new iterate).

  value  : the plain FP64 filter on device-resident FP64 blocks (sgpu_ChebyshevFiltering,
           SGPU_PREC_FP64), the reference's own precision
  e2e    : the same FP64 filter through the drop-in call with FP64 host arrays, host<->device
           copies of X in and X, Y out inside the timed region
  roofline / rooflines : per kernel, algorithmic bytes per launch over the launch's device
           time (the library's own CUDA events) against the measured HBM copy peak; for the
           FP64 kernels also their flops against this GPU's measured FP64 FMA rate
  parity : the timed FP64 and FP32 filters' own outputs (first columns) against the CPU oracle
           on the same input columns
  fp32   : the FP32 filter of the mixed-precision mode (sgpu_ChebyshevFiltering_f32), with its
           e2e and the rooflines of its stencil and fused nonlocal kernel
  scf    : SCF time-to-solution, Si8 (26^3, 32 states) from the reference's set-up fields
  scf_c4 : SCF time-to-solution, Si216 (77^3, 520 states, degree 24) set up on the device from
           the psp8 tables: plain FP64 CheFSI vs the mixed-precision mode, with energy and
           eigenvalue differences against the FP64 run and the reference program's run

usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N3 = (96, 96, 96)
NCOL = 512
M = 20
METRIC = "CheFSI SCF time-to-solution at 1e-5 Ha/atom vs plain FP64 GPU; stencil GB/s"
WORKLOAD = ("chebyshev_filter_microbench: 96^3 periodic grid h=0.35 Bohr, FD order 12, "
            "512 vectors U[-1,1], degree 20, bounds [-1,50] cutoff 0.5, 64 Gaussian Veff, "
            "64 atoms x 9 projectors on 6 Bohr spheres")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ncol", type=int, default=NCOL)
    ap.add_argument("--cpu-cols", type=int, default=16,
                    help="columns in the bounded CPU-baseline sample")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-scf", action="store_true", help="skip the SCF time-to-solution blocks")
    ap.add_argument("--no-c4", action="store_true", help="skip the 216-atom SCF block")
    ap.add_argument("--no-c3", action="store_true", help="skip the batched k-point/spin block")
    ap.add_argument("--rr-gemm", action="store_true",
                    help="only time the Rayleigh-Ritz products at the Si216 shapes")
    ap.add_argument("--rr-grid", type=int, default=77,
                    help="grid edge of the --rr-gemm case (77: Si216; smaller for profiling)")
    ap.add_argument("--rr-ns", type=int, default=520, help="states of the --rr-gemm case")
    ap.add_argument("--rr-only", default=None,
                    help="comma-separated --rr-gemm modes to run (fp32_tc, fp64_tc, fp32, "
                         "fp32_eager, fp32_bf16_split, fp64)")
    ap.add_argument("--fp64-only", action="store_true",
                    help="only the FP64 filter steps, no tuning or side blocks (profiling)")
    ap.add_argument("--fp32-only", "--no-fp64", dest="fp32_only", action="store_true",
                    help="only the tuner and the tuned FP32 filter steps with their kernel times, "
                         "no FP64 headline or side blocks (profiling)")
    ap.add_argument("--c3-prec", type=int, default=0, choices=[0, 32, 64],
                    help="C3 block: only this precision (0: both)")
    ap.add_argument("--c3-filter-only", action="store_true",
                    help="C3 block: the batched filter timing only (no CheFSI pass, no per-block "
                         "calls)")
    ap.add_argument("--c3-only", action="store_true",
                    help="print only the batched k-point/spin block (profiling)")
    ap.add_argument("--stencil-variant", type=int, default=None,
                    help="use this FP32 stencil variant instead of the tuned one (profiling)")
    ap.add_argument("--nl-apply", type=int, default=None,
                    help="use this nonlocal apply form instead of the tuned one (profiling)")
    ap.add_argument("--nl-fuse", type=int, default=None, choices=[0, 2, 3, 4],
                    help="force the projections carried across filter degrees off (0) or on "
                         "with 2 or 4 columns per thread")
    ap.add_argument("--switch-error", type=float, default=1e-4,
                    help="SCF error below which the mixed SCF blocks (C3, C4) move to FP64 / "
                         "complex128")
    ap.add_argument("--nl-project", type=int, default=None,
                    help="use this FP32 projection form instead of the tuned one (profiling)")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                maxs.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sms:
            return None
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": max(maxs),
                "reasons": sorted(reasons), "samples": len(sms)}


def cpu_baseline(wl, ncols, threads=None, X=None):
    """The CPU oracle (a port of the reference's filter) on a bounded sample of the same
    workload: ncols of the 512 vectors (X, or seeded ones), same grid, potential, projectors
    and degree. Returns (baseline record, filtered block)."""
    from oracle.oracle import Oracle
    o = Oracle(wl["grid"], wl["nl"])
    if threads:
        o.set_threads(threads)
    Nd = N3[0] * N3[1] * N3[2]
    if X is None:
        rng = np.random.default_rng(7)
        X = rng.uniform(-1.0, 1.0, size=(ncols, Nd))
    t0 = time.perf_counter()
    _, Yo = o.chebyshev(wl["veff"], M, wl["a"], wl["b"], wl["a0"], X)
    dt = time.perf_counter() - t0
    from sparc_gb300.synthetic import filter_bytes
    gbs = filter_bytes(Nd, ncols, M, 8) / dt / 1e9
    return ({"value": round(gbs, 3), "unit": "GB/s", "cores": o.threads(), "kind": "port",
             "sample": f"FP64 degree-{M} filter of {ncols} of the {NCOL} vectors on the same "
                       f"96^3 grid, potential and projectors ({dt:.2f} s)"}, Yo)


def nonlocal_stats(nl):
    """Covered grid points (union of all projector spheres) and (point, projector) entries of
    the nonlocal set: the algorithmic traffic of a nonlocal launch is the covered tile of every
    column (read, or read and written) plus each Chi entry once."""
    nproj = np.diff(nl["ip_displ"])
    nnz = int((nl["img_ndc"].astype(np.int64) * nproj[nl["img_atom"]]).sum())
    return {"ncov": int(np.unique(nl["grid_pos"]).size), "nnz": nnz}


STENCIL_NAMES = ["k_stencil_f32x2<32x16>", "k_stencil_f32_b22<32x16>",
                 "k_stencil_f32_b22<64x8>", "k_stencil_f32x2<64x8>",
                 "k_stencil_f32_b22<32x16, 3 blocks/SM>",
                 "k_stencil_f32_ring<32x16, 1 plane ahead>",
                 "k_stencil_f32_ring<32x16, 2 planes ahead, potential from L2>",
                 "k_stencil_f32_bulk<32x16, 2 planes ahead>",
                 "k_stencil_f32_bulk<32x16, 1 plane ahead>",
                 "k_stencil_f32_ring<32x32, 1 plane ahead>",
                 "k_stencil_f32_ring<32x32, 2 planes ahead, potential from L2>"]


def scf_block(sg, device=0, repeats=2):
    """SCF time-to-solution on the 8-atom Si cell (a = 10.26 Bohr, 26^3 grid, LDA, 32 states,
    degree 20, TOL_SCF 1e-6) from the reference's own set-up fields, in plain FP64 and in the
    mixed-precision mode; energies and eigenvalues checked against the reference run."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from scf_io import load_scf, scf_params
    d, grid, nl, ref = load_scf("Si8_c1")
    ctx = sg.Context(grid["Nx"], grid["Ny"], grid["Nz"], grid["FDn"], grid["cx"], grid["cy"],
                     grid["cz"], grid["dV"], device=device)
    ctx.set_nonlocal(nl["ip_displ"], nl["gamma"], nl["img_atom"], nl["img_ndc"],
                     nl["grid_pos"], nl["chi"])
    n_atom = int(d["n_atom"])
    occ_ref = np.array(ref["occ"])
    lam_ref = np.array(ref["lambda"])
    out = {"system": "Si8 diamond cell, 26^3 grid, 32 states, LDA_PW, degree 20",
           "reference": {"Etot_per_atom": ref["Etot_per_atom"], "scf_iters": ref["scf_iters"],
                         "walltime_s": ref["walltime_s"],
                         "where": "reference program, single rank + 8-thread OpenBLAS, "
                                  "x86 build host (cannot run on the Arm GPU host)"}}
    for name, prec in (("fp64", 64), ("mixed", 32)):
        best = None
        for rep in range(repeats):
            prm = scf_params(sg, d, ref, precision=prec, switch=1e-4, seed=1 + rep)
            res, rho, lam, occ = ctx.scf(prm, d["b"], d["rho0"], d["rho_core"])
            if best is None or res["time_s"] < best[0]["time_s"]:
                best = (res, lam)
        res, lam = best
        occd = occ_ref > 1e-3
        out[name] = {"time_s": round(res["time_s"], 4), "scf_iters": res["scf_iters"],
                     "Etot_per_atom": res["Etot"] / n_atom,
                     "dE_per_atom_vs_ref": abs(res["Etot"] / n_atom - ref["Etot_per_atom"]),
                     "max_occ_eig_err": float(np.abs(lam[occd] - lam_ref[occd]).max()),
                     "converged": bool(res["converged"]),
                     "fp64_switch_iter": res["fp64_switch_iter"]}
    out["speedup_mixed_vs_fp64"] = round(out["fp64"]["time_s"] / out["mixed"]["time_s"], 3)
    ctx.close()
    # forces on the device from the library's own set-up (psp8 tables -> pseudocharges,
    # projectors -> SCF -> local + nonlocal + core-correction forces), against the reference
    # program's forces of the same input
    golden = os.path.join(ROOT, "tests", "golden")
    sys.path.insert(0, golden)
    import systems
    from sparc_gb300.psp8 import load_tables
    from sparc_gb300.setup import CellSystem
    sysd = systems.si8_c1()
    cs = CellSystem(sysd["L"], (26, 26, 26), sysd["species"],
                    {"Si": load_tables(os.path.join(golden, "psp_Si.npz"))}, device=device)
    Fref = np.array(ref["forces"])
    for name, prec in (("fp64", 64), ("mixed", 32)):
        fields = {}
        res, rho, lam, occ = cs.scf(cs.scf_params(Nstates=32, cheb_degree=20, precision=prec),
                                    fields=fields)
        t0 = time.perf_counter()
        F = cs.forces(fields, occ)
        tf = time.perf_counter() - t0
        out[f"forces_{name}"] = {"max_abs_err_vs_ref_Ha_per_Bohr": float(np.abs(F - Fref).max()),
                                 "max_abs_force": float(np.abs(Fref).max()),
                                 "time_s": round(tf, 4)}
    cs.close()
    return out


def scf_c4_block(sg, torch=None, device=0, switch_error=1e-4):
    """SCF time-to-solution on the 216-atom Si cell (3x3x3 diamond cells, a = 30.78 Bohr,
    77^3 grid, 520 states, degree 24, LDA, TOL_SCF 1e-6), set up on the device from the Si
    psp8 tables (sparc_gb300.setup): plain FP64 CheFSI (the reference's settings, 4 filter
    passes in the first SCF iteration) against the mixed-precision mode (FP32 filter and
    BF16x9 products while the SCF error falls, then the FP32 filter with an FP64 Rayleigh-Ritz
    step), from the atomic superposition and from the learned initial density
    (sparc_gb300/data/si64_density_mlp.npz, trained on Si64 snapshots; 8 first-iteration
    passes, which a good start density turns into an almost converged first iteration; the
    mixed run from rho_at with 8 passes is the ablation). Per run: the time to TOL_SCF, and the
    time until the free energy is within 1e-5 Ha/atom of the reference program's converged
    energy (tests/golden/Si216_c4_scf_ref.json; of the FP64 GPU run without it) and stays."""
    golden = os.path.join(ROOT, "tests", "golden")
    sys.path.insert(0, golden)
    import systems
    from sparc_gb300.psp8 import load_tables
    from sparc_gb300.setup import CellSystem, grid_from_mesh
    sysd = systems.si216_c4()
    N = grid_from_mesh(sysd["L"], float(sysd["keys"]["MESH_SPACING"]))
    t0 = time.perf_counter()
    cs = CellSystem(sysd["L"], N, sysd["species"],
                    {"Si": load_tables(os.path.join(golden, "psp_Si.npz"))}, device=device)
    setup_s = time.perf_counter() - t0
    ref = None
    rpath = os.path.join(golden, "Si216_c4_scf_ref.json")
    if os.path.exists(rpath):
        with open(rpath) as f:
            ref = json.load(f)
    out = {"system": "Si216: 3x3x3 diamond Si, a=30.78 Bohr, sigma 0.1 Bohr displacements, "
                     "77^3 grid h=0.40, 520 states, LDA_PW, degree 24, TOL_SCF 1e-6",
           "setup_s": round(setup_s, 3)}
    if ref:
        out["reference"] = {"Etot_per_atom": ref["Etot_per_atom"], "scf_iters": ref["scf_iters"],
                            "walltime_s": ref.get("walltime_s"),
                            "where": ref.get("where", "reference program, x86 build host")}
    from sparc_gb300.learned_density import DensityMLP, energy_reached, initial_density
    mixed = dict(precision=32, fp64_switch_error=switch_error, graded_tail=1,
                 tail_fp64_degrees=0)
    runs = {"fp64": (dict(precision=64), 4, False),
            "mixed": (mixed, 4, False),
            "mixed_rt8": (mixed, 8, False),
            "mixed_learned": (mixed, 8, True)}
    net = None
    npz = os.path.join(ROOT, "sparc_gb300", "data", "si64_density_mlp.npz")
    if torch is not None and os.path.exists(npz):
        net = DensityMLP.load(npz, device=device)
    else:
        runs.pop("mixed_learned")
    # one untimed SCF iteration in each precision first: library handles, workspaces, module
    # loading and the FP32 kernel tuning are paid there, not by the first timed run
    for kw in (dict(precision=64), mixed):
        cs.scf(cs.scf_params(Nstates=520, cheb_degree=24, maxit_scf=1, **kw), fields={})
    e64 = None
    for name, (kw, rt, learned) in runs.items():
        prm = cs.scf_params(Nstates=520, cheb_degree=24, **kw)
        prm.rho_trigger = rt
        t_pred = 0.0
        rho0 = None
        if learned:
            dev = torch.device("cuda", device)
            torch.cuda.synchronize(dev)
            tp = time.perf_counter()
            rho0 = initial_density(torch, cs, net, dev)
            t_pred = time.perf_counter() - tp
        fields = {}
        res, rho, lam, occ = cs.scf(prm, rho_init=rho0, fields=fields)
        tf = time.perf_counter()
        F = cs.forces(fields, occ)  # after the timed SCF: forces are reported, not timed in it
        tf = time.perf_counter() - tf
        del fields
        e = res["Etot"] / cs.n_atom
        e_target = ref["Etot_per_atom"] if ref else (e64 if e64 is not None else e)
        it, ts = energy_reached(res["history"], e_target, cs.n_atom, 1e-5)
        rec = {"time_s": round(res["time_s"] + t_pred, 3), "scf_iters": res["scf_iters"],
               "converged": bool(res["converged"]), "Etot_per_atom": e,
               "fp64_switch_iter": res["fp64_switch_iter"], "first_iteration_passes": rt,
               "start": "learned" if learned else "rho_at",
               "iters_to_1e-5_Ha_per_atom": it,
               "time_to_1e-5_Ha_per_atom_s": None if ts is None else round(ts + t_pred, 3)}
        if learned:
            rec["predict_s"] = round(t_pred, 3)
        rec["forces_time_s"] = round(tf, 3)
        if name == "fp64":
            e64, lam64, F64 = e, lam, F
            rec["max_abs_force"] = float(np.abs(F).max())
        else:
            rec["dE_per_atom_vs_fp64_gpu"] = abs(e - e64)
            occd = occ > 1e-3
            rec["max_occ_eig_diff_vs_fp64_gpu"] = float(np.abs(lam[occd] - lam64[occd]).max())
            rec["max_force_diff_vs_fp64_gpu"] = float(np.abs(F - F64).max())
        if ref:
            rec["dE_per_atom_vs_ref"] = abs(e - ref["Etot_per_atom"])
            lr, orr = np.array(ref["lambda"]), np.array(ref["occ"])
            occd = orr > 1e-3
            rec["max_occ_eig_err_vs_ref"] = float(np.abs(lam[occd] - lr[occd]).max())
            if ref.get("forces"):
                rec["max_force_err_vs_ref_Ha_per_Bohr"] = float(
                    np.abs(F - np.array(ref["forces"])).max())
        out[name] = rec
    out["speedup_mixed_vs_fp64"] = round(out["fp64"]["time_s"] / out["mixed"]["time_s"], 3)
    t64 = out["fp64"]["time_to_1e-5_Ha_per_atom_s"]
    for name in ("mixed", "mixed_rt8", "mixed_learned"):
        tn = out.get(name, {}).get("time_to_1e-5_Ha_per_atom_s")
        if t64 and tn:
            out[f"speedup_to_1e-5_{name}_vs_fp64"] = round(t64 / tn, 3)
    cs.close()
    return out


def al32_system():
    """32-atom FCC Al (2x2x2 conventional cells, a = 7.65 Bohr, L = 15.3 Bohr), seeded
    N(0, 0.05^2) Bohr displacements."""
    rng = np.random.default_rng(20261205)
    fcc = np.array([[0.0, 0.0, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0]])
    a = 7.65
    pos = np.concatenate([(fcc + np.array([i, j, k])) * a for i in range(2) for j in range(2)
                          for k in range(2)], axis=0)
    return 2 * a, pos + rng.normal(0.0, 0.05, size=pos.shape)


# the 10 points of a Gamma-centred 4x4x4 grid that are distinct under the cubic group, in
# units of (2 pi / L) / 4, with their multiplicities (sum 64)
C3_KRED = [(0, 0, 0), (1, 0, 0), (2, 0, 0), (1, 1, 0), (2, 1, 0), (2, 2, 0), (1, 1, 1),
           (2, 1, 1), (2, 2, 1), (2, 2, 2)]
C3_KWTS = [1, 6, 3, 12, 12, 3, 8, 12, 6, 1]


def scf_c3_block(sg, device=0, switch_error=1e-4):
    """Spin-polarised k-point SCF of the C3 system: Al32 (34^3 grid), the 10 weighted
    k-points, collinear spin from seeded +-0.2 moments, 64 states per (k, spin) block (20
    blocks), degree 18, from the library's own set-up. Plain complex128 against the
    complex64-first mixed mode (complex128 below an SCF error of switch_error) and the graded
    mixed mode (after the switch a complex64 filter with a complex128 Rayleigh-Ritz step and
    density); wall time to TOL_SCF
    and the difference of the two energies. (The SCF machinery is pinned to the reference
    program on the Al4 spin k-point run; the reference has no cubic-symmetry k-reduction, so
    this 10-point set has no reference run.)"""
    golden = os.path.join(ROOT, "tests", "golden")
    from sparc_gb300.psp8 import load_tables
    from sparc_gb300.setup import CellSystem
    L, pos = al32_system()
    cs = CellSystem((L, L, L), (34, 34, 34), [("Al", pos)],
                    {"Al": load_tables(os.path.join(golden, "psp_Al.npz"))}, device=device)
    spins = np.random.default_rng(20261206).choice([-0.2, 0.2], size=len(pos))
    kpts = np.array([[2 * np.pi / L * q / 4 for q in kk] for kk in C3_KRED])
    wts = np.array(C3_KWTS, dtype=np.float64)
    out = {"system": "Al32, 34^3, 10 k (cubic-reduced 4x4x4) x 2 spins, 64 states, degree 18, "
                     "smearing 0.003 Ha, TOL_SCF 1e-6", "net_moment_start": float(spins.sum())}
    for tag, prec, graded in (("complex128", sg.SGPU_PREC_FP64, 0),
                              ("complex64_first", sg.SGPU_PREC_FP32, 0),
                              ("complex64_graded", sg.SGPU_PREC_FP32, 1)):
        prm = cs.scf_params(Nstates=64, cheb_degree=18, smearing=0.003, precision=prec,
                            fp64_switch_error=switch_error, graded_tail=graded)
        res, rho, lam, occ = cs.scf_kpt(prm, kpts, wts, atom_spin_z=spins)
        out[tag] = {"time_s": round(res["time_s"], 3), "scf_iters": res["scf_iters"],
                    "converged": res["converged"], "Etot_per_atom": res["Etot"] / cs.n_atom,
                    "net_mag": round(res["net_mag"], 6),
                    "filter_rr_s": round(res["filter_ms"] / 1e3, 3),
                    "switch_iter": res["fp64_switch_iter"]}
    out["dE_per_atom_mixed_vs_complex128"] = abs(out["complex64_first"]["Etot_per_atom"] -
                                                 out["complex128"]["Etot_per_atom"])
    out["speedup_mixed"] = round(out["complex128"]["time_s"] / out["complex64_first"]["time_s"], 3)
    out["dE_per_atom_graded_vs_complex128"] = abs(out["complex64_graded"]["Etot_per_atom"] -
                                                  out["complex128"]["Etot_per_atom"])
    out["speedup_graded"] = round(out["complex128"]["time_s"] /
                                  out["complex64_graded"]["time_s"], 3)
    cs.close()
    return out


def batched_c3_block(sg, torch, dev, device=0, steps=3, prec_only=0, filter_only=False):
    """Batched complex filter and CheFSI pass over (k-point, spin) blocks: 32-atom Al, 34^3
    grid (h = 0.45),
    the 10 symmetry-distinct points of a 4x4x4 k-grid times 2 spins = 20 blocks of 64 states,
    degree 18, projectors and local potential from the device set-up (Al psp8 tables; the two
    spin potentials are the initial potential shifted by +-0.02 Ha, a stand-in for the spin
    splitting). Times one batched filter call (all blocks, one CUDA graph) against one
    k-point filter call per block, and one batched CheFSI pass (the filter, then per block
    H Y, projection, zhegvd and rotation), in complex128 and complex64."""
    golden = os.path.join(ROOT, "tests", "golden")
    from sparc_gb300.psp8 import load_tables
    from sparc_gb300.setup import CellSystem
    from sparc_gb300.synthetic import filter_bytes
    L, pos = al32_system()
    N = (34, 34, 34)
    cs = CellSystem((L, L, L), N, [("Al", pos)],
                    {"Al": load_tables(os.path.join(golden, "psp_Al.npz"))}, device=device)
    ctx = cs.ctx
    Nd = N[0] * N[1] * N[2]
    f = cs.fields
    phi = np.zeros(Nd)
    ctx.Calculate_elecstPotential(f["rho_at"], f["b"], phi, 1e-8)
    vxc, exc = np.zeros(Nd), np.zeros(Nd)
    ctx.Calculate_Vxc_LDA_PW(f["rho_at"], f["rho_core"], 1e-14, vxc, exc)
    v0 = phi + vxc
    ctx.set_veff(np.concatenate([v0 + 0.02, v0 - 0.02]), nspin=2)
    kred = C3_KRED
    ncol, m = 64, 18
    a0, a, b = -0.6, 0.35, 45.0
    gen = torch.Generator(device=dev)
    gen.manual_seed(77)
    out = {"system": "Al32 FCC 2x2x2 (L=15.3 Bohr), 34^3 grid, 10 k x 2 spins = 20 blocks "
                     "of 64 states, degree 18", "blocks": 20}
    stream = torch.cuda.ExternalStream(ctx.stream(), device=dev)
    for name, prec, cdt in (("complex128", 64, torch.complex128), ("complex64", 32, torch.complex64)):
        if prec_only and prec != prec_only:
            continue
        blocks = []
        for kk in kred:
            for spin in (0, 1):
                x = torch.complex(torch.rand((ncol, Nd), generator=gen, device=dev, dtype=torch.float64),
                                  torch.rand((ncol, Nd), generator=gen, device=dev, dtype=torch.float64)).to(cdt)
                blocks.append(dict(spin=spin, k=[2 * np.pi / L * q / 4 for q in kk], X=x,
                                   Y=torch.empty_like(x), X0=x.clone(), a=a, b=b, a0=a0))

        def reset():
            with torch.cuda.stream(stream):
                for bl in blocks:
                    bl["X"].copy_(bl["X0"])

        def batched():
            reset()
            ctx.ChebyshevFiltering_batched(blocks, m, precision=prec)

        def per_block():  # one sgpu_ChebyshevFiltering_kpt call per block (complex128 only)
            reset()
            for bl in blocks:
                ctx.ChebyshevFiltering_kpt(bl["k"], bl["X"], bl["Y"], m, a, b, a0,
                                           spin=bl["spin"], precision=prec)

        def chefsi():  # the filter plus the Rayleigh-Ritz step of every block
            reset()
            lam_last[0] = ctx.CheFSI_batched(blocks, m, precision=prec)

        lam_last = [None]
        res = {}
        def batched_one_point():  # complex64 with the one-point-per-thread stencil
            ctx.set_zstencil_pairs(False)
            try:
                batched()
            finally:
                ctx.set_zstencil_pairs(True)

        runs = [("batched_graph", batched)]
        if prec == 32:
            runs.append(("batched_graph_one_point_stencil", batched_one_point))
        if not filter_only:
            runs += [("chefsi_pass", chefsi)] + \
                ([("per_block_calls", per_block)] if prec == 64 else [])
        for tag, fn in runs:
            fn()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(steps):
                fn()
            torch.cuda.synchronize()
            dt = (time.perf_counter() - t0) / steps
            gbs = 20 * filter_bytes(Nd, ncol, m, 16 if prec == 64 else 8) / dt / 1e9
            res[tag] = {"ms": round(dt * 1e3, 3), "GBs": round(gbs, 1)}
            if tag == "chefsi_pass":  # filter GB/s of the whole pass (the RR step included)
                res[tag]["rayleigh_ritz_ms"] = round(
                    dt * 1e3 - res["batched_graph"]["ms"], 3)
        if "per_block_calls" in res:
            res["speedup_batched"] = round(res["per_block_calls"]["ms"] /
                                           res["batched_graph"]["ms"], 3)
        out[name] = res
        del blocks
    cs.close()
    return out


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    from sparc_gb300.synthetic import microbench_workload
    wl = microbench_workload(N=N3, ncol=NCOL, with_vectors=False)
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(wl, args.cpu_cols)
    for _ in range(args.steps):
        vals.append(cpu_baseline(wl, args.cpu_cols)[0])
    v = statistics.median([c["value"] for c in vals])
    cb = dict(vals[0])
    cb["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "GB/s", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "dtype": "f64", "data": "synthetic", "config": {"workload": WORKLOAD},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "vs_baseline": None}
    print(json.dumps(line), flush=True)


def rr_gemm_block(sg, torch, dev, device=0, steps=3, grid=77, ns=520, only=None):
    """The Rayleigh-Ritz products at the Si216 shapes (77^3 grid at h = 0.40, 520 states):
    the library's tcgen05 split-slice products (FP32-accurate on FP32 blocks, FP64-accurate on
    FP64 blocks), cuBLAS's FP32 forms (BF16x9 emulation requested, eager, three-part BF16
    split) and cuBLAS DGEMM/DSYRK, timed with CUDA events on the library's stream, with the
    achieved TFLOP/s of the rotation (one GEMM, 2 Nd Ns^2 flops) and of the two products of
    the projection (2 Nd Ns^2 each; its H Y apply timed and subtracted)."""
    from sparc_gb300.synthetic import fd_d2_coeffs, gaussian_potential
    N, h = (grid, grid, grid), 0.40
    c = fd_d2_coeffs(6, h)
    rng = np.random.default_rng(7)
    ctx = sg.Context(*N, 6, c, c, c, h ** 3, device=device)
    ctx.set_veff(gaussian_potential(rng, N, h))
    nd = N[0] * N[1] * N[2]
    stream = torch.cuda.ExternalStream(ctx.stream())
    out = {"shape": f"Nd = {nd} ({grid}^3), Ns = {ns}"}
    for name, dt in (("fp32_tc", torch.float32), ("fp64_tc", torch.float64),
                     ("fp32", torch.float32), ("fp32_eager", torch.float32),
                     ("fp32_bf16_split", torch.float32), ("fp64", torch.float64)):
        # *_tc: the library's tcgen05 split-slice products (FP32-accurate on FP32 blocks,
        # FP64-accurate on FP64 blocks); the others: cuBLAS
        if only and name not in only:
            continue
        ctx.set_rr_products({"fp32_tc": 1, "fp64_tc": 2}.get(name, 0))
        ctx.set_gemm_emulation({"fp32_eager": 1, "fp32_bf16_split": 2}.get(name, 0))
        Y = torch.rand((ns, nd), device=dev, dtype=dt) - 0.5
        HY = torch.empty_like(Y)
        X = torch.empty_like(Y)
        Hp = torch.empty((ns, ns), device=dev, dtype=torch.float64)
        Mp = torch.empty_like(Hp)
        Q = (torch.rand((ns, ns), device=dev, dtype=torch.float64) - 0.5) / ns ** 0.5
        f32 = dt == torch.float32
        proj = (lambda: ctx.Project_Hamiltonian_f32(Y, HY, Hp, Mp)) if f32 else \
            (lambda: ctx.Project_Hamiltonian(Y, HY, Hp, Mp))
        rot = (lambda: ctx.Subspace_Rotation_f32(Y, Q, X)) if f32 else \
            (lambda: ctx.Subspace_Rotation(Y, Q, X))
        ham = (lambda: ctx.Hamiltonian_vectors_mult(0.0, Y, HY)) if not f32 else None

        def timed_ms(fn):
            for _ in range(2):
                fn()
            ev0 = torch.cuda.Event(enable_timing=True)
            ev1 = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            ev0.record(stream)
            for _ in range(steps):
                fn()
            ev1.record(stream)
            torch.cuda.synchronize()
            return ev0.elapsed_time(ev1) / steps

        t_rot = timed_ms(rot)
        t_proj = timed_ms(proj)
        gemm = 2.0 * nd * ns * ns
        out[name] = {"rotation_ms": round(t_rot, 3),
                     "rotation_tflops": round(gemm / (t_rot / 1e3) / 1e12, 2),
                     "projection_ms_incl_HY": round(t_proj, 3)}
        if ham is not None:
            t_h = timed_ms(ham)
            out[name]["projection_products_tflops"] = round(
                2 * gemm / ((t_proj - t_h) / 1e3) / 1e12, 2)
        del Y, HY, X
    # the FP64 generalized eigensolve of the subspace (cuSOLVER dsygvd), once per filter pass
    A = torch.rand((ns, ns), device=dev, dtype=torch.float64) - 0.5
    H0 = (A + A.T).contiguous()
    B = torch.rand((ns, ns), device=dev, dtype=torch.float64) / ns
    M0 = (B @ B.T + torch.eye(ns, device=dev, dtype=torch.float64)).contiguous()
    Hp, Mp = H0.clone(), M0.clone()
    lam = torch.empty(ns, device=dev, dtype=torch.float64)

    def eig():
        Hp.copy_(H0)
        Mp.copy_(M0)
        ctx.Solve_Generalized_EigenProblem(Hp, Mp, lam)

    lam_ref = None
    for mode, tag in ((0, "dsygvd"), (1, "potrf_trsm_syevd"), (2, "potrf_trsm_syevj")):
        ctx.set_eig_solver(mode)
        for _ in range(2):
            eig()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            eig()
        torch.cuda.synchronize()
        rec = {"ms": round((time.perf_counter() - t0) / steps * 1e3, 3)}
        if lam_ref is None:
            lam_ref = lam.clone()
            out["generalized_eig_fp64_ms"] = rec["ms"]
        else:
            rec["max_eig_diff_vs_dsygvd"] = float((lam - lam_ref).abs().max().item())
        out.setdefault("generalized_eig", {})[tag] = rec
    ctx.set_eig_solver(0)
    ctx.close()
    return out


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    world, rank, local = dist_env()
    import torch
    import sparc_gb300 as sg
    from sparc_gb300.synthetic import filter_bytes, microbench_workload

    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.c3_only:
        c3 = batched_c3_block(sg, torch, dev, device=local, steps=args.steps,
                              prec_only=args.c3_prec, filter_only=args.c3_filter_only)
        if not args.no_scf:
            c3["scf"] = scf_c3_block(sg, device=local, switch_error=args.switch_error)
        print(json.dumps({"batched_c3": c3}), flush=True)
        return
    if args.rr_gemm:
        only = args.rr_only.split(",") if args.rr_only else None
        print(json.dumps({"rayleigh_ritz": rr_gemm_block(sg, torch, dev, device=local,
                                                         steps=args.steps, grid=args.rr_grid,
                                                         ns=args.rr_ns, only=only)}),
              flush=True)
        return

    wl = microbench_workload(N=N3, ncol=args.ncol, with_vectors=False)
    g = wl["grid"]
    Nd = g["Nx"] * g["Ny"] * g["Nz"]
    ncol = args.ncol
    ctx = sg.Context(g["Nx"], g["Ny"], g["Nz"], g["FDn"], g["cx"], g["cy"], g["cz"], g["dV"],
                     device=local)
    ctx.set_veff(wl["veff"])
    nl = wl["nl"]
    ctx.set_nonlocal(nl["ip_displ"], nl["gamma"], nl["img_atom"], nl["img_ndc"],
                     nl["grid_pos"], nl["chi"])
    stream = torch.cuda.ExternalStream(ctx.stream(), device=dev)
    if args.fp64_only:  # the FP64 filter steps alone, for a launch list under a profiler
        Xp0 = torch.rand((ncol, Nd), device=dev, dtype=torch.float64) * 2 - 1
        Xp, Yp = Xp0.clone(), torch.empty_like(Xp0)
        for _ in range(args.warmup + args.steps):
            with torch.cuda.stream(stream):
                Xp.copy_(Xp0)
            ctx.ChebyshevFiltering(Xp, Yp, M, wl["a"], wl["b"], wl["a0"],
                                   precision=sg.SGPU_PREC_FP64)
        torch.cuda.synchronize()
        print(json.dumps({"fp64_only": True, "steps": args.steps}), flush=True)
        return
    # pick the FP32 kernel forms for this grid and block width (stencil variants give
    # identical results)
    variant, variant_ms = ctx.autotune(ncol=ncol)
    if args.stencil_variant is not None:
        variant = args.stencil_variant
        ctx.set_stencil_variant(variant)
    if args.nl_apply is not None:
        ctx.set_nonlocal_apply_variant(args.nl_apply)
    if args.nl_project is not None:
        ctx.set_nonlocal_project_variant(args.nl_project)
    if args.nl_fuse is not None:
        ctx.set_nonlocal_fuse(args.nl_fuse != 0, args.nl_fuse or None)
    forms = ctx.variants()
    fuse_on, fuse_cpl, fuse_ms = ctx.nonlocal_fuse()
    fuse_tc_avail, fuse_tc_ms = ctx.nonlocal_fuse_tc()
    kernel_name = STENCIL_NAMES[variant]
    nls = nonlocal_stats(nl)

    gen = torch.Generator(device=dev)
    gen.manual_seed(1234 + rank)
    X0 = (torch.rand((ncol, Nd), generator=gen, device=dev, dtype=torch.float32) * 2 - 1)
    a, b, a0 = wl["a"], wl["b"], wl["a0"]

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record()
        for _ in range(steps):
            fn()
        with torch.cuda.stream(stream):
            e1.record()
        barrier()
        ms = e0.elapsed_time(e1)
        if world > 1:
            t = torch.tensor([ms], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms / steps

    def profiled(fn, steps, warmup):
        """Time fn; per-kernel device time per step from the library's own events."""
        ctx.profile_enable(True)
        ms = timed(fn, steps, warmup)
        kinds = {}
        for name, kind in (("stencil", sg.KERNEL_STENCIL), ("nl_project", sg.KERNEL_NL_PROJECT),
                           ("nl_apply", sg.KERNEL_NL_APPLY)):
            t, n = ctx.profile_read(kind)
            kinds[name] = (t, n)
        _, launches = ctx.profile_read(sg.KERNEL_KINDS)
        ctx.profile_enable(False)
        # profile counters cover warm-up and timed steps alike: report per step
        nst = steps + warmup
        per_step = {k: round(t / nst, 3) for k, (t, n) in kinds.items()}
        per_launch = {k: (t / n if n else None) for k, (t, n) in kinds.items()}
        return ms, per_step, per_launch, int(launches * steps / nst)

    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            peak = float(json.load(f)["hbm_gbs"])
        peak_src = "measured"
    traffic_tab = {}
    tpath = os.path.join(ROOT, "profiles", "stencil_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic_tab = json.load(f)

    def traffic_of(name, key):
        for ent in traffic_tab.get("kernels", []):  # the captured kernel that matches
            if name.startswith(ent["prefix"]) and key in ent:
                return ent[key]
        return None

    def hbm_roofline(kernel, alg_bytes, launch_ms, traffic):
        ach = alg_bytes / (launch_ms / 1e3) / 1e9
        return {"bound": "hbm", "kernel": kernel, "achieved": round(ach, 1), "peak": peak,
                "unit": "GB/s", "frac": round(ach / peak, 4), "peak_source": peak_src,
                "traffic": traffic, "algorithmic_bytes_per_launch": int(alg_bytes),
                "ms_per_launch": round(launch_ms, 4)}

    if args.fp32_only:  # the tuned FP32 filter alone: kernel times, forms, rooflines
        X, Y = X0.clone(), torch.empty_like(X0)

        def step32_only():
            with torch.cuda.stream(stream):
                X.copy_(X0)
            ctx.ChebyshevFiltering_f32(X, Y, M, a, b, a0)

        ms32, k32_step, k32_launch, _ = profiled(step32_only, args.steps, args.warmup)
        nl_b = (2 * nls["ncov"] * ncol + nls["nnz"]) * 4.0
        out = {"fp32_only": True, "ms_per_filter": round(ms32, 3),
               "GBs": round(filter_bytes(Nd, ncol, M, 4) / (ms32 / 1e3) / 1e9, 1),
               "kernels_per_step_ms": k32_step,
               "ms_per_launch": {k: (round(v, 4) if v else None) for k, v in k32_launch.items()},
               "fused_form": fuse_cpl if fuse_on else 0, "fused_ms_cuda_cores": fuse_ms,
               "fused_ms_tensor_cores": fuse_tc_ms if fuse_tc_avail else None,
               "tuning_ms": ctx.tuning(), "stencil": kernel_name}
        if k32_launch["nl_apply"]:
            out["nl_apply_roofline"] = hbm_roofline("nl_apply", nl_b, k32_launch["nl_apply"],
                                                    None)
        print(json.dumps(out), flush=True)
        return

    # ---------------- headline: the plain FP64 filter (the drop-in), device-resident blocks
    X64_0 = X0.double()
    X64 = X64_0.clone()
    Y64 = torch.empty_like(X64)

    def step64():
        with torch.cuda.stream(stream):  # reset the input block (the filter overwrites X)
            X64.copy_(X64_0)
        ctx.ChebyshevFiltering(X64, Y64, M, a, b, a0, precision=sg.SGPU_PREC_FP64)

    clocks = ClockSampler(local)
    clocks.start()
    ms64, k64_step, k64_launch, launches64 = profiled(step64, args.steps, args.warmup)
    ck = clocks.stop()
    bytes64 = filter_bytes(Nd, ncol, M, 8)
    value = world * bytes64 / (ms64 / 1e3) / 1e9
    y64_sample = Y64[:args.cpu_cols].cpu().numpy()
    del X64, X64_0  # Y64 stays: the FP32 filter's whole output is compared with it below

    # the FP64 kernels are bound by this part's FP64 pipe, not by HBM: the pipe's measured
    # FMA rate is their ceiling
    fp64_tflops = ctx.measure_fp64_rate()
    rl64 = {}
    for kname, label, alg_b, alg_f in (
            ("stencil", "k_stencil_orth<double>", bytes64 / M, Nd * ncol * 61.0),
            ("nl_apply", "k_nl_apply (FP64)", (2 * nls["ncov"] * ncol + nls["nnz"]) * 8.0,
             2.0 * nls["nnz"] * ncol),
            ("nl_project", "k_nl_project (FP64)", (nls["ncov"] * ncol + nls["nnz"]) * 8.0,
             2.0 * nls["nnz"] * ncol)):
        t = k64_launch[kname]
        if not t:
            continue
        ent = hbm_roofline(label, alg_b, t, traffic_of(label, "fp64_bytes_per_launch_at_bench"))
        ach_f = alg_f / (t / 1e3) / 1e12
        ent["fp64_pipe"] = {"achieved_tflops": round(ach_f, 3),
                            "peak_tflops": round(fp64_tflops, 3),
                            "frac": round(ach_f / fp64_tflops, 4),
                            "algorithmic_flops_per_launch": alg_f,
                            "peak_source": "measured FP64 FMA rate of this GPU "
                                           "(sgpu_measure_fp64_rate)"}
        ent["share_of_step"] = round(k64_step[kname] / ms64, 4)
        rl64[kname] = ent
    dom64 = max(rl64, key=lambda k: k64_step[k])

    # ---------------- e2e: the drop-in call with FP64 pinned host arrays, FP64 arithmetic.
    # The call overwrites X, so every step gets its own pinned copy of the input, made
    # before the timed region: a step times exactly the call (copies in, filter, copies out).
    e2e_steps = max(1, min(args.steps, 3))
    Xh0 = X0[:, :].double().cpu()
    Xhs = [Xh0.clone().pin_memory() for _ in range(e2e_steps + 1)]
    Yh = torch.empty_like(Xh0).pin_memory()
    del Xh0

    def e2e_run(prec, steps):
        barrier()
        ctx.ChebyshevFiltering(Xhs[steps], Yh, M, a, b, a0, precision=prec)  # warm-up
        barrier()
        t0 = time.perf_counter()
        for i in range(steps):
            ctx.ChebyshevFiltering(Xhs[i], Yh, M, a, b, a0, precision=prec)
        barrier()
        return (time.perf_counter() - t0) / steps

    e2e_s = e2e_run(sg.SGPU_PREC_FP64, e2e_steps)
    e2e_val = world * bytes64 / e2e_s / 1e9

    # ---------------- FP32 filter (the mixed mode's filter), device-resident FP32 blocks
    X = X0.clone()
    Y = torch.empty_like(X)

    def step32():
        with torch.cuda.stream(stream):
            X.copy_(X0)
        ctx.ChebyshevFiltering_f32(X, Y, M, a, b, a0)

    ms32, k32_step, k32_launch, launches32 = profiled(step32, args.steps, args.warmup)
    bytes32 = filter_bytes(Nd, ncol, M, 4)
    y32_sample = Y[:args.cpu_cols].double().cpu().numpy()
    # every column of the FP32 filter against the FP64 filter of the same input (on the GPU)
    fp32_vs_fp64_all = float(((Y.double() - Y64).abs().max() / Y64.abs().max()).item())
    del Y64
    rl32 = {"stencil": hbm_roofline(kernel_name, bytes32 / M, k32_launch["stencil"],
                                    traffic_of(kernel_name, "fp32_bytes_per_launch_at_bench"))}
    rl32["stencil"]["share_of_step"] = round(k32_step["stencil"] / ms32, 4)
    if k32_launch["nl_apply"]:
        nlname = ("nonlocal apply" if not fuse_on else
                  "k_nl_apply_project_tc (apply + next projection, tensor cores)"
                  if fuse_cpl == 3 else "k_nl_apply_project_range (apply + next projection)")
        nl_b = (2 * nls["ncov"] * ncol + nls["nnz"]) * 4.0
        rl32["nl_apply"] = hbm_roofline(nlname, nl_b, k32_launch["nl_apply"],
                                        traffic_of(nlname, "fp32_bytes_per_launch_at_bench"))
        rl32["nl_apply"]["share_of_step"] = round(k32_step["nl_apply"] / ms32, 4)
    e2e32_s = e2e_run(sg.SGPU_PREC_FP32, e2e_steps)
    # the call a SPARC shim makes for CheFSI, which never reads X after the filter: X input
    # only, Y returned (the input copies are not overwritten, so they are reused)
    barrier()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        ctx.ChebyshevFiltering_y(Xhs[i], Yh, M, a, b, a0, precision=sg.SGPU_PREC_FP32)
    barrier()
    e2e_y_s = (time.perf_counter() - t0) / e2e_steps
    del Xhs, Yh

    # --- the stencil's access mix (two FP32 blocks read, one written) as PyTorch's own
    # elementwise add over blocks of the same size: the bandwidth a plain 2-read/1-write pass
    # reaches on this GPU, beside the copy peak
    Zmix = torch.empty_like(X)

    def mix():
        torch.add(X, Y, alpha=0.5, out=Zmix)

    for _ in range(3):
        mix()
    ev_a = torch.cuda.Event(enable_timing=True)
    ev_b = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev_a.record()
    for _ in range(5):
        mix()
    ev_b.record()
    torch.cuda.synchronize()
    mix_gbs = 3 * X.numel() * 4 / (ev_a.elapsed_time(ev_b) / 5 / 1e3) / 1e9
    del Zmix, X, Y

    # ---------------- parity of this run's own outputs: the CPU oracle filters the same
    # first columns of the same input block (its FP64 run is also the CPU baseline)
    cpu = parity = None
    if rank == 0 and not args.no_cpu:
        cpu, y_cpu = cpu_baseline(wl, args.cpu_cols, X=X0[:args.cpu_cols].double().cpu().numpy())
        scale = float(np.abs(y_cpu).max())
        parity = {"columns": args.cpu_cols,
                  "fp64_max_rel_err": float(np.abs(y64_sample - y_cpu).max() / scale),
                  "fp32_max_rel_err": float(np.abs(y32_sample - y_cpu).max() / scale),
                  "fp64_tol": 1e-12, "fp32_tol": 5e-4,
                  "what": "max |Y_gpu - Y_oracle| / max |Y_oracle| over the first columns "
                          "of the timed filter's own output (FP64 oracle, oracle/sparc_oracle.c)"}
        parity["fp32_vs_fp64_all_columns_max_rel_err"] = fp32_vs_fp64_all
        parity["ok"] = bool(parity["fp64_max_rel_err"] <= 1e-12 and
                            parity["fp32_max_rel_err"] <= 5e-4 and fp32_vs_fp64_all <= 5e-4)
    scf = scf_c4 = None
    if rank == 0 and not args.no_scf:
        scf = scf_block(sg, device=local)
        if not args.no_c4:
            scf_c4 = scf_c4_block(sg, torch, device=local, switch_error=args.switch_error)
    c3 = None
    if rank == 0 and not args.no_c3:
        c3 = batched_c3_block(sg, torch, dev, device=local)
        if not args.no_scf:
            c3["scf"] = scf_c3_block(sg, device=local, switch_error=args.switch_error)

    if rank == 0:
        tune = {"stencil_variant": {"chosen": kernel_name,
                                    "autotune_ms": [round(float(v), 4) for v in variant_ms]},
                "nonlocal_forms": {
                    "apply": ["per point", "staged per chunk", "per point, Chi hoisted",
                              "dense per chunk", "per range, tile in shared memory"][
                        forms["nl_apply"]],
                    "project": ["per image segment", "per range of covered points"][
                        forms["nl_project"]],
                    "autotune_ms": {k: [round(float(v), 4) for v in vs]
                                    for k, vs in ctx.tuning().items()},
                    "projection_carried": fuse_on,
                    "fused_form": {0: "off", 2: "CUDA cores, 2 columns per thread",
                                   3: "tensor cores (tcgen05, three-slice BF16 products)",
                                   4: "CUDA cores, 4 columns per thread"}[fuse_cpl],
                    "fused_apply_project_ms": [round(v, 4) for v in fuse_ms],
                    "fused_apply_project_tc_ms": round(fuse_tc_ms, 4) if fuse_tc_avail
                    else None}}
        line = {
            "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms64, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "parallelism": f"replicas{world}",
                       "l2": "inputs larger than L2 (3.6 GB FP64 block), no flush",
                       "step": "X reset copy + degree-20 FP64 filter over 512 vectors"},
            "roofline": rl64[dom64],
            "rooflines": {"fp64": rl64, "fp32": rl32},
            "kernels_per_step_ms": k64_step,
            "gpu_launches": launches64,
            "e2e": {"value": round(e2e_val, 2), "unit": "GB/s",
                    "h2d_bytes_per_step": int(ncol * Nd * 8),
                    "d2h_bytes_per_step": int(2 * ncol * Nd * 8),
                    "api": "sgpu_ChebyshevFiltering(host FP64 arrays, SGPU_PREC_FP64)"},
            "parity": parity,
            "fp32": {"value": round(world * bytes32 / (ms32 / 1e3) / 1e9, 2), "unit": "GB/s",
                     "ms_per_step": round(ms32, 3), "kernels_per_step_ms": k32_step,
                     "gpu_launches": launches32,
                     "elementwise_2r1w_gbs": round(mix_gbs, 1),
                     "e2e": {"value": round(world * bytes32 / e2e32_s / 1e9, 2), "unit": "GB/s",
                             "api": "sgpu_ChebyshevFiltering(host FP64 arrays, "
                                    "SGPU_PREC_FP32)"},
                     "e2e_x_input_only": {
                         "value": round(world * bytes32 / e2e_y_s / 1e9, 2), "unit": "GB/s",
                         "api": "sgpu_ChebyshevFiltering_y(host FP64 arrays, SGPU_PREC_FP32): "
                                "X input only, as eigSolve_CheFSI uses it"},
                     "tuning": tune},
            "scf": scf,
            "scf_c4": scf_c4,
            "batched_c3": c3,
            "cpu_baseline": cpu,
            "clocks": ck,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
