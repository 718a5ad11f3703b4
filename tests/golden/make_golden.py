"""Generate the committed golden fixtures from the reference SPARC program.

Needs the reference sources ($SPARC_REFERENCE, default /root/reference) and the oracle build
(`make -C oracle/ref REF=...`). For each system in systems.py it runs the reference's own
set-up, records grid, FD weights and nonlocal projectors, then calls the reference kernels
(Lap_plus_diag_vec_mult_orth, Vnl_vec_mult, Hamiltonian_vectors_mult, ChebyshevFiltering,
poisson_residual) on seeded inputs and stores inputs and outputs in tests/golden/<name>.npz.

usage: python tests/golden/make_golden.py [--ref /path/to/SPARC]
"""
import argparse
import multiprocessing as mp
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import systems  # noqa: E402

sys.path.insert(0, os.path.join(HERE, "..", ".."))
from oracle.refpath import reference_root  # noqa: E402


def flatten_nonlocal(types, images, n_atom):
    """Flatten reference nonlocal data into the library's layout (see include/sparc_gpu.h)."""
    # per-atom projector count: atoms are numbered type by type, as in the reference
    nproj_atom = []
    gamma_atom = []
    for t in types:
        g = []
        off = 0
        for l in range(t["lmax"] + 1):
            if l == t["lloc"]:
                off += int(t["ppl"][l])
                continue
            for p in range(int(t["ppl"][l])):
                g += [t["gamma"][off + p]] * (2 * l + 1)
            off += int(t["ppl"][l])
        for _ in range(t["natom"]):
            nproj_atom.append(len(g))
            gamma_atom.append(np.array(g))
    assert len(nproj_atom) == n_atom
    ip = np.concatenate([[0], np.cumsum(nproj_atom)]).astype(np.int32)
    gamma = np.concatenate(gamma_atom) if gamma_atom else np.zeros(0)
    img_atom = np.array([im["atom_index"] for im in images], dtype=np.int32)
    img_ndc = np.array([len(im["grid_pos"]) for im in images], dtype=np.int32)
    grid_pos = np.concatenate([im["grid_pos"] for im in images]).astype(np.int32)
    chi = np.concatenate([im["chi"].T.reshape(-1) for im in images])  # column-major per image
    return dict(ip_displ=ip, gamma=gamma, img_atom=img_atom, img_ndc=img_ndc,
                grid_pos=grid_pos, chi=chi)


def smooth_potential(rng, Nx, Ny, Nz, L, ncenters=6, amp=-1.5, width=1.2):
    """Sum of periodic Gaussians: a seeded, smooth stand-in for a local potential."""
    x = (np.arange(Nx) + 0.0) * L[0] / Nx
    y = (np.arange(Ny) + 0.0) * L[1] / Ny
    z = (np.arange(Nz) + 0.0) * L[2] / Nz
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    v = np.zeros((Nz, Ny, Nx))
    for c in rng.uniform(0, 1, size=(ncenters, 3)) * np.array(L):
        d = [np.minimum(np.abs(G - cc), Ld - np.abs(G - cc)) for G, cc, Ld in zip((X, Y, Z), c, L)]
        v += amp * np.exp(-(d[0] ** 2 + d[1] ** 2 + d[2] ** 2) / (2 * width ** 2))
    return v.reshape(-1)


def capture(sysd, psp_dir, out_path, ncol, seed, cheb_m, cheb_bounds):
    from ref_capture import RefSystem

    tmp = tempfile.mkdtemp(prefix="sparc_golden_")
    base = systems.write_system(sysd, tmp, psp_dir)
    r = RefSystem(base)
    types, images = r.nonlocal_data()
    flat = flatten_nonlocal(types, images, r.n_atom)
    rng = np.random.default_rng(seed)
    Nd = r.Nd
    x = rng.uniform(-1.0, 1.0, size=(ncol, Nd))
    veff = smooth_potential(rng, r.Nx, r.Ny, r.Nz, r.L)
    fields = r.setup_fields()
    out = dict(
        Nx=r.Nx, Ny=r.Ny, Nz=r.Nz, FDn=r.order // 2, h=r.h, L=r.L, dV=r.dV,
        cx=r.cx, cy=r.cy, cz=r.cz, n_atom=r.n_atom, x=x, veff=veff,
        lap_plus_diag=r.lap_plus_diag(-0.5, 1.0, 0.3, veff, x),
        lap=r.lap_plus_diag(1.0, 0.0, 0.0, None, x[:1]),
        vnl=r.vnl(x),
        hamiltonian=r.hamiltonian(veff, -1.2, x),
        b=fields["b"], rho0=fields["rho0"],
        poisson_residual=r.poisson_residual(0.0, x[0], fields["b"]),
        cheb_m=cheb_m, cheb_bounds=np.array(cheb_bounds),
        **{"nl_" + k: v for k, v in flat.items()},
    )
    Xo, Yo = r.chebyshev(veff, cheb_m, cheb_bounds[0], cheb_bounds[1], cheb_bounds[2], x)
    out["cheb_X"] = Xo
    out["cheb_Y"] = Yo
    np.savez_compressed(out_path, **out)


def capture_kpt(sysd, psp_dir, out_path, ncol, seed, kpts, cheb_m, cheb_bounds):
    """Reference k-point kernels (complex orbitals, Bloch phases) on seeded inputs."""
    from ref_capture import RefKpt, RefSystem

    tmp = tempfile.mkdtemp(prefix="sparc_golden_kpt_")
    base = systems.write_system(sysd, tmp, psp_dir)
    r = RefSystem(base)
    rk = RefKpt(r)
    types, images = rk.images()
    flat = flatten_nonlocal(types, images, r.n_atom)
    coords = np.stack([im["coords"] for im in images]) if images else np.zeros((0, 3))
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (ncol, r.Nd)) + 1j * rng.uniform(-1, 1, (ncol, r.Nd))
    veff = smooth_potential(rng, r.Nx, r.Ny, r.Nz, r.L)
    out = dict(Nx=r.Nx, Ny=r.Ny, Nz=r.Nz, FDn=r.order // 2, h=r.h, L=r.L, dV=r.dV, cx=r.cx,
               cy=r.cy, cz=r.cz, n_atom=r.n_atom, x=x, veff=veff, kpts=rk.kpts[list(kpts)],
               kpt_index=np.array(kpts), img_coords=coords, cheb_m=cheb_m,
               cheb_bounds=np.array(cheb_bounds), **{"nl_" + k: v for k, v in flat.items()})
    for slot, kp in enumerate(kpts):
        out[f"lap_plus_diag_{slot}"] = rk.lap_plus_diag(kp, -0.5, 1.0, 0.3, veff, x)
        out[f"vnl_{slot}"] = rk.vnl(kp, x)
        out[f"hamiltonian_{slot}"] = rk.hamiltonian(kp, veff, -1.2, x)
        Xo, Yo = rk.chebyshev(kp, veff, cheb_m, cheb_bounds[0], cheb_bounds[1], cheb_bounds[2],
                              x)
        out[f"cheb_X_{slot}"] = Xo
        out[f"cheb_Y_{slot}"] = Yo
    np.savez_compressed(out_path, **out)


def capture_scf(sysd, psp_dir, out_npz, out_json, sparc_bin):
    """Reference SCF run of the system (the program itself, single rank) plus the set-up
    data an SCF needs, so the GPU SCF can start from the reference's own inputs."""
    import json
    import subprocess
    from ref_capture import RefSystem, parse_reference_outputs, scf_setup

    tmp = tempfile.mkdtemp(prefix="sparc_scf_")
    base = systems.write_system(sysd, tmp, psp_dir)
    env = dict(os.environ, OMP_NUM_THREADS=str(os.cpu_count() or 1))
    subprocess.run([sparc_bin, "-name", os.path.basename(base)], cwd=tmp, env=env, check=True,
                   stdout=subprocess.DEVNULL)
    ref = parse_reference_outputs(base)
    r = RefSystem(base)
    extra = {}
    if "kpoint_grid" in sysd:
        # k-point run: the reduced k-points with their weights (k1_loc.., kptWts_loc) and the
        # projector images with their coordinates (the Bloch phases need them)
        from ref_capture import RefKpt
        rk = RefKpt(r)
        types, images = rk.images()
        extra = dict(kpts=rk.kpts, kpt_wts=rk.wts,
                     img_coords=np.stack([im["coords"] for im in images]) if images
                     else np.zeros((0, 3)))
    else:
        types, images = r.nonlocal_data()
    flat = flatten_nonlocal(types, images, r.n_atom)
    fields, params = scf_setup(r)
    if sysd.get("spins"):
        # collinear spin: initial [total, up, down] density and magnetization, the reference's
        # spin Vxc on them, and a spin mixing sequence from the same start
        from ref_capture import mix_spin, spin_fields, vxc_spin
        st, rho3, mag0, mprm = spin_fields(r)
        assert st == 1
        vxc2, exc_s = vxc_spin(r, rho3)
        outs = mixing_inputs(rho3[0], nsteps=9, seed=37)
        rng = np.random.default_rng(41)
        mouts = np.array([mag0 * (1.0 + 0.05 * rng.standard_normal(r.Nd)) + 0.01 * o
                          for o in outs])
        rho_m, mag_m = mix_spin(r, rho3[0], mag0, outs, mouts)
        extra.update(rho3_0=rho3, mag0=mag0, vxc0_spin=vxc2, exc0_spin=exc_s,
                     mix_outputs=outs, mix_mag_outputs=mouts, mix_rho=rho_m, mix_mag=mag_m)
        params.update(mprm)
    np.savez_compressed(
        out_npz, Nx=r.Nx, Ny=r.Ny, Nz=r.Nz, FDn=r.order // 2, h=r.h, L=r.L, dV=r.dV,
        cx=r.cx, cy=r.cy, cz=r.cz, n_atom=r.n_atom, Nstates=r.Nstates, **extra,
        **{k: v for k, v in fields.items()}, **{"nl_" + k: v for k, v in flat.items()})
    ref["params"] = params
    ref["system"] = sysd["name"]
    with open(out_json, "w") as fh:
        json.dump(ref, fh, indent=1)


def capture_scf_result(sysd, psp_dir, out_json, sparc_bin):
    """Reference SCF result only (energies, eigenvalues, occupations, forces, wall time), for
    systems too large to store their set-up as a fixture (Si216: the GPU side builds its own
    set-up, which is pinned on the smaller systems)."""
    import json
    import subprocess
    from ref_capture import parse_reference_outputs

    tmp = tempfile.mkdtemp(prefix="sparc_scf_")
    base = systems.write_system(sysd, tmp, psp_dir)
    nthr = os.cpu_count() or 1
    env = dict(os.environ, OMP_NUM_THREADS=str(nthr), OPENBLAS_NUM_THREADS=str(nthr))
    subprocess.run([sparc_bin, "-name", os.path.basename(base)], cwd=tmp, env=env, check=True,
                   stdout=subprocess.DEVNULL)
    ref = parse_reference_outputs(base)
    ref["system"] = sysd["name"]
    ref["where"] = (f"reference program, single rank (MPI stub) + {nthr}-thread OpenBLAS, "
                    "x86 build host")
    with open(out_json, "w") as fh:
        json.dump(ref, fh, indent=1)


def mixing_inputs(rho0, nsteps=9, seed=31):
    """A seeded sequence of SCF output densities around rho0 for the mixing fixtures: each is
    the previous mixed density perturbed by 2 % (multiplicative, seeded), independent of the
    mixer, so the reference and the restatement see the same inputs."""
    rng = np.random.default_rng(seed)
    g = rho0.copy()
    out = []
    for _ in range(nsteps):
        g = g * (1.0 + 0.02 * rng.standard_normal(g.size))
        out.append(g.copy())
    return np.array(out)


def capture_mixing(sysd, psp_dir, out_npz):
    """Golden vectors of the SCF-side solvers from the reference itself on the system's own
    set-up: periodic Pulay mixing over nine iterations (past the history of seven), a Kerker
    preconditioning, and AAR solves of b + (Lap + c) x = 0 (c = 0 and c = -1)."""
    from ref_capture import RefSystem

    tmp = tempfile.mkdtemp(prefix="sparc_mix_")
    base = systems.write_system(sysd, tmp, psp_dir)
    r = RefSystem(base)
    f = r.setup_fields()
    rho0 = f["rho0"]
    outputs = mixing_inputs(rho0)
    mixed = r.mix(rho0, outputs)
    rng = np.random.default_rng(5)
    kf = rho0 * 0.05 * rng.standard_normal(rho0.size)
    Pf = r.kerker(kf, 0.3)
    b = rng.standard_normal(r.Nd)
    aar_c0 = r.aar(0.0, np.zeros(r.Nd), b - b.mean(), 1e-10)
    aar_c1 = r.aar(-1.0, np.zeros(r.Nd), b, 1e-10)
    np.savez_compressed(out_npz, rho0=rho0, outputs=outputs, mixed=mixed, kerker_f=kf,
                        kerker_a=0.3, kerker_Pf=Pf, aar_b=b, aar_x_c0=aar_c0, aar_x_c1=aar_c1,
                        aar_tol=1e-10)


def capture_setup(sysd, psp_dir, out_npz):
    """Inputs and outputs of the reference's per-geometry set-up: parsed pseudopotential
    tables, atom positions as read, pseudocharge cut-offs, pseudocharge densities, initial and
    core densities, Esc, and the nonlocal projectors."""
    from ref_capture import RefSystem

    tmp = tempfile.mkdtemp(prefix="sparc_setup_")
    base = systems.write_system(sysd, tmp, psp_dir)
    r = RefSystem(base)
    types, images = r.nonlocal_data()
    flat = flatten_nonlocal(types, images, r.n_atom)
    out = dict(Nx=r.Nx, Ny=r.Ny, Nz=r.Nz, FDn=r.order // 2, h=r.h, L=r.L, dV=r.dV, cx=r.cx,
               cy=r.cy, cz=r.cz, n_atom=r.n_atom, Ntypes=r.Ntypes,
               atom_pos=r.atom_positions(), **{"nl_" + k: v for k, v in flat.items()})
    nat = []
    for t in range(r.Ntypes):
        tab = r.psd_tables(t)
        out.update({f"t{t}_{k}": v for k, v in tab.items()})
        cut = r.cutoff(t)
        out[f"t{t}_cutoff"] = cut["cutoff"]
        nat.append(cut["natom"])
        out.update(tol_pseudocharge=cut["tol"], ref_cutoff=cut["ref_cutoff"],
                   net_charge=cut["net_charge"])
    out["nAtomv"] = np.array(nat, dtype=np.int32)
    f = r.setup_fields()
    f2 = r.setup_fields2()
    out.update(b=f["b"], b_ref=f2["b_ref"], rho0=f["rho0"], rho_at=f2["rho_at"],
               rho_core=r.core_density(), Esc=f["Esc"], PosCharge=f["PosCharge"],
               NegCharge=f["NegCharge"], Nelectron=f["Nelectron"])
    np.savez_compressed(out_npz, **out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=reference_root(),
                    help="reference tree (default: $SPARC_REFERENCE, else /root/reference)")
    ap.add_argument("--only", choices=["kernels", "kpt", "scf", "scf_kpt", "setup", "si216",
                                       "mixing"],
                    default=None,
                    help="regenerate one group of fixtures only")
    args = ap.parse_args()
    psp_dir = os.path.join(args.ref, "psps")
    ctx = mp.get_context("spawn")
    if args.only == "si216":
        # about half an hour on 8 x86 threads; not part of the default run
        sparc_bin = os.path.join(HERE, "..", "..", "oracle", "_ref", "sparc")
        js = os.path.join(HERE, "Si216_c4_scf_ref.json")
        capture_scf_result(systems.si216_c4(), psp_dir, js, sparc_bin)
        print("wrote", js)
        return
    if args.only in (None, "scf_kpt"):
        sparc_bin = os.path.join(HERE, "..", "..", "oracle", "_ref", "sparc")
        for sysd in (systems.si2_kpt(), systems.al4_spin_kpt()):
            npz = os.path.join(HERE, f"{sysd['name']}_scf.npz")
            js = os.path.join(HERE, f"{sysd['name']}_scf_ref.json")
            p = ctx.Process(target=capture_scf, args=(sysd, psp_dir, npz, js, sparc_bin))
            p.start()
            p.join()
            if p.exitcode != 0:
                raise SystemExit(f"k-point SCF capture failed for {sysd['name']}")
            print("wrote", npz, os.path.getsize(npz), "bytes and", js)
        if args.only == "scf_kpt":
            return
    if args.only in (None, "mixing"):
        path = os.path.join(HERE, "Si8_c1_mixing.npz")
        p = ctx.Process(target=capture_mixing, args=(systems.si8_c1(), psp_dir, path))
        p.start()
        p.join()
        if p.exitcode != 0:
            raise SystemExit("mixing capture failed")
        print("wrote", path, os.path.getsize(path), "bytes")
        if args.only == "mixing":
            return
    if args.only in (None, "setup"):
        for sysd in (systems.si2_small(), systems.si8_c1(), systems.al4_small()):
            path = os.path.join(HERE, f"{sysd['name']}_setup.npz")
            p = ctx.Process(target=capture_setup, args=(sysd, psp_dir, path))
            p.start()
            p.join()
            if p.exitcode != 0:
                raise SystemExit(f"set-up capture failed for {sysd['name']}")
            print("wrote", path, os.path.getsize(path), "bytes")
        if args.only == "setup":
            return
    jobs = [
        (systems.si2_small(), os.path.join(HERE, "si2_small_kernels.npz"), 3, 11, 12,
         (0.5, 40.0, -0.8)),
        (systems.si8_c1(), os.path.join(HERE, "si8_kernels.npz"), 1, 12, 20, (0.4, 45.0, -1.0)),
    ]
    ctx = mp.get_context("spawn")
    for sysd, path, ncol, seed, m, bounds in jobs:
        p = ctx.Process(target=capture, args=(sysd, psp_dir, path, ncol, seed, m, bounds))
        p.start()
        p.join()
        if p.exitcode != 0:
            raise SystemExit(f"capture failed for {sysd['name']}")
        print("wrote", path, os.path.getsize(path), "bytes")
    kpath = os.path.join(HERE, "si2_kpt_kernels.npz")
    p = ctx.Process(target=capture_kpt, args=(systems.si2_kpt(), psp_dir, kpath, 2, 13, (0, 8),
                                              12, (0.5, 40.0, -0.8)))
    p.start()
    p.join()
    if p.exitcode != 0:
        raise SystemExit("k-point capture failed")
    print("wrote", kpath, os.path.getsize(kpath), "bytes")
    sparc_bin = os.path.join(HERE, "..", "..", "oracle", "_ref", "sparc")
    for sysd in (systems.si8_c1(),):
        npz = os.path.join(HERE, f"{sysd['name']}_scf.npz")
        js = os.path.join(HERE, f"{sysd['name']}_scf_ref.json")
        p = ctx.Process(target=capture_scf, args=(sysd, psp_dir, npz, js, sparc_bin))
        p.start()
        p.join()
        if p.exitcode != 0:
            raise SystemExit(f"SCF capture failed for {sysd['name']}")
        print("wrote", npz, os.path.getsize(npz), "bytes and", js)


if __name__ == "__main__":
    main()
