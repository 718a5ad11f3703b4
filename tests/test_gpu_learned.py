"""GPU checks of the learned initial density (sparc_gb300/csrc/mlp.cu).

* descriptors against the CPU oracle (float32 sums vs float64: 1e-5 relative);
* the network's forward pass, loss and gradient against the oracle (same BF16 weights; FP32
  activations on the device vs float64 in the oracle: 1e-4 relative, normwise);
* Adam lowers the loss on a fixed batch;
* the gain: on 8-atom Si cells (26^3 grid, 32 states) a network trained on 16 converged
  snapshots starts held-out SCFs closer to their solution and needs fewer SCF iterations than
  the superposition of atomic densities, at the same converged energy (1e-5 Ha/atom).
"""
import os

import numpy as np
import pytest

import sparc_gb300 as sg
from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_descriptors_match_oracle(gpu_available):
    import torch
    from sparc_gb300.learned_density import NIN, si_snapshot
    from sparc_gb300.synthetic import fd_d2_coeffs
    L, pos, _, _ = si_snapshot(3, reps=1)
    N = (18, 17, 16)
    h = [L / n for n in N]
    ctx = sg.Context(*N, 6, fd_d2_coeffs(6, h[0]), fd_d2_coeffs(6, h[1]), fd_d2_coeffs(6, h[2]),
                     h[0] * h[1] * h[2])
    desc = torch.empty((int(np.prod(N)), NIN), dtype=torch.float32, device="cuda")
    pos = np.mod(pos, L)
    ctx.density_descriptors((L, L, L), pos, desc)
    ref = mo.descriptors((L, L, L), pos, N)
    got = desc.cpu().numpy().astype(np.float64)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()


def test_mlp_forward_and_gradient_match_oracle(gpu_available):
    import torch
    from sparc_gb300.learned_density import DensityMLP
    rng = np.random.default_rng(11)
    net = DensityMLP(width=128, seed=5)
    shift = rng.normal(0, 1, 24).astype(np.float32)
    scale = rng.uniform(0.5, 2.0, 24).astype(np.float32)
    net.set_normalization(shift, scale)
    p = net.params.astype(np.float64)
    n = 777  # not a multiple of the 64-row tiles
    x = rng.normal(0, 1, (n, 24)).astype(np.float32)
    t = rng.normal(0, 0.05, n).astype(np.float32)
    xd, td = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    y = torch.empty(n, dtype=torch.float32, device="cuda")
    net.forward(xd, y)
    yo, _, _ = mo.forward(p, shift.astype(np.float64), scale.astype(np.float64), x, 24, 128)
    assert np.abs(y.cpu().numpy() - yo).max() <= 1e-4 * max(1.0, np.abs(yo).max())
    net.zero_grad()
    loss = net.loss_grad(xd, td, tscale=10.0)
    lo, go = mo.loss_grad(p, shift.astype(np.float64), scale.astype(np.float64), x, t, 10.0,
                          24, 128)
    assert abs(loss - lo) <= 1e-4 * lo
    g = net.grads.astype(np.float64)
    assert np.linalg.norm(g - go) <= 1e-4 * np.linalg.norm(go)
    # per layer as well, so a small layer cannot hide behind a large one
    offs, _ = mo.layout(24, 128)
    for (ow, ob, fi, fo) in offs:
        sl = slice(ow, ob + fo)
        assert np.linalg.norm(g[sl] - go[sl]) <= 1e-4 * np.linalg.norm(go[sl]) + 1e-12


def test_adam_lowers_the_loss(gpu_available):
    import torch
    from sparc_gb300.learned_density import DensityMLP
    rng = np.random.default_rng(2)
    net = DensityMLP(width=64, seed=3)
    x = torch.from_numpy(rng.normal(0, 1, (4096, 24)).astype(np.float32)).cuda()
    t = torch.from_numpy(np.sin(rng.normal(0, 1, 4096)).astype(np.float32)).cuda()
    first = None
    for it in range(60):
        net.zero_grad()
        l = net.loss_grad(x, t, tscale=1.0)
        first = l if first is None else first
        net.adam_step(3e-3)
    assert l < 0.5 * first


def test_learned_start_reduces_scf_iterations(gpu_available):
    import torch
    from sparc_gb300.learned_density import DensityMLP, evaluate, generate, si_snapshot, train
    from sparc_gb300.psp8 import load_tables
    from sparc_gb300.setup import CellSystem

    def snap(i):
        return si_snapshot(i, reps=1, base_seed=99)

    tab = {"Si": load_tables(os.path.join(GOLDEN, "psp_Si.npz"))}
    L0, pos0, _, _ = snap(0)
    cs = CellSystem((L0, L0, L0), (26, 26, 26), [("Si", pos0)], tab)
    dev = torch.device("cuda", 0)
    kw = dict(Nstates=32, cheb_degree=20)
    descs, targs, _ = generate(torch, cs, list(range(16)), dev, precision=64, snap=snap,
                               scf_kw=kw)
    net = DensityMLP(width=64, seed=7)
    hist = train(torch, net, descs, targs, dev, epochs=30, batch=16384, lr=3e-3)
    assert hist[-1] < hist[0]
    ev = evaluate(torch, cs, net, list(range(16, 20)), dev, precision=64, snap=snap, scf_kw=kw)
    it_at = np.mean([r["rho_at"]["scf_iters"] for r in ev])
    it_ml = np.mean([r["learned"]["scf_iters"] for r in ev])
    err_at = np.mean([r["rho_at"]["start_error"] for r in ev])
    err_ml = np.mean([r["learned"]["start_error"] for r in ev])
    assert err_ml < err_at
    assert it_ml < it_at
    for r in ev:
        assert r["learned"]["converged"] and r["rho_at"]["converged"]
        assert abs(r["learned"]["Etot_per_atom"] - r["rho_at"]["Etot_per_atom"]) < 1e-5
