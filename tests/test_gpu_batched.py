"""GPU parity of the batched (k-point, spin) filter against one k-point filter call per block.

The per-block k-point filter is itself pinned to the reference's ChebyshevFiltering_kpt
(tests/test_gpu_kpt.py). The batched call must give the same blocks: complex128 to 1e-12 and
complex64 to 1e-5 relative (the projection's atomic additions may land in another order).
Blocks have uneven column counts, different k-points, spins and filter bounds; repeated calls
replay the cached CUDA graph with new inputs; changed shapes re-capture it.
"""
import numpy as np
import pytest

import sparc_gb300 as sg
from golden_io import rel_err
from test_oracle_kpt import load_kpt

pytestmark = pytest.mark.gpu


def make_ctx(d, grid, nl):
    ctx = sg.Context(grid["Nx"], grid["Ny"], grid["Nz"], grid["FDn"], grid["cx"], grid["cy"],
                     grid["cz"], grid["dV"])
    v = d["veff"]
    ctx.set_veff(np.concatenate([v, v + 0.05 * np.cos(np.arange(v.size) * 0.01)]), nspin=2)
    ctx.set_nonlocal(nl["ip_displ"], nl["gamma"], nl["img_atom"], nl["img_ndc"],
                     nl["grid_pos"], nl["chi"])
    ctx.set_kpoint_geometry(d["L"], d["img_coords"])
    return ctx


BLOCKS = [dict(spin=0, kslot=0, ncol=5, a=0.5, b=40.0, a0=-0.8),
          dict(spin=1, kslot=1, ncol=3, a=0.3, b=38.0, a0=-1.0),
          dict(spin=0, kslot=1, ncol=8, a=0.6, b=42.0, a0=-0.7)]


def run(ctx, d, blocks, m, precision, seed):
    import torch
    rng = np.random.default_rng(seed)
    Nd = d["x"].shape[1]
    cdt = torch.complex128 if precision == 64 else torch.complex64
    ref, dev = [], []
    for bl in blocks:
        x = rng.uniform(-1, 1, (bl["ncol"], Nd)) + 1j * rng.uniform(-1, 1, (bl["ncol"], Nd))
        k = d["kpts"][bl["kslot"]]
        X, Y = x.copy(), np.zeros_like(x)
        ctx.ChebyshevFiltering_kpt(k, X, Y, m, bl["a"], bl["b"], bl["a0"], spin=bl["spin"],
                                   precision=precision)
        ref.append((X, Y))
        xd = torch.from_numpy(x).to(cdt).cuda()
        dev.append(dict(spin=bl["spin"], k=k, X=xd, Y=torch.zeros_like(xd), a=bl["a"],
                        b=bl["b"], a0=bl["a0"]))
    ctx.ChebyshevFiltering_batched(dev, m, precision=precision)
    return ref, [(b["X"].cpu().numpy().astype(np.complex128),
                  b["Y"].cpu().numpy().astype(np.complex128)) for b in dev]


@pytest.mark.parametrize("m", [5, 6, 2])
@pytest.mark.parametrize("precision", [64, 32])
def test_batched_matches_per_block(gpu_available, m, precision):
    d, grid, nl = load_kpt()
    ctx = make_ctx(d, grid, nl)
    tol = 1e-12 if precision == 64 else 1e-5
    for seed in (1, 2):  # the second call replays the captured graph
        ref, out = run(ctx, d, BLOCKS, m, precision, seed)
        for (Xr, Yr), (Xo, Yo) in zip(ref, out):
            assert rel_err(Yo, Yr) < tol
            assert rel_err(Xo, Xr) < tol
    # new shapes: the graph is captured again
    ref, out = run(ctx, d, BLOCKS[:2], m, precision, 3)
    for (Xr, Yr), (Xo, Yo) in zip(ref, out):
        assert rel_err(Yo, Yr) < tol


def test_batched_rejects_host_arrays_and_bad_spin(gpu_available):
    import torch
    d, grid, nl = load_kpt()
    ctx = make_ctx(d, grid, nl)
    Nd = d["x"].shape[1]
    x = torch.zeros((2, Nd), dtype=torch.complex128)
    with pytest.raises(sg.SgpuError):
        ctx.ChebyshevFiltering_batched([dict(spin=0, k=(0, 0, 0), X=x, Y=x.clone(), a=0.5,
                                             b=40.0, a0=-1.0)], 4)
    xd = x.cuda()
    with pytest.raises(sg.SgpuError):
        ctx.ChebyshevFiltering_batched([dict(spin=3, k=(0, 0, 0), X=xd, Y=xd.clone(), a=0.5,
                                             b=40.0, a0=-1.0)], 4)


def test_complex64_pair_stencil_matches_one_point_kernel(gpu_available):
    """The complex64 stencil with two points per thread and tabulated Bloch factors against the
    one-point kernel, single-block and batched (FP32 rounding of the factors only)."""
    import torch
    d, grid, nl = load_kpt()
    ctx = make_ctx(d, grid, nl)
    dev = torch.device("cuda", 0)
    gen = torch.Generator(device=dev)
    Nd = ctx.Nd
    outs = {}
    for on in (True, False):
        ctx.set_zstencil_pairs(on)
        gen.manual_seed(5)  # the same inputs for both forms
        blocks = []
        for b, k in enumerate(d["kpts"][:2]):
            x = torch.complex(torch.rand((5, Nd), generator=gen, device=dev, dtype=torch.float32),
                              torch.rand((5, Nd), generator=gen, device=dev, dtype=torch.float32))
            blocks.append(dict(spin=0, k=list(k), X=x, Y=torch.empty_like(x), a=0.5, b=40.0,
                               a0=-0.8))
        ctx.ChebyshevFiltering_batched(blocks, 7, precision=sg.SGPU_PREC_FP32)
        # the single-block call takes complex128 arrays and filters them in complex64
        rng = np.random.default_rng(6)
        xs = rng.uniform(-1, 1, (3, Nd)) + 1j * rng.uniform(-1, 1, (3, Nd))
        ys = np.zeros_like(xs)
        ctx.ChebyshevFiltering_kpt(d["kpts"][1], xs, ys, 7, 0.5, 40.0, -0.8,
                                   precision=sg.SGPU_PREC_FP32)
        outs[on] = [bl["Y"].cpu().numpy() for bl in blocks] + [ys]
    ctx.set_zstencil_pairs(True)
    for a, b in zip(outs[True], outs[False]):
        assert rel_err(a, b) < 2e-6
