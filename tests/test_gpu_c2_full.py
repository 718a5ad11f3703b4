"""C2 at full size: the degree-20 Chebyshev filter (bounds [-1, 50], cutoff 0.5) over all 512
vectors of the 96^3 grid (h = 0.35, FD order 12) with 64 Gaussian wells and 64 atoms x 9
projectors on 6 Bohr spheres, in FP64 (the drop-in) and FP32 (the mixed mode's filter, with the
tuned kernel forms), through the C ABI on device blocks. Columns spread over the block are
checked against the CPU oracle (oracle/sparc_oracle.c, pinned to the reference's
ChebyshevFiltering, src/eigenSolver.c:722-798): FP64 within 1e-12 and FP32 within 5e-4 of the
largest output magnitude, the tolerances of the smaller filter tests."""
import numpy as np
import pytest

import sparc_gb300 as sg
from oracle.oracle import Oracle
from sparc_gb300.synthetic import microbench_workload

pytestmark = pytest.mark.gpu

COLS = [0, 1, 255, 510, 511]


@pytest.fixture(scope="module")
def c2():
    import torch
    wl = microbench_workload(with_vectors=False)
    g, nl = wl["grid"], wl["nl"]
    ctx = sg.Context(g["Nx"], g["Ny"], g["Nz"], g["FDn"], g["cx"], g["cy"], g["cz"], g["dV"])
    ctx.set_veff(wl["veff"])
    ctx.set_nonlocal(nl["ip_displ"], nl["gamma"], nl["img_atom"], nl["img_ndc"],
                     nl["grid_pos"], nl["chi"])
    Nd = g["Nx"] * g["Ny"] * g["Nz"]
    gen = torch.Generator(device="cuda")
    gen.manual_seed(99)
    X0 = torch.rand((512, Nd), generator=gen, device="cuda", dtype=torch.float64) * 2 - 1
    o = Oracle(g, nl)
    x = X0[COLS].cpu().numpy()
    _, Yo = o.chebyshev(wl["veff"], 20, wl["a"], wl["b"], wl["a0"], x)
    yield ctx, wl, X0, Yo
    ctx.close()


def test_full_size_fp64_filter(gpu_available, c2):
    import torch
    ctx, wl, X0, Yo = c2
    X = X0.clone()
    Y = torch.empty_like(X)
    ctx.ChebyshevFiltering(X, Y, 20, wl["a"], wl["b"], wl["a0"], precision=sg.SGPU_PREC_FP64)
    y = Y[COLS].cpu().numpy()
    assert np.abs(y - Yo).max() <= 1e-12 * np.abs(Yo).max()


def test_full_size_fp32_filter(gpu_available, c2):
    import torch
    ctx, wl, X0, Yo = c2
    ctx.autotune(ncol=512)
    X = X0.float()
    Y = torch.empty_like(X)
    ctx.ChebyshevFiltering_f32(X, Y, 20, wl["a"], wl["b"], wl["a0"])
    assert ctx.kernel_status() == 0
    y = Y[COLS].double().cpu().numpy()
    # the FP32 input is the rounded FP64 block: compare against the oracle on that input
    ctx2_in = X0[COLS].float().double().cpu().numpy()
    from oracle.oracle import Oracle
    o = Oracle(wl["grid"], wl["nl"])
    _, Yo32 = o.chebyshev(wl["veff"], 20, wl["a"], wl["b"], wl["a0"], ctx2_in)
    assert np.abs(y - Yo32).max() <= 5e-4 * np.abs(Yo32).max()
