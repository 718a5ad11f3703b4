"""sgpu_Vnl_vec_mult_noalloc: the nonlocal apply for callers that cannot allocate device
memory (a host application whose pool allocator owns all GPU memory, or one that cannot
accept cudaFree's device-wide synchronisation). It must give the same result as
sgpu_Vnl_vec_mult and as the CPU oracle, on consecutive calls that reuse its fixed scratch
array, leave the device's free memory unchanged, and reject sizes beyond that array.
Collected last (file name) so that a run stopping at the first failure has run every other
test; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

import sparc_gb300 as sg
from sparc_gb300.synthetic import fd_d2_coeffs, synthetic_nonlocal

pytestmark = pytest.mark.gpu

TOL = 1e-12  # same FP64 kernels; the two paths differ only in where alpha is stored


def _case(seed):
    rng = np.random.default_rng(seed)
    N = (28, 24, 20)
    h = 0.4
    c = fd_d2_coeffs(6, h)
    nl = synthetic_nonlocal(rng, N, h, natom=5, rc=2.2)
    ctx = sg.Context(N[0], N[1], N[2], 6, c, c, c, h ** 3)
    ctx.set_nonlocal(nl["ip_displ"], nl["gamma"], nl["img_atom"], nl["img_ndc"],
                     nl["grid_pos"], nl["chi"])
    return ctx, nl, rng


def _noalloc(ctx, x, hx, ncol=None):
    n, ld = x.shape
    return sg.lib().sgpu_Vnl_vec_mult_noalloc(ctx._h, n if ncol is None else ncol, sg._ptr(x),
                                              ld, sg._ptr(hx), ld)


def test_noalloc_matches_vnl_vec_mult_on_consecutive_calls(gpu_available):
    import torch
    from oracle.oracle import Oracle
    ctx, nl, rng = _case(21)
    N = (ctx.Nx, ctx.Ny, ctx.Nz)
    c = fd_d2_coeffs(6, 0.4)
    o = Oracle(dict(Nx=N[0], Ny=N[1], Nz=N[2], FDn=6, cx=c, cy=c, cz=c, dV=0.4 ** 3), nl)
    free = []
    for call in range(3):
        ncol = 7 if call == 0 else 13  # later calls also use more of the shared scratch
        x = rng.uniform(-1, 1, (ncol, ctx.Nd))
        h0 = rng.uniform(-1, 1, (ncol, ctx.Nd))
        ref = h0.copy()
        ctx.Vnl_vec_mult(x, ref)
        xd = torch.from_numpy(x).cuda()
        hd = torch.from_numpy(h0.copy()).cuda()
        torch.cuda.synchronize()
        before = torch.cuda.mem_get_info()[0]
        assert _noalloc(ctx, xd, hd) == 0, sg.lib().sgpu_last_error().decode()
        torch.cuda.synchronize()
        free.append((before, torch.cuda.mem_get_info()[0]))
        got = hd.cpu().numpy()
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err < TOL, (call, err)
        want = o.vnl(x, h0.copy())
        err_o = np.abs(got - want).max() / np.abs(want).max()
        assert err_o < TOL, (call, err_o)
    # the first call may load the library's device image into the context (which holds the
    # scratch array); the calls after it must leave the free device memory as it was
    for before, after in free[1:]:
        assert before == after, free


def test_noalloc_rejects_oversized_and_host_arrays(gpu_available):
    import torch
    ctx, nl, rng = _case(5)
    nproj = int(nl["ip_displ"][-1])
    too_many = (1 << 20) // nproj + 16  # n_proj * round_up(ncol, 8) > 1048576
    # the size is checked before any launch, so small buffers with a large ncol suffice
    x = torch.zeros((2, ctx.Nd), dtype=torch.float64, device="cuda")
    hx = torch.zeros_like(x)
    assert _noalloc(ctx, x, hx, ncol=too_many) == 1
    assert "exceeds the fixed scratch" in sg.lib().sgpu_last_error().decode()
    xh = np.zeros((2, ctx.Nd))
    assert _noalloc(ctx, xh, xh.copy()) == 1
