"""GPU parity of the hot-path kernels, through the C ABI (libsparc_gpu.so).

Reference values: the golden fixtures produced by the reference SPARC program
(tests/golden/*.npz), and the CPU oracle on fresh seeded inputs at other sizes.
Tolerances: FP64 paths 1e-12 relative to the largest output magnitude (the reference and the
GPU differ only by rounding and FMA contraction); FP32 filter 5e-4 relative."""
import numpy as np
import pytest

import sparc_gb300 as sg
from golden_io import CASES, load, rel_err
from oracle.oracle import Oracle
from sparc_gb300.synthetic import fd_d2_coeffs, synthetic_nonlocal

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32_H = 2e-6
TOL32_FILTER = 5e-4


def make_ctx(grid, nl, veff):
    ctx = sg.Context(grid["Nx"], grid["Ny"], grid["Nz"], grid["FDn"], grid["cx"], grid["cy"],
                     grid["cz"], grid["dV"])
    if veff is not None:
        ctx.set_veff(veff)
    if nl is not None:
        ctx.set_nonlocal(nl["ip_displ"], nl["gamma"], nl["img_atom"], nl["img_ndc"],
                         nl["grid_pos"], nl["chi"])
    return ctx


@pytest.mark.parametrize("case", CASES)
def test_golden_stencil(gpu_available, case):
    d, grid, nl = load(case)
    ctx = make_ctx(grid, nl, d["veff"])
    x = d["x"]
    y = np.zeros_like(x)
    ctx.Lap_plus_diag_vec_mult_orth(-0.5, 1.0, 0.3, d["veff"], x, y)
    assert rel_err(y, d["lap_plus_diag"]) < TOL64
    y1 = np.zeros_like(x[:1])
    ctx.Lap_vec_mult(0.0, np.ascontiguousarray(x[:1]), y1)
    assert rel_err(y1, d["lap"]) < TOL64
    r = np.zeros(ctx.Nd)
    ctx.poisson_residual(0.0, np.ascontiguousarray(x[0]), d["b"], r)
    assert rel_err(r, d["poisson_residual"]) < TOL64


@pytest.mark.parametrize("case", CASES)
def test_golden_nonlocal_and_hamiltonian(gpu_available, case):
    d, grid, nl = load(case)
    ctx = make_ctx(grid, nl, d["veff"])
    hx = np.zeros_like(d["x"])
    ctx.Vnl_vec_mult(d["x"], hx)
    assert rel_err(hx, d["vnl"]) < TOL64
    hx2 = np.zeros_like(d["x"])
    ctx.Hamiltonian_vectors_mult(-1.2, d["x"], hx2)
    assert rel_err(hx2, d["hamiltonian"]) < TOL64


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("prec", [sg.SGPU_PREC_FP64, sg.SGPU_PREC_FP32])
def test_golden_chebyshev(gpu_available, case, prec):
    d, grid, nl = load(case)
    ctx = make_ctx(grid, nl, d["veff"])
    X = d["x"].copy()
    Y = np.zeros_like(X)
    b = d["cheb_bounds"]
    ctx.ChebyshevFiltering(X, Y, int(d["cheb_m"]), b[0], b[1], b[2], precision=prec)
    tol = TOL64 if prec == sg.SGPU_PREC_FP64 else TOL32_FILTER
    assert rel_err(Y, d["cheb_Y"]) < tol
    assert rel_err(X, d["cheb_X"]) < tol


GRIDS = [(13, 17, 19), (32, 8, 12), (40, 33, 7), (6, 6, 6), (64, 24, 30)]


def _random_case(shape, seed, natom=3):
    rng = np.random.default_rng(seed)
    h = (0.41, 0.37, 0.45)
    grid = dict(Nx=shape[0], Ny=shape[1], Nz=shape[2], FDn=6, cx=fd_d2_coeffs(6, h[0]),
                cy=fd_d2_coeffs(6, h[1]), cz=fd_d2_coeffs(6, h[2]), dV=h[0] * h[1] * h[2])
    Nd = shape[0] * shape[1] * shape[2]
    veff = rng.normal(0.0, 1.0, Nd)
    nl = synthetic_nonlocal(rng, shape, 0.4, natom=natom, rc=1.6) if natom else None
    return grid, nl, veff, rng


@pytest.mark.parametrize("shape", GRIDS)
def test_random_grids_vs_oracle(gpu_available, shape):
    grid, nl, veff, rng = _random_case(shape, seed=sum(shape))
    Nd = shape[0] * shape[1] * shape[2]
    ctx = make_ctx(grid, nl, veff)
    o = Oracle(grid, nl)
    x = rng.uniform(-1, 1, (5, Nd))
    y = np.zeros_like(x)
    ctx.Lap_plus_diag_vec_mult_orth(0.7, -0.4, 1.3, veff, x, y)
    assert rel_err(y, o.lap_plus_diag(0.7, -0.4, 1.3, veff, x)) < TOL64
    h = np.zeros_like(x)
    ctx.Hamiltonian_vectors_mult(0.25, x, h)
    assert rel_err(h, o.hamiltonian(veff, 0.25, x)) < TOL64
    for m in (1, 2, 3, 8):
        X = x.copy(); Y = np.zeros_like(x)
        ctx.ChebyshevFiltering(X, Y, m, 0.2, 30.0, -3.0)
        Xo, Yo = o.chebyshev(veff, m, 0.2, 30.0, -3.0, x)
        assert rel_err(Y, Yo) < TOL64, m
        assert rel_err(X, Xo) < TOL64, m


def test_fp32_hamiltonian_and_filter_tolerance(gpu_available):
    grid, nl, veff, rng = _random_case((48, 40, 36), seed=5, natom=6)
    Nd = 48 * 40 * 36
    ctx = make_ctx(grid, nl, veff)
    o = Oracle(grid, nl)
    x = rng.uniform(-1, 1, (4, Nd))
    X = x.copy(); Y = np.zeros_like(x)
    ctx.ChebyshevFiltering(X, Y, 20, 0.5, 50.0, -1.0, precision=sg.SGPU_PREC_FP32)
    Xo, Yo = o.chebyshev(veff, 20, 0.5, 50.0, -1.0, x)
    assert rel_err(Y, Yo) < TOL32_FILTER
    assert rel_err(X, Xo) < TOL32_FILTER


@pytest.mark.parametrize("shape", [(48, 40, 36), (45, 19, 30), (52, 20, 17), (8, 12, 6),
                                   (96, 24, 40)])
def test_fp32_stencil_variants_identical(gpu_available, shape):
    """Every FP32 stencil variant (tiles, 2x2 register blocking, 8-byte or 4-byte accesses,
    plane rings fed by cp.async or by bulk copies) gives bit-identical filter output; the
    autotuner picks one of them. Nx % 4 == 0 shapes take the 16-byte and bulk-copy paths,
    including tiles cut by the grid edge (52 x 20), rows that wrap several times in x (Nx = 8)
    and z slabs of exactly the stencil radius (Nz = 6)."""
    grid, nl, veff, rng = _random_case(shape, seed=11, natom=4)
    Nd = shape[0] * shape[1] * shape[2]
    ctx = make_ctx(grid, nl, veff)
    x = rng.uniform(-1, 1, (3, Nd)).astype(np.float32)
    outs = []
    for v in range(sg.STENCIL_VARIANTS):
        ctx.set_stencil_variant(v)
        X = x.copy(); Y = np.zeros_like(x)
        ctx.ChebyshevFiltering_f32(X, Y, 7, 0.5, 50.0, -1.0)
        outs.append((X, Y))
    for X, Y in outs[1:]:
        np.testing.assert_array_equal(Y, outs[0][1])
        np.testing.assert_array_equal(X, outs[0][0])
    best, ms = ctx.autotune(ncol=3)
    assert 0 <= best < sg.STENCIL_VARIANTS and np.all(ms > 0) and np.all(ms < 1e29)
    assert ctx.kernel_status() == 0


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_nonlocal_apply_forms_identical(gpu_available, dtype):
    """The per-point, staged and hoisted nonlocal apply forms give bit-identical results."""
    grid, nl, veff, rng = _random_case((30, 26, 22), seed=21, natom=7)
    Nd = 30 * 26 * 22
    ctx = make_ctx(grid, nl, veff)
    x = rng.uniform(-1, 1, (37, Nd)).astype(dtype)  # not a multiple of any column block
    outs = []
    for v in (0, 1, 2):
        ctx.set_nonlocal_apply_variant(v)
        if dtype == np.float64:
            h = np.zeros_like(x)
            ctx.Hamiltonian_vectors_mult(0.1, x, h)
            outs.append(h)
        else:
            X = x.copy(); Y = np.zeros_like(x)
            ctx.ChebyshevFiltering_f32(X, Y, 3, 0.5, 50.0, -1.0)
            outs.append(Y)
    np.testing.assert_array_equal(outs[0], outs[1])
    np.testing.assert_array_equal(outs[0], outs[2])
    if dtype == np.float32:  # the dense and range forms sum in other orders
        for v in (3, 4):
            ctx.set_nonlocal_apply_variant(v)
            X = x.copy(); Y = np.zeros_like(x)
            ctx.ChebyshevFiltering_f32(X, Y, 3, 0.5, 50.0, -1.0)
            assert rel_err(Y.astype(np.float64), outs[0].astype(np.float64)) < 1e-5, v


@pytest.mark.parametrize("natom,rc,lmax", [(7, 1.6, 2), (40, 3.0, 2), (12, 2.0, 3)])
def test_fp32_projection_forms_agree(gpu_available, natom, rc, lmax):
    """The per-segment and the per-range FP32 projection agree to FP32 rounding, and both
    match the oracle: sparse spheres, heavy overlap (ranges cut by their entry count, work
    items cut by size) and 16 projectors per atom."""
    shape = (30, 26, 22)
    rng = np.random.default_rng(31 + natom)
    h = (0.41, 0.37, 0.45)
    grid = dict(Nx=shape[0], Ny=shape[1], Nz=shape[2], FDn=6, cx=fd_d2_coeffs(6, h[0]),
                cy=fd_d2_coeffs(6, h[1]), cz=fd_d2_coeffs(6, h[2]), dV=h[0] * h[1] * h[2])
    Nd = shape[0] * shape[1] * shape[2]
    veff = rng.normal(0.0, 1.0, Nd)
    nl = synthetic_nonlocal(rng, shape, 0.4, natom=natom, rc=rc, lmax=lmax)
    ctx = make_ctx(grid, nl, veff)
    o = Oracle(grid, nl)
    x = rng.uniform(-1, 1, (70, Nd))  # two column groups of 64, the second partial
    outs = []
    for v in (0, 1):
        ctx.set_nonlocal_project_variant(v)
        X = x.astype(np.float32); Y = np.zeros_like(X)
        ctx.ChebyshevFiltering_f32(X, Y, 3, 0.5, 50.0, -1.0)
        outs.append(Y.astype(np.float64))
    _, Yo = o.chebyshev(veff, 3, 0.5, 50.0, -1.0, x)
    for Y in outs:
        assert rel_err(Y, Yo) < TOL32_FILTER
    assert rel_err(outs[1], outs[0]) < 1e-5


def test_device_pointers_match_host(gpu_available):
    import torch
    grid, nl, veff, rng = _random_case((24, 20, 16), seed=9)
    Nd = 24 * 20 * 16
    ctx = make_ctx(grid, nl, veff)
    x = rng.uniform(-1, 1, (3, Nd))
    Xh = x.copy(); Yh = np.zeros_like(x)
    ctx.ChebyshevFiltering(Xh, Yh, 7, 0.3, 25.0, -2.0)
    Xd = torch.from_numpy(x.copy()).cuda(); Yd = torch.zeros_like(Xd)
    ctx.ChebyshevFiltering(Xd, Yd, 7, 0.3, 25.0, -2.0)
    np.testing.assert_array_equal(Yd.cpu().numpy(), Yh)
    np.testing.assert_array_equal(Xd.cpu().numpy(), Xh)


def test_leading_dimension_padding(gpu_available):
    import ctypes
    grid, nl, veff, rng = _random_case((16, 18, 14), seed=11)
    Nd = 16 * 18 * 14
    ld = Nd + 37
    ctx = make_ctx(grid, nl, veff)
    o = Oracle(grid, nl)
    xb = rng.uniform(-1, 1, (2, ld))
    hb = np.full((2, ld), 7.0)
    rc = sg.lib().sgpu_Hamiltonian_vectors_mult(ctx._h, 0, 2, ctypes.c_double(-0.5),
                                                sg._ptr(xb), ld, sg._ptr(hb), ld)
    assert rc == 0
    ref = o.hamiltonian(veff, -0.5, np.ascontiguousarray(xb[:, :Nd]))
    assert rel_err(hb[:, :Nd], ref) < TOL64
    assert np.all(hb[:, Nd:] == 7.0)  # padding untouched


def test_bad_arguments_fail_with_status(gpu_available):
    grid, nl, veff, rng = _random_case((16, 16, 16), seed=2)
    ctx = make_ctx(grid, nl, veff)
    X = rng.uniform(-1, 1, (1, ctx.Nd)); Y = np.zeros_like(X)
    with pytest.raises(sg.SgpuError):
        ctx.ChebyshevFiltering(X, Y, 5, 0.3, 25.0, -2.0, precision=16)
    with pytest.raises(sg.SgpuError):
        ctx.ChebyshevFiltering(X, Y, 5, 30.0, 25.0, -2.0)  # a > b
    with pytest.raises(sg.SgpuError):
        sg.Context(16, 16, 16, 4, np.ones(5), np.ones(5), np.ones(5), 1.0)  # FD order 8
    with pytest.raises(sg.SgpuError):
        ctx.set_nonlocal([0, 9], np.ones(9), [0], [3], [0, 1, ctx.Nd], np.ones(27))


def test_empty_block_is_a_no_op(gpu_available):
    grid, nl, veff, rng = _random_case((16, 16, 16), seed=4)
    ctx = make_ctx(grid, nl, veff)
    X = np.zeros((0, ctx.Nd)); Y = np.zeros((0, ctx.Nd))
    ctx.ChebyshevFiltering(X, Y, 5, 0.3, 25.0, -2.0)


def test_bounded_wait_reports_and_context_stays_usable(gpu_available):
    """A barrier wait that nothing completes runs out after its bound (about a millisecond
    here), sets the status word and lets the kernel exit; the context then works as before:
    a bulk-copy filter afterwards gives the same result as the cp.async ring and leaves the
    status word clear."""
    grid, nl, veff, rng = _random_case((48, 40, 36), seed=9, natom=3)
    ctx = make_ctx(grid, nl, veff)
    assert ctx.kernel_status() == 0
    assert ctx.check_wait_bound() == 2
    assert ctx.kernel_status() == 0
    x = rng.uniform(-1, 1, (2, ctx.Nd)).astype(np.float32)
    outs = []
    for v in (6, 7):
        ctx.set_stencil_variant(v)
        X = x.copy(); Y = np.zeros_like(x)
        ctx.ChebyshevFiltering_f32(X, Y, 4, 0.5, 50.0, -1.0)
        outs.append(Y)
    np.testing.assert_array_equal(outs[0], outs[1])
    assert ctx.kernel_status() == 0


@pytest.mark.parametrize("lmax,m,cpl", [(2, 20, 2), (2, 20, 4), (3, 7, 2), (3, 7, 4), (2, 1, 4),
                                        (2, 2, 2), (2, 20, 3), (3, 7, 3), (2, 1, 3)])
def test_fp32_filter_with_carried_projections(gpu_available, lmax, m, cpl):
    """Nonlocal projections carried across filter degrees (each degree's range apply also
    projects the iterate it finishes): the FP32 filter matches the FP64 oracle within the FP32
    filter tolerance, and the filter that launches the range apply and the range projection
    separately to FP32 rounding (the two sum the projections in other atomic orders).
    67 columns: two column groups, the second ragged, an odd last pair. cpl 3 is the
    tensor-core form (three-slice BF16 products, FP32-accurate)."""
    shape = (40, 36, 30)
    rng = np.random.default_rng(77 + lmax)
    h = (0.41, 0.37, 0.45)
    grid = dict(Nx=shape[0], Ny=shape[1], Nz=shape[2], FDn=6, cx=fd_d2_coeffs(6, h[0]),
                cy=fd_d2_coeffs(6, h[1]), cz=fd_d2_coeffs(6, h[2]), dV=h[0] * h[1] * h[2])
    Nd = shape[0] * shape[1] * shape[2]
    veff = rng.normal(0.0, 1.0, Nd)
    nl = synthetic_nonlocal(rng, shape, 0.4, natom=9, rc=2.4, lmax=lmax)
    ctx = make_ctx(grid, nl, veff)
    o = Oracle(grid, nl)
    x = rng.uniform(-1, 1, (67, Nd))
    ctx.set_nonlocal_apply_variant(4)
    ctx.set_nonlocal_project_variant(1)
    if cpl == 3:
        assert ctx.nonlocal_fuse_tc()[0]  # at most 64 projector rows at any covered point
    outs = {}
    for fuse in (False, True):
        ctx.set_nonlocal_fuse(fuse, cpl)
        assert ctx.nonlocal_fuse()[:2] == (fuse, cpl if fuse else 0)
        X = x.astype(np.float32); Y = np.zeros_like(X)
        ctx.ChebyshevFiltering_f32(X, Y, m, 0.5, 50.0, -1.0)
        outs[fuse] = (X.astype(np.float64), Y.astype(np.float64))
    Xo, Yo = o.chebyshev(veff, m, 0.5, 50.0, -1.0, x)
    for fuse in (False, True):
        assert rel_err(outs[fuse][1], Yo) < TOL32_FILTER, fuse
        assert rel_err(outs[fuse][0], Xo) < TOL32_FILTER, fuse
    assert rel_err(outs[True][1], outs[False][1]) < 1e-5
    assert rel_err(outs[True][0], outs[False][0]) < 1e-5


@pytest.mark.parametrize("precision,ncol", [(sg.SGPU_PREC_FP64, 150), (sg.SGPU_PREC_FP32, 150),
                                            (sg.SGPU_PREC_FP32, 256)])
def test_host_arrays_stream_through_column_chunks(gpu_available, precision, ncol):
    """Host blocks of >= 128 columns are filtered in column chunks whose copies overlap the
    filter (three device slots, copy-in / filter / copy-out streams). 150 columns: chunks of
    64, 64 and 22, every slot used and the last chunk ragged; 256 columns: the schedule with
    small end chunks (16, 48, 64, 64, 48, 16); leading dimensions padded. The result matches
    the same call on device arrays (one unchunked pass) and the FP64 oracle."""
    import ctypes
    import torch
    grid, nl, veff, rng = _random_case((30, 26, 22), seed=31, natom=5)
    Nd = 30 * 26 * 22
    ctx = make_ctx(grid, nl, veff)
    o = Oracle(grid, nl)
    ld, m = Nd + 5, 5
    x = rng.uniform(-1, 1, (ncol, Nd))
    Xb = np.full((ncol, ld), 3.0); Xb[:, :Nd] = x
    Yb = np.full((ncol, ld), 4.0)
    rc = sg.lib().sgpu_ChebyshevFiltering(ctx._h, 0, sg._ptr(Xb), ld, sg._ptr(Yb), ld, ncol, m,
                                          ctypes.c_double(0.3), ctypes.c_double(25.0),
                                          ctypes.c_double(-2.0), precision)
    assert rc == 0, sg.lib().sgpu_last_error()
    assert np.all(Xb[:, Nd:] == 3.0) and np.all(Yb[:, Nd:] == 4.0)  # padding untouched
    Xd = torch.from_numpy(x.copy()).cuda(); Yd = torch.zeros_like(Xd)
    ctx.ChebyshevFiltering(Xd, Yd, m, 0.3, 25.0, -2.0, precision=precision)
    Yref, Xref = Yd.cpu().numpy(), Xd.cpu().numpy()
    tol = 1e-13 if precision == sg.SGPU_PREC_FP64 else 1e-5
    assert rel_err(Yb[:, :Nd], Yref) < tol
    assert rel_err(Xb[:, :Nd], Xref) < tol
    Xo, Yo = o.chebyshev(veff, m, 0.3, 25.0, -2.0, x)
    tol_o = TOL64 if precision == sg.SGPU_PREC_FP64 else TOL32_FILTER
    assert rel_err(Yb[:, :Nd], Yo) < tol_o
    assert rel_err(Xb[:, :Nd], Xo) < tol_o
    # X as input only: the same Y, X untouched
    Xi = x.copy(); Yi = np.zeros_like(x)
    ctx.ChebyshevFiltering_y(Xi, Yi, m, 0.3, 25.0, -2.0, precision=precision)
    np.testing.assert_array_equal(Xi, x)
    assert rel_err(Yi, Yref) < tol
    with pytest.raises(sg.SgpuError):  # device X would be overwritten in place: refused
        ctx.ChebyshevFiltering_y(Xd, Yd, m, 0.3, 25.0, -2.0, precision=precision)
    assert ctx.kernel_status() == 0


@pytest.mark.parametrize("natom,rc", [(20, 3.0), (6, 2.0)])
def test_tensor_core_fused_form_availability(gpu_available, natom, rc):
    """The tensor-core fused form needs every covered point's atoms to own at most 64
    projector rows. With 16 rows per atom (lmax 3) and points inside five or more spheres no
    tables are built: mode 3 is refused and the tuner keeps a CUDA-core form. Otherwise the
    tables exist and the form is tuned beside the others. Either way the filter matches the
    oracle."""
    rng = np.random.default_rng(5)
    shape, h = (24, 24, 24), 0.4
    grid = dict(Nx=shape[0], Ny=shape[1], Nz=shape[2], FDn=6, cx=fd_d2_coeffs(6, h),
                cy=fd_d2_coeffs(6, h), cz=fd_d2_coeffs(6, h), dV=h ** 3)
    Nd = shape[0] * shape[1] * shape[2]
    veff = rng.normal(0.0, 1.0, Nd)
    nl = synthetic_nonlocal(rng, shape, h, natom=natom, rc=rc, lmax=3)
    cover = np.bincount(nl["grid_pos"], minlength=Nd)  # one image per atom here
    rows_max = 16 * int(cover.max())
    ctx = make_ctx(grid, nl, veff)
    avail, _ = ctx.nonlocal_fuse_tc()
    assert avail == (rows_max <= 64), rows_max
    if not avail:
        with pytest.raises(sg.SgpuError):
            ctx.set_nonlocal_fuse(True, 3)
    ctx.autotune(ncol=16)
    on, form, _ = ctx.nonlocal_fuse()
    assert form in ((0, 2, 3, 4) if avail else (0, 2, 4))
    x = rng.uniform(-1, 1, (16, Nd))
    X = x.astype(np.float32); Y = np.zeros_like(X)
    ctx.ChebyshevFiltering_f32(X, Y, 5, 0.5, 50.0, -1.0)
    Xo, Yo = Oracle(grid, nl).chebyshev(veff, 5, 0.5, 50.0, -1.0, x)
    assert rel_err(Y.astype(np.float64), Yo) < TOL32_FILTER
    if avail:  # a projector set without tables replaces this one: the CUDA-core form takes over
        ctx.set_nonlocal_fuse(True, 3)
        nl2 = synthetic_nonlocal(np.random.default_rng(6), shape, h, natom=20, rc=3.0, lmax=3)
        assert 16 * int(np.bincount(nl2["grid_pos"], minlength=Nd).max()) > 64
        ctx.set_nonlocal(nl2["ip_displ"], nl2["gamma"], nl2["img_atom"], nl2["img_ndc"],
                         nl2["grid_pos"], nl2["chi"])
        assert not ctx.nonlocal_fuse_tc()[0] and ctx.nonlocal_fuse()[:2] == (True, 2)
        X = x.astype(np.float32); Y = np.zeros_like(X)
        ctx.ChebyshevFiltering_f32(X, Y, 5, 0.5, 50.0, -1.0)
        Xo, Yo = Oracle(grid, nl2).chebyshev(veff, 5, 0.5, 50.0, -1.0, x)
        assert rel_err(Y.astype(np.float64), Yo) < TOL32_FILTER
    assert ctx.kernel_status() == 0


@pytest.mark.parametrize("ncol", [1, 2, 63, 64, 65, 128])
@pytest.mark.parametrize("cpl", [2, 4, 3])
def test_carried_projections_column_edges(gpu_available, ncol, cpl):
    """The fused range apply + projection at column counts that end a 64-column group
    exactly, one short, one over, a single column and an odd last pair (each form, cpl 3 the
    tensor-core kernel), against the oracle within the FP32 filter tolerance."""
    grid, nl, veff, rng = _random_case((32, 26, 22), seed=41 + ncol, natom=6)
    Nd = 32 * 26 * 22
    ctx = make_ctx(grid, nl, veff)
    o = Oracle(grid, nl)
    ctx.set_stencil_variant(6)
    ctx.set_nonlocal_apply_variant(4)
    ctx.set_nonlocal_project_variant(1)
    ctx.set_nonlocal_fuse(True, cpl)
    x = rng.uniform(-1, 1, (ncol, Nd))
    X = x.astype(np.float32); Y = np.zeros_like(X)
    ctx.ChebyshevFiltering_f32(X, Y, 4, 0.5, 50.0, -1.0)
    Xo, Yo = o.chebyshev(veff, 4, 0.5, 50.0, -1.0, x)
    assert rel_err(Y.astype(np.float64), Yo) < TOL32_FILTER
    assert rel_err(X.astype(np.float64), Xo) < TOL32_FILTER
    assert ctx.kernel_status() == 0


@pytest.mark.parametrize("mode", ["tc", 0, 1, 2])
def test_fp32_rayleigh_ritz_products(gpu_available, mode):
    """sgpu_Project_Hamiltonian_f32 / sgpu_Subspace_Rotation_f32 against FP64 products of the
    same FP32 inputs, with H from the oracle: the library's tcgen05 split-slice products
    (sgpu_set_rr_products 1) and the cuBLAS forms (sgpu_set_gemm_emulation 0-2); relative
    error within FP32 accumulation over Nd terms (1e-4)."""
    import torch
    grid, nl, veff, rng = _random_case((30, 26, 22), seed=51, natom=4)
    Nd = 30 * 26 * 22
    ctx = make_ctx(grid, nl, veff)
    if mode == "tc":
        ctx.set_rr_products(1)
    else:
        ctx.set_rr_products(0)
        ctx.set_gemm_emulation(mode)
    o = Oracle(grid, nl)
    ncol = 40
    y = rng.uniform(-1, 1, (ncol, Nd)).astype(np.float32)
    Yd = torch.from_numpy(y).cuda(); HYd = torch.zeros_like(Yd)
    Hp = np.zeros((ncol, ncol)); Mp = np.zeros((ncol, ncol))
    ctx.Project_Hamiltonian_f32(Yd, HYd, Hp, Mp)
    y64 = y.astype(np.float64)
    hy = o.hamiltonian(veff, 0.0, y64)
    assert rel_err(HYd.cpu().numpy().astype(np.float64), hy) < TOL32_H * 10
    assert rel_err(Hp, y64 @ hy.T) < 1e-4
    assert rel_err(Mp, y64 @ y64.T) < 1e-4
    q = rng.normal(size=(ncol, ncol))
    Xd = torch.zeros_like(Yd)
    ctx.Subspace_Rotation_f32(Yd, q, Xd)
    # X (column-major Nd x ncol) = Y Q with Q column-major: row n of q holds column n of Q,
    # so row n of the (ncol, Nd) result is sum_k q[n, k] y[k]
    assert rel_err(Xd.cpu().numpy().astype(np.float64), q @ y64) < 1e-4
