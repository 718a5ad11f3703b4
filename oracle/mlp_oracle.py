"""CPU oracle for the learned-density kernels (test infrastructure only).

Restates in numpy (float64 arithmetic on BF16-rounded weights, as the device kernels use them)
the descriptors of sgpu_density_descriptors and the forward pass, loss and gradient of the
network of sgpu_mlp_* (sparc_gb300/csrc/mlp.cu). Its own backward pass is checked against
finite differences in tests/test_learned_oracle.py, and the device kernels are checked
against it in tests/test_gpu_learned.py. There is no counterpart in the reference program
(parity for this part is unpinned by construction: the reference has no learned density).
"""
import numpy as np

NBINS = 8


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even) and back to float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def layout(nin, width):
    """Offsets of (W, b) for the three hidden layers and the output layer."""
    offs = []
    off = 0
    fi = [nin, width, width, width]
    fo = [width, width, width, 1]
    for l in range(4):
        offs.append((off, off + fi[l] * fo[l], fi[l], fo[l]))
        off += fi[l] * fo[l] + fo[l]
    return offs, off


def unpack(params, nin, width):
    offs, _ = layout(nin, width)
    Ws, bs = [], []
    for (ow, ob, fi, fo) in offs:
        Ws.append(bf16(params[ow:ow + fi * fo]).reshape(fi, fo))
        bs.append(np.asarray(params[ob:ob + fo], dtype=np.float64))
    return Ws, bs


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(params, shift, scale, x, nin, width):
    Ws, bs = unpack(params, nin, width)
    a = (np.asarray(x, dtype=np.float64) - shift) * scale
    cache = [a]
    zs = []
    for l in range(3):
        z = a @ Ws[l] + bs[l]
        a = silu(z)
        zs.append(z)
        cache.append(a)
    y = (a @ Ws[3] + bs[3])[:, 0]
    return y, zs, cache


def loss_grad(params, shift, scale, x, target, tscale, nin, width):
    """(loss, gradient) of mean (net(x) - tscale*target)^2; the gradient uses the BF16 weights
    in the backward products and is taken with respect to the FP32 master parameters."""
    Ws, bs = unpack(params, nin, width)
    y, zs, acts = forward(params, shift, scale, x, nin, width)
    n = x.shape[0]
    r = y - tscale * np.asarray(target, dtype=np.float64)
    loss = float(np.mean(r * r))
    dy = 2.0 * r / n
    offs, total = layout(nin, width)
    g = np.zeros(total)
    ow, ob, fi, fo = offs[3]
    g[ow:ow + fi] = acts[3].T @ dy
    g[ob] = dy.sum()
    dH = np.outer(dy, Ws[3][:, 0])
    for l in (2, 1, 0):
        dZ = dH * dsilu(zs[l])
        ow, ob, fi, fo = offs[l]
        g[ow:ow + fi * fo] = (acts[l].T @ dZ).reshape(-1)
        g[ob:ob + fo] = dZ.sum(axis=0)
        dH = dZ @ Ws[l].T
    return loss, g


def descriptors(cell, atom_pos, N, rcut=6.0, width=0.5):
    """The 24 per-point descriptors (point-major) of a periodic orthogonal cell."""
    cell = np.asarray(cell, dtype=np.float64)
    h = cell / np.array(N)
    imgs = []
    for p in np.asarray(atom_pos, dtype=np.float64):
        lo = np.floor((-rcut - p) / cell).astype(int)
        hi = np.ceil((cell + rcut - p) / cell).astype(int)
        for r in range(lo[2], hi[2] + 1):
            for q in range(lo[1], hi[1] + 1):
                for s in range(lo[0], hi[0] + 1):
                    c = p + np.array([s, q, r]) * cell
                    if np.all(c >= -rcut) and np.all(c <= cell + rcut):
                        imgs.append(c)
    imgs = np.array(imgs)
    Nx, Ny, Nz = N
    k, j, i = np.meshgrid(np.arange(Nz), np.arange(Ny), np.arange(Nx), indexing="ij")
    P = np.stack([i.ravel() * h[0], j.ravel() * h[1], k.ravel() * h[2]], axis=1)
    s = np.zeros((P.shape[0], NBINS))
    v1 = np.zeros((P.shape[0], NBINS, 3))
    v2 = np.zeros((P.shape[0], NBINS, 5))
    mu = rcut * np.arange(NBINS) / (NBINS - 1)
    c2a, c2b, c2c = 0.5 * np.sqrt(15 / np.pi), 0.25 * np.sqrt(5 / np.pi), 0.25 * np.sqrt(15 / np.pi)
    for c in imgs:
        d = c - P
        r = np.sqrt((d * d).sum(axis=1))
        m = r < rcut
        if not m.any():
            continue
        dm, rm = d[m], r[m]
        u = dm / np.maximum(rm, 1e-8)[:, None]
        fc = 0.5 * (np.cos(np.pi * rm / rcut) + 1.0)
        g = fc[:, None] * np.exp(-0.5 * ((rm[:, None] - mu[None, :]) / width) ** 2)
        y2 = np.stack([c2a * u[:, 0] * u[:, 1], c2a * u[:, 1] * u[:, 2],
                       c2b * (2 * u[:, 2] ** 2 - u[:, 0] ** 2 - u[:, 1] ** 2),
                       c2a * u[:, 2] * u[:, 0], c2c * (u[:, 0] ** 2 - u[:, 1] ** 2)], axis=1)
        s[m] += g
        v1[m] += g[:, :, None] * u[:, None, :]
        v2[m] += g[:, :, None] * y2[:, None, :]
    return np.concatenate([s, (v1 ** 2).sum(axis=2), (v2 ** 2).sum(axis=2)], axis=1)
