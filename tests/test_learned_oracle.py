"""The learned-density oracle checked against itself (CPU only): its analytic gradient against
central finite differences, BF16 rounding, and descriptor invariances."""
import numpy as np

from oracle import mlp_oracle as mo


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0], dtype=np.float32)
    r = mo.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # exactly halfway to 1.0078125: ties to even
    assert r[2] == 1.0078125
    assert abs(r[3] - (-3.140625)) < 1e-12
    assert r[4] == 0.0


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    nin, width, n = 24, 16, 40
    _, total = mo.layout(nin, width)
    # weights representable in BF16 so the rounding does not move under the perturbation
    p = mo.bf16(rng.normal(0, 0.3, total).astype(np.float32))
    shift, scale = rng.normal(0, 1, nin), rng.uniform(0.5, 2, nin)
    x, t = rng.normal(0, 1, (n, nin)), rng.normal(0, 1, n)
    loss, g = mo.loss_grad(p, shift, scale, x, t, 1.0, nin, width)
    offs, _ = mo.layout(nin, width)
    # biases are not rounded: check them by finite differences, weights by a directional test
    for (ow, ob, fi, fo) in offs:
        for j in range(min(fo, 3)):
            e = np.zeros(total)
            e[ob + j] = 1e-6
            lp, _ = mo.loss_grad(p + e, shift, scale, x, t, 1.0, nin, width)
            lm, _ = mo.loss_grad(p - e, shift, scale, x, t, 1.0, nin, width)
            assert abs((lp - lm) / 2e-6 - g[ob + j]) < 1e-6 * max(1.0, abs(g[ob + j]))
    # weights: the loss as a function of unrounded weights (replace bf16 by identity)
    orig = mo.bf16
    try:
        mo.bf16 = lambda v: np.asarray(v, dtype=np.float64)
        loss0, g0 = mo.loss_grad(p, shift, scale, x, t, 1.0, nin, width)
        for (ow, ob, fi, fo) in offs:
            for q in (0, fi * fo // 2, fi * fo - 1):
                e = np.zeros(total)
                e[ow + q] = 1e-6
                lp, _ = mo.loss_grad(p + e, shift, scale, x, t, 1.0, nin, width)
                lm, _ = mo.loss_grad(p - e, shift, scale, x, t, 1.0, nin, width)
                assert abs((lp - lm) / 2e-6 - g0[ow + q]) < 1e-6 * max(1.0, abs(g0[ow + q]))
    finally:
        mo.bf16 = orig


def test_descriptors_invariant_under_rotation_of_the_environment():
    # one atom near a point: swapping x and y axes must leave the descriptors unchanged
    cell = (12.0, 12.0, 12.0)
    a = mo.descriptors(cell, [[6.3, 5.1, 6.0]], (8, 8, 8))
    b = mo.descriptors(cell, [[5.1, 6.3, 6.0]], (8, 8, 8))
    # point (i, j, k) of the first equals point (j, i, k) of the second
    a3 = a.reshape(8, 8, 8, 24)
    b3 = b.reshape(8, 8, 8, 24)
    assert np.allclose(a3, b3.transpose(0, 2, 1, 3), atol=1e-12)
