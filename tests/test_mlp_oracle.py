"""The MLP oracle's analytic gradients against finite differences (CPU)."""
import numpy

from oracle import mlp_ref


def test_oracle_gradients_match_finite_differences():
    rng = numpy.random.default_rng(0)
    dIn, H, d, B = 5, 7, 3, 4
    n = H * dIn + H + H * H + H + 2 * d * H + 2 * d
    p = (0.3 * rng.standard_normal(n)).astype(numpy.float64)
    x = rng.standard_normal((B, dIn))
    t = rng.standard_normal((B, d))
    loss, g = mlp_ref.loss_and_grads(p, x, t, dIn, H, 2 * d)
    # biases are not rounded to BF16, so finite differences are exact there
    for i in [H * dIn, H * dIn + 3, H * dIn + H + H * H + 1, n - 1, n - 2 * d, n - d - 1]:
        e = 1e-6
        p2 = p.copy()
        p2[i] += e
        l2, _ = mlp_ref.loss_and_grads(p2, x, t, dIn, H, 2 * d)
        assert abs(g[i] - (l2 - loss) / e) < 1e-5 * (1 + abs(g[i]))


def test_bf16_rounding():
    a = numpy.array([1.0, 1.00390625, 1.005859375, -3.14159265, 1e-3], numpy.float32)
    r = mlp_ref.bf16(a)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-12


def test_nan_targets_are_left_out():
    rng = numpy.random.default_rng(1)
    dIn, H, d, B = 6, 5, 3, 4
    n = H * dIn + H + H * H + H + 2 * d * H + 2 * d
    p = 0.3 * rng.standard_normal(n)
    x = rng.standard_normal((B, dIn))
    t = rng.standard_normal((B, d))
    t[0, 1] = numpy.nan
    t[2, :] = numpy.nan
    loss, g = mlp_ref.loss_and_grads(p, x, t, dIn, H, 2 * d)
    assert numpy.isfinite(loss) and numpy.isfinite(g).all()
    keep = numpy.isfinite(t)
    l_masked = loss
    t3 = numpy.where(keep, t, 0.0)   # the same targets with the masked ones scored as 0
    l3, _ = mlp_ref.loss_and_grads(p, x, t3, dIn, H, 2 * d)
    assert l3 != l_masked
    y, _ = mlp_ref.forward(p, x, dIn, H, 2 * d)
    s = numpy.clip(y[:, d:], mlp_ref.S_MIN, mlp_ref.S_MAX)
    r = (t3 - y[:, :d]) * numpy.exp(-s)
    direct = float(numpy.where(keep, s + 0.5 * r * r, 0.0).sum() / B)
    assert abs(direct - l_masked) < 1e-12
