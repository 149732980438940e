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
