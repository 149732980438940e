"""TEST INFRASTRUCTURE: FP64 numpy restatement of the learned-proposal MLP
(forward, Gaussian negative-log-density loss, backward), used only to check
the GPU kernels' outputs and gradients.

Network: x -> tanh(W1 x + b1) -> tanh(W2 h1 + b2) -> W3 h2 + b3 = (mu, s),
weights rounded to BF16 (round to nearest even) as the GPU stores them;
loss = mean over rows of sum_i [s_i + (t_i - mu_i)^2 exp(-2 s_i) / 2] with
s clamped to [-12, 6] (zero gradient where clamped); a NaN target leaves its
coordinate out of the loss (zero contribution and gradient).
"""
import numpy

S_MIN, S_MAX = -12.0, 6.0


def bf16(a):
    b = numpy.ascontiguousarray(a, numpy.float32).view(numpy.uint32).astype(numpy.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(numpy.uint32).view(numpy.float32).astype(numpy.float64)


def unpack(params, dIn, H, dOut):
    p = numpy.asarray(params, numpy.float64)
    o = 0
    W1 = p[o:o + H * dIn].reshape(H, dIn); o += H * dIn
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + dOut * H].reshape(dOut, H); o += dOut * H
    b3 = p[o:o + dOut]
    return W1, b1, W2, b2, W3, b3


def forward(params, x, dIn, H, dOut):
    W1, b1, W2, b2, W3, b3 = unpack(params, dIn, H, dOut)
    W1, W2, W3 = bf16(W1), bf16(W2), bf16(W3)
    x = numpy.asarray(x, numpy.float64)
    h1 = numpy.tanh(x @ W1.T + b1)
    h2 = numpy.tanh(h1 @ W2.T + b2)
    return h2 @ W3.T + b3, (x, h1, h2, W1, W2, W3)


def loss_and_grads(params, x, t, dIn, H, dOut):
    y, (x, h1, h2, W1, W2, W3) = forward(params, x, dIn, H, dOut)
    B = x.shape[0]
    d = dOut // 2
    mu, sr = y[:, :d], y[:, d:]
    s = numpy.clip(sr, S_MIN, S_MAX)
    e = numpy.exp(-s)
    t = numpy.asarray(t, numpy.float64)
    on = numpy.isfinite(t)
    r = numpy.where(on, (numpy.where(on, t, 0.0) - mu) * e, 0.0)
    loss = float(numpy.where(on, s + 0.5 * r * r, 0.0).sum() / B)
    dy = numpy.zeros_like(y)
    dy[:, :d] = -r * e / B
    dy[:, d:] = numpy.where(on & (sr > S_MIN) & (sr < S_MAX), (1.0 - r * r) / B, 0.0)
    dW3 = dy.T @ h2
    db3 = dy.sum(0)
    dh2 = (dy @ W3) * (1 - h2 * h2)
    dW2 = dh2.T @ h1
    db2 = dh2.sum(0)
    dh1 = (dh2 @ W2) * (1 - h1 * h1)
    dW1 = dh1.T @ x
    db1 = dh1.sum(0)
    g = numpy.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dW3.ravel(), db3])
    return loss, g
