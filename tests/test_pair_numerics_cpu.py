"""The numerical methods of the setPrams kernels (csrc/p4g_pmat.cu), replayed
on the CPU with numpy's IEEE FP32 arithmetic, against FP64 references:

  - pairExp: e^x as an FP32 pair (FP64 range reduction x = k ln2 + r, the
    Taylor series of e^r to r^13/13! in pair arithmetic, scaling by 2^k);
  - the eigensystem of a 20-state symmetric form: an FP32 start refined by
    two steps of Ogita and Aishima's method (R = I - X^T X and S = X^T A X in
    FP64; the correction E and the product X E in FP32), with the kernel's
    acceptance rule (second correction <= 1e-7, unresolved coupling <= 256 eps
    ||A||) deciding between the result and the FP64 Jacobi fallback;
  - the P decks as Dot2 compensated sums in FP32 pairs, scaled by
    sqrt(pi_j / pi_i), on skewed compositions.

The GPU tests pin the kernels themselves to the reference core; these check
that the methods, with the kernels' parameters, have the accuracy the design
relies on.  Host-only: no GPU."""
import math

import numpy

f32 = numpy.float32


def fma(a, b, c):
    # an FP32 fused multiply-add: the product of two floats is exact in FP64
    return f32(numpy.float64(a) * numpy.float64(b) + numpy.float64(c))


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def fast_two_sum(a, b):
    s = f32(a + b)
    return s, f32(b - f32(s - a))


def pair_mul(a, b):
    p = f32(a[0] * b[0])
    e = fma(a[0], b[0], -p)
    e = fma(a[0], b[1], e)
    e = fma(a[1], b[0], e)
    return fast_two_sum(p, e)


def pair_add(a, b):
    s, e = two_sum(a[0], b[0])
    e = f32(e + f32(a[1] + b[1]))
    return fast_two_sum(s, e)


def split(x):
    h = f32(x)
    return h, f32(x - numpy.float64(h))


INV_FACT = [split(1.0 / math.factorial(j)) for j in range(14)]


def pair_exp(x):
    if x < -87.0:
        return f32(0.0), f32(0.0)
    k = f32(numpy.rint(f32(f32(x) * f32(1.0 / math.log(2.0)))))
    r = split(x - float(k) * math.log(2.0))   # the kernel's FP64 FMA; within an ulp of it here
    y = INV_FACT[13]
    for j in range(12, -1, -1):
        y = pair_add(pair_mul(y, r), INV_FACT[j])
    sc = f32(2.0 ** int(k))
    return f32(y[0] * sc), f32(y[1] * sc)


def symmetric_form(R, pi):
    Q = R * pi[None, :]
    numpy.fill_diagonal(Q, 0.0)
    numpy.fill_diagonal(Q, -Q.sum(1))
    Q /= -(pi * numpy.diag(Q)).sum()
    sq = numpy.sqrt(pi)
    A = Q * sq[:, None] / sq[None, :]
    return (A + A.T) / 2, sq


def refine(A, X, normA):
    """Two Ogita-Aishima steps as the kernel takes them; returns X, lambda and
    whether the kernel's acceptance rule holds."""
    n = A.shape[0]
    emax = cmax = 0.0
    for _ in range(2):
        G = X.T @ X
        S = X.T @ (A @ X)
        lam = numpy.diag(S) / numpy.diag(G)
        R = numpy.eye(n) - G
        so = numpy.linalg.norm(S - numpy.diag(lam))
        delta = 2.0 * (so + normA * numpy.linalg.norm(R))
        gap = lam[None, :] - lam[:, None]
        off = ~numpy.eye(n, dtype=bool)
        far = (numpy.abs(gap) > delta) & off
        E = (R / 2).astype(f32)
        num = S + lam[None, :] * R                   # FP64 numerator, FP32 division
        E[far] = (num[far].astype(f32) / gap[far].astype(f32)).astype(f32)
        emax = float(numpy.abs(E[far]).max(initial=0.0))
        cmax = float(numpy.abs(S[off & ~far]).max(initial=0.0))
        if not emax <= 1e-3:
            return X, lam, False
        X = X + (X.astype(f32) @ E).astype(numpy.float64)   # the correction in FP32
    ok = emax <= 1e-7 and cmax <= 256 * numpy.finfo(float).eps * normA
    return X, lam, ok


def test_pair_exp_relative_error():
    rng = numpy.random.default_rng(1)
    xs = list(-numpy.abs(rng.standard_normal(400)) * 12) + list(-rng.uniform(0, 1e-3, 100)) + [0.0, -86.9]
    worst = 0.0
    for x in xs:
        h, l = pair_exp(float(x))
        ref = math.exp(x)
        if ref >= 1e-20:
            worst = max(worst, abs(float(h) + float(l) - ref) / ref)
        else:   # near FP32's range limit the low part underflows: negligible beside a deck's terms
            assert abs(float(h) + float(l) - ref) < 1e-30, x
    assert worst < 2e-14, worst
    assert pair_exp(-100.0) == (0.0, 0.0)


def test_refinement_from_fp32_start():
    rng = numpy.random.default_rng(2)
    n = 20
    for trial in range(12):
        R = numpy.exp(rng.normal(0.0, 1.5, (n, n)))
        R = (R + R.T) / 2
        pi = numpy.maximum(rng.dirichlet(numpy.full(n, [0.3, 1.0, 5.0][trial % 3])), 1e-6)
        pi /= pi.sum()
        A, sq = symmetric_form(R, pi)
        _, X32 = numpy.linalg.eigh(A.astype(f32))          # an FP32-accurate start
        X, lam, ok = refine(A, X32.astype(numpy.float64), numpy.linalg.norm(A))
        assert ok, trial
        w, U = numpy.linalg.eigh(A)
        assert numpy.abs(X.T @ X - numpy.eye(n)).max() < 1e-13
        for t in (0.01, 0.5, 3.0):
            P1 = (X * numpy.exp(lam * t)) @ X.T * sq[None, :] / sq[:, None]
            P2 = (U * numpy.exp(w * t)) @ U.T * sq[None, :] / sq[:, None]
            assert numpy.abs(P1 - P2).max() < 1e-12, (trial, t)


def test_refinement_rejects_near_degenerate_spectra():
    """Eigenvalues closer than the FP32 start can separate: the acceptance rule
    sends the eigensystem to the FP64 Jacobi fallback."""
    rng = numpy.random.default_rng(3)
    n = 20
    for eps in (1e-9, 1e-5):
        N = rng.standard_normal((n, n))
        R = 1.0 + eps * (N + N.T) / 2
        A, _ = symmetric_form(R, numpy.full(n, 1.0 / n))
        _, X32 = numpy.linalg.eigh(A.astype(f32))
        assert not refine(A, X32.astype(numpy.float64), numpy.linalg.norm(A))[2], eps


def test_dot2_pair_decks():
    rng = numpy.random.default_rng(4)
    n = 20
    R = numpy.exp(rng.normal(0.0, 1.0, (n, n)))
    R = (R + R.T) / 2
    pi = numpy.maximum(rng.dirichlet(numpy.full(n, 0.5)), 1e-5)
    pi /= pi.sum()
    A, sq = symmetric_form(R, pi)
    lam, U = numpy.linalg.eigh(A)
    Up = [[split(U[i, k]) for k in range(n)] for i in range(n)]
    S2 = [split(x) for x in sq]
    Q2 = [split(1.0 / x) for x in sq]
    for t in (0.001, 0.2, 2.0):
        E2 = [pair_exp(float(lam[k] * t)) for k in range(n)]
        Ap = [[pair_mul(Up[i][k], E2[k]) for k in range(n)] for i in range(n)]
        ref = (U * numpy.exp(lam * t)) @ U.T * sq[None, :] / sq[:, None]
        for i in range(0, n, 3):
            for j in range(i, n, 2):
                ps = es = f32(0.0)
                for k in range(n):
                    ah, al = Ap[i][k]
                    uh, ul = Up[j][k]
                    h = f32(ah * uh)
                    r = fma(al, uh, fma(ah, ul, fma(ah, uh, -h)))
                    ps, q = two_sum(ps, h)
                    es = f32(es + f32(q + r))
                m = two_sum(ps, es)
                for (a, b, ratio) in ((i, j, pair_mul(S2[j], Q2[i])), (j, i, pair_mul(S2[i], Q2[j]))):
                    v = pair_mul(m, ratio)
                    assert abs(float(v[0]) + float(v[1]) - ref[a, b]) < 1e-12, (t, a, b)
