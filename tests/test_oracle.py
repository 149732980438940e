"""The oracle pinned against the reference's own outputs (CPU only).

The golden fixtures were produced by the reference p4 likelihood core
(Pf/*.c, compiled from the reference sources); the project's CPU
restatement (oracle/p4port.c) must reproduce them.
"""
import numpy
import pytest

from conftest import golden_files, golden_ids
from p4gpu import sim


@pytest.fixture(params=golden_files(), ids=golden_ids())
def golden(request):
    return sim.load_problem(request.param)


def test_port_lnl_matches_reference(golden, port):
    prob, z = golden
    lnl, parts = port.port_loglike64(prob)
    ref = float(z["ref_lnL"])
    assert abs(lnl - ref) <= 1e-12 * abs(ref)
    numpy.testing.assert_allclose(parts, z["ref_partLikes"], rtol=1e-12)


def test_port_patterns_bitexact(golden, port):
    prob, z = golden
    for p, sp in enumerate(prob.parts):
        k = "p%d_" % p
        codes = port.encode_part(sp, prob.nTax)
        pats, cnt, spi = port.make_patterns(codes)
        iv, ia = port.invar_sites(pats, sp)
        assert numpy.array_equal(pats, z[k + "ref_patterns"])
        assert numpy.array_equal(cnt, z[k + "ref_counts"])
        assert numpy.array_equal(spi, z[k + "ref_seqPosIdx"])
        assert numpy.array_equal(iv, z[k + "ref_invVec"])
        assert numpy.array_equal(ia, z[k + "ref_invArr"])


def test_port_gamma_rates_match_reference(golden, port):
    prob, z = golden
    for p, sp in enumerate(prob.parts):
        if sp.nCat == 1:
            continue
        ref = z["p%d_ref_gammaRates" % p]
        for g, a in enumerate(sp.gammaShapes):
            numpy.testing.assert_allclose(port.discrete_gamma(a, sp.nCat), ref[g], rtol=1e-14, atol=0)


def test_port_pdecks_match_reference(golden, port):
    prob, z = golden
    for p, sp in enumerate(prob.parts):
        k = "p%d_" % p
        decks = port.port_pdecks(prob, p)
        for i, v in enumerate(z[k + "ref_deckNodes"]):
            numpy.testing.assert_allclose(decks[v], z[k + "ref_decks"][i], rtol=0, atol=1e-13)


def test_port_site_likes_match_reference(golden, port):
    prob, z = golden
    for p in range(len(prob.parts)):
        _, pl, spi = port.port_part_loglike64(prob, p, patLikes=True)
        numpy.testing.assert_allclose(pl[spi], z["p%d_ref_siteLikes" % p], rtol=1e-9)


def test_discrete_gamma_properties(port):
    # equal-weight category means average to 1 (Pf/gamma.c:17-50)
    for a in (0.1, 0.3, 0.5, 1.0, 3.7, 50.0, 299.0):
        for K in (2, 3, 4, 6, 8):
            r = port.discrete_gamma(a, K)
            assert abs(r.mean() - 1.0) < 1e-6
            assert numpy.all(numpy.diff(r) > 0)


def test_pmatrix_properties(port):
    rng = numpy.random.default_rng(3)
    for dim in (4, 20):
        R = sim.random_gtr(rng, 4) if dim == 4 else sim.random_lognormal_R(rng, 20)
        pi = sim.random_comp(rng, 2.0, dim)
        Q = port.bigQ(R, pi)
        # rows sum to 0, mean rate 1, detailed balance
        assert numpy.allclose(Q.sum(1), 0, atol=1e-13)
        assert abs(-(pi * numpy.diag(Q)).sum() - 1.0) < 1e-13
        assert numpy.allclose(pi[:, None] * Q, (pi[:, None] * Q).T, atol=1e-14)
        U, lam = port.eig_sym(Q, pi)
        assert numpy.allclose(U @ U.T, numpy.eye(dim), atol=1e-13)
        assert numpy.allclose(port.pmatrix(U, lam, pi, 0.0), numpy.eye(dim), atol=1e-13)
        P = port.pmatrix(U, lam, pi, 0.37)
        assert numpy.allclose(P.sum(1), 1.0, atol=1e-13)
        assert numpy.allclose(pi @ P, pi, atol=1e-13)
        # Chapman-Kolmogorov
        assert numpy.allclose(port.pmatrix(U, lam, pi, 0.2) @ port.pmatrix(U, lam, pi, 0.17), P, atol=1e-13)


def test_jc_closed_form(port):
    # JC69 two-state probabilities, the analytic known answer
    pi = numpy.full(4, 0.25)
    R = numpy.ones((4, 4))
    U, lam = port.eig_sym(port.bigQ(R, pi), pi)
    for t in (0.01, 0.1, 1.0):
        P = port.pmatrix(U, lam, pi, t)
        same = 0.25 + 0.75 * numpy.exp(-4.0 * t / 3.0)
        diff = 0.25 - 0.25 * numpy.exp(-4.0 * t / 3.0)
        assert abs(P[0, 0] - same) < 1e-14 and abs(P[0, 1] - diff) < 1e-14


def test_live_reference_reproduces_fixture():
    """Where the reference sources exist, re-run the reference on a fixture."""
    from oracle import oracle
    import os
    if not oracle.have_ref():
        pytest.skip("the reference core is not built on this machine")
    prob, z = sim.load_problem(golden_files()[0])
    lnl, pl = oracle.RefTree(prob).logLike()
    assert lnl == float(z["ref_lnL"])


def test_fp32_mirror_matches_fp64_port(port):
    """The FP32 mirror (kernel arithmetic) on FP32-rounded P decks stays
    within the lnL tolerance of the FP64 port."""
    prob, z = sim.load_problem(golden_files()[0])
    sp = prob.parts[0]
    decks = port.port_pdecks(prob, 0)
    d32 = decks.astype(numpy.float32)
    leafNodes = numpy.nonzero(prob.tree.isLeaf)[0]
    eqsyms = sp.equateSymbols()
    partial = [e for e in eqsyms if len(sp.equates[e]) < sp.dim]
    eq = numpy.zeros((prob.tree.nNodes, max(len(partial), 1), sp.nCat, sp.dim), numpy.float32)
    for q, e in enumerate(partial):
        mem = [sp.symbols.index(c) for c in sp.equates[e]]
        eq[:, q] = decks[:, :, :, mem].sum(-1).astype(numpy.float32)
    codes = port.encode_part(sp, prob.nTax)
    pats, cnt, spi = port.make_patterns(codes)
    cc = numpy.where(pats >= 0, pats, sp.dim)
    for q, e in enumerate(partial):
        cc[pats == -64 + eqsyms.index(e)] = sp.dim + 1 + q
    masks = numpy.array([sum(1 << sp.symbols.index(c) for c in sp.equates[e]) for e in partial] or [0],
                        numpy.uint32)
    tot, like, exps, lnl = port.port_prune32(prob, 0, d32, eq if partial else eq[:, :0], cc.astype(numpy.uint8),
                                             masks, cnt.astype(float), numpy.zeros(len(cnt), numpy.uint32))
    ref = float(z["ref_lnL"])
    assert abs(tot - ref) <= 1e-6 * abs(ref)
    assert len(leafNodes) == prob.nTax
    # skipping the rescale step at cherries moves only exact powers of two
    # between like32 and E: every pattern's log likelihood is the same
    tot2, like2, exps2, lnl2 = port.port_prune32(prob, 0, d32, eq if partial else eq[:, :0],
                                                 cc.astype(numpy.uint8), masks, cnt.astype(float),
                                                 numpy.zeros(len(cnt), numpy.uint32), cherries=False)
    assert numpy.array_equal(lnl, lnl2) and tot == tot2


def test_port_site_rates_match_reference(port):
    """The port's restatement of p4_partLogLikeSiteRates (Pf/p4_tree.c:1383-1627)
    against the reference's own output stored in the fixtures."""
    n = 0
    for f in golden_files():
        prob, z = sim.load_problem(f)
        if prob.tree.isLeaf[prob.tree.root]:
            continue        # the reference routine reads an internal root's CLs only
        for p, sp in enumerate(prob.parts):
            k = "p%d_ref_siteRates" % p
            if k not in z.files:
                continue
            rates, cats = port.port_site_rates(prob, p)
            numpy.testing.assert_allclose(rates, z[k], rtol=1e-10, atol=0)
            assert numpy.array_equal(cats, z["p%d_ref_gammaCats" % p])
            n += 1
    assert n >= 8
