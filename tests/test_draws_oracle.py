"""Ancestral-state draws and simulation: the oracle pinned to the reference
(CPU only).

The golden fixtures hold, per case, the reference's own draws
(p4_drawAncStateP, Pf/p4_treeSim.c:847) with the libc uniforms it used, and
the reference's own simulation (p4_simulate, Pf/p4_treeSim.c:14) fed the
Philox4x32-10 stream of seed 5 through the stubbed gsl_rng_uniform.  The
oracle restates both by sites in parallel (every decision takes the stream
value the sequential loop would draw), as the GPU kernels do.
"""
import numpy
import pytest

from conftest import golden_files, golden_ids
from p4gpu import sim

SIM_SEED = 5


@pytest.fixture(params=golden_files(), ids=golden_ids())
def golden(request):
    return sim.load_problem(request.param)


def test_philox_known_answers(port):
    """Philox4x32-10 known-answer vectors (Random123 kat_vectors)."""
    _, c = port.philox_uniform(0, 0)
    assert c == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    # the general form of the vectors: counter and key words all set
    M = 0xffffffff

    def block(ctr, key):
        cc = list(ctr)
        k = list(key)
        for _ in range(10):
            p0, p1 = 0xD2511F53 * cc[0], 0xCD9E8D57 * cc[2]
            cc = [(p1 >> 32) ^ cc[1] ^ k[0], p1 & M, (p0 >> 32) ^ cc[3] ^ k[1], p0 & M]
            k = [(k[0] + 0x9E3779B9) & M, (k[1] + 0xBB67AE85) & M]
        return cc
    assert block([M] * 4, [M] * 2) == [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert block([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]) == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]
    # the vectorised stream agrees with the scalar one
    u = port.philox_uniforms(1234567, 10 ** 6, 50)
    assert all(u[i] == port.philox_uniform(1234567, 10 ** 6 + i)[0] for i in range(50))


def test_preorder_is_p4s(golden, port):
    prob, z = golden
    assert port.preorder(prob.tree) == [int(v) for v in prob.tree.preOrder if v >= 0]


def test_port_simulation_matches_reference(golden, port):
    """The parallel restatement reproduces the reference's sequential
    simulation from the same stream (port P decks, which agree with the
    reference's to 1e-12: a decision can differ only where a uniform falls
    within that distance of a picker boundary)."""
    prob, z = golden
    decks = [port.port_pdecks(prob, p) for p in range(len(prob.parts))]
    states = port.port_simulate(prob, SIM_SEED, decks)
    leaves = [v for v in range(prob.tree.nNodes) if prob.tree.isLeaf[v]]
    for p, sp in enumerate(prob.parts):
        ref = z["p%d_ref_simSeqs" % p].astype(int)
        got = numpy.zeros_like(ref)
        for v in leaves:
            got[prob.tree.seqNum[v]] = states[p][v]
        bad = numpy.nonzero((got != ref).any(axis=0))[0]
        assert len(bad) <= 1, (p, bad[:10])


def test_port_draws_match_reference(golden, port):
    """p4_drawAncState restated on the port's FP64 root CLs, with the
    reference's own uniforms: the same draws."""
    prob, z = golden
    if "p0_ref_ancDraws" not in z.files:
        pytest.skip("leaf root: the reference draws need an internal root")
    for p in range(len(prob.parts)):
        cl = port.port_root_cl(prob, p)
        d = port.port_draw_anc(prob, p, cl, z["p%d_ref_ancUniforms" % p])
        ref = z["p%d_ref_ancDraws" % p].astype(numpy.int32)
        assert (d != ref).any(axis=1).sum() <= 1, p


def test_live_reference_newton_reproduces_fixture():
    """Where the reference sources exist, re-run its Newton optimisation."""
    from oracle import oracle
    import os
    if not oracle.have_ref():
        pytest.skip("the reference core is not built on this machine")
    prob, z = sim.load_problem(golden_files()[0])
    r = oracle.RefTree(prob)
    r.logLike()
    lnl, bl = r.newtOptimize()
    assert lnl == float(z["ref_newtLnL"])
    assert numpy.array_equal(bl, z["ref_newtBrLens"])
