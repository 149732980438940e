"""MCMC over the GPU likelihood (p4's Mcmc/Chain semantics)."""
import numpy
import pytest

from conftest import golden_files
from p4gpu import mcmc, sim

pytestmark = pytest.mark.gpu


def problem_of_state(prob, st):
    """The Problem a chain state describes, for an independent FP64 check."""
    t = sim.TreeSpec(st.parent, st.leftChild, st.sibling, prob.tree.isLeaf, prob.tree.seqNum,
                     st.brLen, st.root)
    parts = []
    for sp, ps in zip(prob.parts, st.parts):
        R = numpy.stack([sim.sym_from_upper(r, sp.dim) for r in ps.rvals])
        parts.append(sim.PartSpec(sp.dataType, sp.sequences, ps.comps, R, ps.gamma, sp.nCat,
                                  sp.compNums, sp.rMatrixNums, sp.gdasrvNums, pInvar=ps.pInvar,
                                  relRate=ps.relRate, equates=sp.equates))
    return sim.Problem(t, parts, "state")


def test_single_chain_cur_lnl_is_consistent(lib, port):
    prob, _ = sim.load_problem(golden_files()[0])      # dna16: 16 taxa, 1000 sites
    m = mcmc.Mcmc(prob, nChains=1, seed=4, sampleInterval=10)
    m.run(1500)
    ch = m.coldChain()
    ref, _ = port.port_loglike64(problem_of_state(prob, ch.cur))
    assert abs(ch.curLogLike - ref) <= 1e-6 * abs(ref)
    acc = m.acceptance()
    assert 0.01 < acc["local"] < 0.99
    # p4's default allBrLens window is wide for 1000 sites: the tuner shrinks it
    allBr = next(p for p in m.proposals if p.name == "allBrLens")
    assert allBr.tuning[0] < 2.0 * numpy.log(1.02)
    assert sum(p.nTopologyChanges[0] for p in m.proposals if p.name == "local") > 0
    assert len(m.samples["lnL"]) == 150


def test_mcmcmc_swaps_and_heated_chains(lib, port):
    prob, _ = sim.load_problem(golden_files()[0])
    m = mcmc.Mcmc(prob, nChains=4, chainTemp=0.1, seed=5, sampleInterval=20)
    m.run(300)
    assert sum(m.swapAttempts) == 300 and sum(m.swapAccepts) > 0
    assert sorted(ch.tempNum for ch in m.chains) == [0, 1, 2, 3]
    for ch in m.chains:
        ref, _ = port.port_loglike64(problem_of_state(prob, ch.cur))
        assert abs(ch.curLogLike - ref) <= 1e-6 * abs(ref)


def test_heterogeneous_multipart_mcmc(lib, port):
    prob = sim.make_config("mcmcmc32", scale=0.02)
    m = mcmc.Mcmc(prob, nChains=2, seed=6, sampleInterval=0)
    m.run(120)
    for ch in m.chains:
        ref, _ = port.port_loglike64(problem_of_state(prob, ch.cur))
        assert abs(ch.curLogLike - ref) <= 1e-6 * abs(ref)


def test_batch_graph_matches_single_evaluations(lib, port):
    """All chains through the captured CUDA graph == one tree at a time, also
    after topology and model changes that re-capture the graph."""
    from p4gpu import pf
    from p4gpu.engine import Engine, make_data
    prob = sim.make_config("mcmcmc32", scale=0.02)
    shared = make_data(prob)
    engines = [Engine(prob, shared=shared) for _ in range(4)]
    rng = numpy.random.default_rng(0)
    for k, e in enumerate(engines):
        e.setBrLensFast(prob.tree.brLen * numpy.exp(rng.normal(0, 0.2, prob.tree.nNodes)))
    b = pf.Batch([e.cTree for e in engines], graph=True)
    for rnd in range(3):
        got = b.logLike()
        want = [e.calcLogLike() for e in engines]
        numpy.testing.assert_allclose(got, want, rtol=1e-12)
        # change one tree's topology (NNI) and another's gamma shape
        t = prob.tree
        v = next(x for x in range(t.nNodes) if not t.isLeaf[x] and x != t.root and t.parent[x] != t.root)
        u = int(t.parent[v])
        sib = next(c for c in t.children(u) if c != v)
        t2 = t.swapped(sib, next(iter(t.children(v))))
        engines[rnd % 4].setTopologyArrays(t2.parent, t2.leftChild, t2.sibling, t2.root)
        engines[(rnd + 1) % 4].setGamma(0, 0, 0.3 + 0.2 * rnd)
    b.free()
