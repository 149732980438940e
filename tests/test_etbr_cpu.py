"""eTBR (p4's Chain.proposeETBR_Blaise, p4/chain.py:4128) and the tree
primitives it uses, on the host (no GPU).

  - structure: every move leaves a valid tree on the same leaves with the same
    root and node degrees, changes at most three branch lengths (the central
    branch and one branch at each unconstrained end), and reports a topology
    change exactly when the tree's splits change;
  - reRoot keeps every branch with its length (p4/tree.py:3527);
  - the Hastings ratio: a chain that sees no data (lnL = 0) must sample the
    prior -- every one of the 15 unrooted topologies of 5 taxa with
    probability 1/15, and exponential(10) branch lengths (tree length 0.7).
    Each topology's frequency is held to 1/15 within 4.5 of its Monte Carlo
    standard errors (from the indicator series' ESS), the tree length within 4.
"""
import collections
import math

import numpy
import pytest

from p4gpu import mcmc, sim
from p4gpu.topology import LinkedTree, propose_etbr


def splits(t, isLeaf, seqNum, nTax):
    st = mcmc.State(numpy.array(t.parent), numpy.array(t.leftChild), numpy.array(t.sibling), t.root,
                    numpy.array(t.brLens()), [])
    return mcmc.splits_of(st, isLeaf, seqNum, nTax)


def check_valid(t, tree):
    n = len(t.parent)
    assert t.root == tree.root and t.parent[t.root] == -1
    seen = set()
    stack = [t.root]
    while stack:
        v = stack.pop()
        assert v not in seen
        seen.add(v)
        for c in t.children(v):
            assert t.parent[c] == v
            stack.append(c)
    assert seen == set(range(n))
    for v in range(n):
        assert bool(tree.isLeaf[v]) == (t.leftChild[v] < 0 or v == t.root and tree.isLeaf[v])


def test_etbr_structure():
    rng = numpy.random.default_rng(11)
    tree = sim.yule_tree(20, rng)
    lam = 2.0 * math.log(1.6)
    t = LinkedTree(tree.parent, tree.leftChild, tree.sibling, tree.root, tree.brLen, tree.isLeaf)
    degrees = [t.getDegree(v) for v in range(tree.nNodes)]
    nChanged = 0
    for _ in range(400):
        before = splits(t, tree.isLeaf, tree.seqNum, tree.nLeaves)
        bl0 = list(t.length)
        lnPrior, lnProp, changed = propose_etbr(t, rng, lam, 0.8, 10.0)
        check_valid(t, tree)
        assert [t.getDegree(v) for v in range(tree.nNodes)] == degrees
        after = splits(t, tree.isLeaf, tree.seqNum, tree.nLeaves)
        assert changed == (before != after)
        nChanged += changed
        # at most three branches change length (by id), each by a factor in
        # [1/1.6, 1.6]; the other branches keep theirs wherever they moved
        diff = [(a, b) for a, b in zip(bl0, t.length) if a != b]
        assert 1 <= len(diff) <= 3
        assert all(1 / 1.6 - 1e-12 <= b / a <= 1.6 + 1e-12 for a, b in diff)
        assert math.isfinite(lnPrior) and math.isfinite(lnProp)
    assert 100 < nChanged < 400


def test_reroot_keeps_branches():
    rng = numpy.random.default_rng(2)
    tree = sim.yule_tree(12, rng)
    t = LinkedTree(tree.parent, tree.leftChild, tree.sibling, tree.root, tree.brLen, tree.isLeaf)
    s0 = splits(t, tree.isLeaf, tree.seqNum, tree.nLeaves)
    tl0 = sum(t.brLens())
    for target in range(tree.nNodes):
        if tree.isLeaf[target] or t.nChildren(target) < 2:
            continue
        t.reRoot(target)
        assert t.root == target
        assert splits(t, tree.isLeaf, tree.seqNum, tree.nLeaves) == s0
        assert abs(sum(t.brLens()) - tl0) < 1e-12
    t.reRoot(tree.root)
    assert sorted(t.length) == sorted(tree.brLen)


def prior_chain(probs, nGen, seed):
    rng = numpy.random.default_rng(3)
    t = sim.yule_tree(5, rng)
    prob = sim.Problem(t, [sim.make_part(t, rng, "dna", 20, nComps=1, gammaShape=0.5)], "p5")
    pp = mcmc.McmcProposalProbs(allCompsDir=0, allRMatricesDir=0, gdasrv=0, pInvar=0, relRate=0, **probs)
    m = mcmc.Mcmc(prob, nChains=1, seed=seed, sampleInterval=1, prob=pp, evaluator=mcmc.PriorEvaluator())
    m.run(nGen)
    return m


@pytest.mark.parametrize("probs", [dict(eTBR=1.0, allBrLens=1.0, local=0.0),
                                   dict(eTBR=1.0, allBrLens=0.0, local=0.0)],
                         ids=["etbr+allBrLens", "etbr-only"])
def test_etbr_samples_the_prior(probs):
    m = prior_chain(probs, 40000, 7)
    sp = m.samples["splits"][2000:]
    topo = collections.Counter(sp)
    assert len(topo) == 15
    n = len(sp)
    for key in topo:
        ind = numpy.array([1.0 if s == key else 0.0 for s in sp])
        p = ind.mean()
        ess = mcmc.effective_sample_size(ind)
        se = math.sqrt((1.0 / 15) * (14.0 / 15) / ess)
        assert abs(p - 1.0 / 15) < 4.5 * se, (p, ess, se)
    tl = numpy.array(m.samples["treeLength"][2000:])
    ess = mcmc.effective_sample_size(tl)
    assert abs(tl.mean() - 0.7) < 4.0 * tl.std() / math.sqrt(ess), (tl.mean(), ess)
    assert n > 30000
    acc = m.acceptance()
    assert 0.2 < acc["eTBR"] < 1.0


def test_default_mixture_has_etbr():
    rng = numpy.random.default_rng(4)
    t = sim.yule_tree(8, rng)
    prob = sim.Problem(t, [sim.make_part(t, rng, "dna", 20, nComps=1, gammaShape=0.5)], "p8")
    m = mcmc.Mcmc(prob, nChains=1, seed=1, evaluator=mcmc.PriorEvaluator())
    w = {p.name: p.weight for p in m.proposals}
    assert w["eTBR"] == w["local"] == t.nNodes - 1          # p4/mcmc.py:1380-1386
    assert "eTBR" not in mcmc.TUNABLE
