"""p4's Mcmc surface on the host: Mcmc(aTree, nChains, runNum,
sampleInterval, checkPointInterval) over a Tree with data and model, its
sample files in p4's formats, and checkpoint / restart (func.unPickleMcmc).

The likelihood is the reference's own C core (oracle.RefChainEvaluator), so
no GPU is needed.  A run of 300 generations that checkpoints, restarts from
its last checkpoint and runs 200 more must write the same files, byte for
byte, as one uninterrupted run of 500 (the random-number state, tunings and
chain states all travel in the checkpoint), and the restart's recomputed
lnL must agree with the checkpointed one within p4's 0.01.
"""
import os
import re

import numpy
import pytest

from p4gpu import func, mcmc, sim
from p4gpu.p4exceptions import P4Error
from p4gpu.tree import Tree

oracle = pytest.importorskip("oracle.oracle")


@pytest.fixture(scope="module")
def problem():
    if not oracle.have_ref():
        pytest.skip("the reference core is not built on this machine")
    return sim.make_config("dna16")


def new_mcmc(prob, **kw):
    t = Tree.fromProblem(prob, taxNames=["taxon_%02d" % i for i in range(prob.nTax)])
    return t, mcmc.Mcmc(t, nChains=2, runNum=0, sampleInterval=10, checkPointInterval=100, seed=3,
                        evaluator=oracle.RefChainEvaluator, **kw)


def parse_newick_splits(s, nTax):
    """Non-trivial splits (bitmasks over taxon numbers 1..nTax, normalised so
    that taxon 1 is outside) of a translated Newick string."""
    s = re.sub(r"\[[^\]]*\]", "", s).strip().rstrip(";")
    stack, out = [[]], set()
    full = (1 << nTax) - 1
    tok = re.findall(r"\(|\)|,|[^(),:]+|:[^(),]+", s)
    for t in tok:
        if t == "(":
            stack.append([])
        elif t == ")":
            kids = stack.pop()
            m = 0
            for k in kids:
                m |= k
            stack[-1].append(m)
            if 1 < bin(m).count("1") < nTax - 1:
                out.add(m if not (m & 1) else full ^ m)
        elif t == "," or t.startswith(":"):
            continue
        else:
            t = t.strip()
            if t:
                stack[-1].append(1 << (int(t) - 1))
    return out


def test_files_checkpoint_restart(problem, tmp_path, monkeypatch):
    prob = problem
    straight = tmp_path / "straight"
    split = tmp_path / "split"
    straight.mkdir()
    split.mkdir()

    monkeypatch.chdir(straight)
    _, m = new_mcmc(prob)
    m.run(500)

    monkeypatch.chdir(split)
    t, m1 = new_mcmc(prob)
    m1.run(300)
    likes = open("mcmc_likes_0").read().split("\n")[:-1]
    assert len(likes) == 30 and [int(x.split()[0]) for x in likes] == list(range(10, 301, 10))
    numpy.testing.assert_allclose([float(x.split()[1]) for x in likes], m1.samples["lnL"], atol=1e-6)
    trees = open("mcmc_trees_0.nex").read()
    assert trees.startswith("#nexus\n\nbegin taxa;\n  dimensions ntax=16;\n  taxlabels taxon_00")
    assert "  translate\n      1 taxon_00,\n" in trees and "     16 taxon_15\n  ;\n" in trees
    assert trees.endswith("  tree t_300 = [&U] " + trees.split("  tree t_300 = [&U] ")[1])
    assert trees.endswith(";\nend;\n\n")
    lines = [ln for ln in trees.split("\n") if ln.startswith("  tree t_")]
    assert len(lines) == 30
    last = parse_newick_splits(lines[-1].split("= [&U] ")[1], 16)
    # the file's translation number k is the sampler's taxon k - 1
    assert {int(x) for x in m1.samples["splits"][-1]} == last
    prams = open("mcmc_prams_0").read().split("\n")
    head = [ln for ln in prams if ln.startswith("genPlus1")]
    assert head and head[0].split("\t")[:2] == ["genPlus1", "comp.0.0.0"]
    rows = [ln for ln in prams if ln and not ln.startswith("#") and not ln.startswith("genPlus1")]
    assert len(rows) == 30 and len(rows[0].split("\t")) == len(head[0].split("\t"))
    assert sorted(f for f in os.listdir(".") if f.startswith("mcmc_checkPoint_0.")) == \
        ["mcmc_checkPoint_0.100", "mcmc_checkPoint_0.200", "mcmc_checkPoint_0.300"]
    assert os.path.exists("mcmc_pramsProfile_0.py")

    # a new run may not overwrite the checkpoints
    with pytest.raises(P4Error):
        new_mcmc(prob)
    # restart from the latest checkpoint, data re-attached
    m2 = func.unPickleMcmc(0, t.data, evaluator=oracle.RefChainEvaluator, verbose=False)
    assert m2.gen == 299
    assert [ch.curLogLike for ch in m2.chains] == [ch.curLogLike for ch in m1.chains]
    m2.run(200)
    for name in ("mcmc_likes_0", "mcmc_trees_0.nex", "mcmc_prams_0"):
        assert open(name).read() == open(os.path.join(straight, name)).read(), name
    assert open("mcmc_trees_0.nex").read().count("end;") == 2       # taxa block + trees block


def test_restart_checks_the_likelihood(problem, tmp_path, monkeypatch):
    """A checkpoint whose recomputed lnL is off by more than 0.01 (the data
    re-attached are not the data the run used) is refused."""
    monkeypatch.chdir(tmp_path)
    t, m = new_mcmc(problem)
    m.run(100)
    other = sim.make_config("dna16", seed=77)      # another alignment of 16 taxa
    bad = Tree.fromProblem(other).data
    with pytest.raises(P4Error):
        func.unPickleMcmc(0, bad, evaluator=oracle.RefChainEvaluator, verbose=False)


def test_incremental_reference_evaluator_matches_full(tmp_path, monkeypatch):
    """The reference-likelihood chain's part-level updates (only the parts a
    proposal changed are recomputed) give the lnL a full evaluation gives."""
    if not oracle.have_ref():
        pytest.skip("the reference core is not built on this machine")
    from conftest import golden_files
    prob, _ = sim.load_problem([f for f in golden_files() if f.endswith("dna_2part_relrate.npz")][0])
    monkeypatch.chdir(tmp_path)
    ev = oracle.RefChainEvaluator(prob)
    m = mcmc.Mcmc(prob, nChains=2, seed=5, sampleInterval=0, evaluator=ev, freeRelRates=True)
    m.run(300)
    assert ev.nPartUpdates > 20
    for ch in m.chains:
        full = oracle.RefTree(prob)
        full.setState(ch.cur)
        lnl, _ = full.logLike()
        assert abs(lnl - ch.curLogLike) <= 1e-9 * abs(lnl), (lnl, ch.curLogLike)
