"""Host-side MCMC logic (no GPU): diagnostics and proposal kernels."""
import math
import types

import numpy
import pytest

from p4gpu import mcmc, sim
from p4gpu.var import var


def ess_reference_loop(vals):
    """Direct restatement of pf_effectiveSampleSize (Pf/pfmodule.c:2631-2698)."""
    n = len(vals)
    mean = sum(vals) / n
    maxLag = min(int(n / 3), 1000)
    prev = gamma = var0 = varStat = 0.0
    lag = 0
    while lag < maxLag:
        gamma = 0.0
        for j in range(n - lag):
            gamma += (vals[j] - mean) * (vals[j + lag] - mean)
        gamma /= (n - lag)
        if lag == 0:
            varStat = gamma
            var0 = gamma
        elif lag % 2 == 0:
            if prev + gamma > 0.0:
                varStat += 2.0 * (prev + gamma)
            else:
                break
        lag += 1
        prev = gamma
    return n * (var0 / varStat)


def test_ess_matches_reference_loop():
    rng = numpy.random.default_rng(0)
    for rho in (0.0, 0.5, 0.9):
        x = numpy.zeros(600)
        for i in range(1, 600):
            x[i] = rho * x[i - 1] + rng.normal()
        assert abs(mcmc.effective_sample_size(x) - ess_reference_loop(list(x))) < 1e-8


def test_ess_ar1_order_of_magnitude():
    rng = numpy.random.default_rng(1)
    rho = 0.9
    x = numpy.zeros(20000)
    for i in range(1, len(x)):
        x[i] = rho * x[i - 1] + rng.normal()
    ess = mcmc.effective_sample_size(x)
    expect = len(x) * (1 - rho) / (1 + rho)
    assert 0.7 * expect < ess < 1.3 * expect


def test_asdsf_known_answers():
    a = [frozenset([3, 12])] * 10
    assert mcmc.asdsf(a, a) == 0.0
    b = [frozenset([3])] * 5 + [frozenset([12])] * 5
    # split 3: 1.0 vs 0.5, split 12: 1.0 vs 0.5 -> sd = 0.5/sqrt(2) each
    assert abs(mcmc.asdsf(a, b) - 0.5 / math.sqrt(2)) < 1e-15


def test_dirichlet_lnpdf_matches_scipy():
    stats = pytest.importorskip("scipy.stats")
    rng = numpy.random.default_rng(2)
    for d in (4, 6, 20):
        alpha = rng.uniform(0.5, 300, size=d)
        x = rng.dirichlet(numpy.ones(d))
        assert abs(mcmc.dirichlet_lnpdf(alpha, x) - stats.dirichlet.logpdf(x, alpha)) < 1e-8 * max(
            1.0, abs(stats.dirichlet.logpdf(x, alpha)))


def _fake_mcmc(seed):
    return types.SimpleNamespace(rng=numpy.random.default_rng(seed), brLenPriorLambda=10.0,
                                 _reroot_to_child=lambda st, r: mcmc.Mcmc._reroot_to_child(None, st, r))


def _check_tree(st, nLeaves, isLeaf):
    n = len(st.parent)
    seen = set()
    stack = [st.root]
    while stack:
        v = stack.pop()
        assert v not in seen
        seen.add(v)
        for c in st.children(v):
            assert st.parent[c] == v
            stack.append(c)
    assert len(seen) == n
    assert sum(1 for v in range(n) if isLeaf[v]) == nLeaves
    for v in range(n):
        if not isLeaf[v]:
            assert len(list(st.children(v))) >= (2 if v != st.root else 2)


def test_local_keeps_a_valid_tree_and_changes_topology():
    rng = numpy.random.default_rng(3)
    t = sim.yule_tree(12, rng)
    prob = sim.Problem(t, [sim.make_part(t, rng, "dna", 50)], "x")
    st0 = mcmc.state_from_problem(prob)
    nChanged = 0
    for seed in range(300):
        fake = _fake_mcmc(seed)
        st = st0.copy()
        ch = types.SimpleNamespace(changed=set())
        fake._topoChanged = False
        ok = mcmc.Mcmc._proposeLocal(fake, st, 2.0 * math.log(1.1), ch)
        if not ok:
            continue
        _check_tree(st, 12, t.isLeaf)
        # three branches rescaled by one ratio: log proposal ratio = 3 log ratio
        assert abs(st.tree_length() - st0.tree_length()) < 1.0
        s0 = mcmc.splits_of(st0, t.isLeaf, t.seqNum, 12)
        s1 = mcmc.splits_of(st, t.isLeaf, t.seqNum, 12)
        if s0 != s1:
            nChanged += 1
            assert len(s0 ^ s1) == 2            # an NNI changes exactly one split
    assert nChanged > 10


def test_splits_of_known_tree():
    kids = {"r": ["A", "B", "x"], "x": ["C", "y"], "y": ["D", "E"]}
    t = sim.tree_from_children(kids, "r")
    st = mcmc.State(t.parent.copy(), t.leftChild.copy(), t.sibling.copy(), t.root, t.brLen.copy(), [])
    sp = mcmc.splits_of(st, t.isLeaf, t.seqNum, 5)
    # taxa in pre-order: A0 B1 C2 D3 E4; internal splits {C,D,E} and {D,E}
    assert sp == frozenset([0b11100, 0b11000])
