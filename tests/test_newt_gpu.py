"""Newton branch-length optimisation on the GPU against the reference's own
p4_newtAround (Pf/p4_treeNewt.c, compiled into the oracle; results in the
golden fixtures).

Both run the same algorithm in FP64 from the same start; their CLs differ
by rounding only, so the optimised lnL agrees to 1e-9 relative (measured in
FP64 on both sides) and the branch lengths to the convergence tolerance
(|d lnL/dt| < 1e-5 at the end: 1e-4 relative or 1e-6 absolute).
"""
import numpy
import pytest

from conftest import golden_files, golden_ids
from p4gpu import pf, sim
from p4gpu.engine import Engine

pytestmark = pytest.mark.gpu


@pytest.fixture(params=golden_files(), ids=golden_ids())
def golden(request, lib):
    return sim.load_problem(request.param)


def test_newton_matches_reference(golden):
    prob, z = golden
    if "ref_newtLnL" not in z.files:
        pytest.skip("leaf root: the reference's cl2 needs an internal root")
    e = Engine(prob)
    start = e.calcLogLike()
    pf.p4_newtSetup(e.cTree)
    pf.p4_newtAndBrentPowellOpt(e.cTree)
    pf.setPrecision(e.cTree, 1)
    lnl = e.calcLogLike()
    bl = pf.p4_getBrLens(e.cTree, prob.tree.nNodes)
    ref = float(z["ref_newtLnL"])
    assert lnl > start
    assert abs(lnl - ref) <= 1e-9 * abs(ref), (lnl, ref)
    rb = z["ref_newtBrLens"]
    nonroot = [v for v in range(prob.tree.nNodes) if v != prob.tree.root]
    numpy.testing.assert_allclose(bl[nonroot], rb[nonroot], rtol=1e-4, atol=1e-6)
    e.free()


def test_opt_loglike_updates_the_tree(port):
    """Engine.optLogLike: the FP32 lnL at the optimum agrees with the FP64
    oracle at the returned branch lengths."""
    prob, z = sim.load_problem(golden_files()[0])
    e = Engine(prob)
    lnl = e.optLogLike()
    ref, _ = port.port_loglike64(prob, brLen=prob.tree.brLen)
    assert abs(lnl - ref) <= 1e-6 * abs(ref)
    assert abs(lnl - float(z["ref_newtLnL"])) <= 1e-6 * abs(lnl)
    e.free()
