"""Maximum likelihood over branch lengths and free model parameters
(p4g_newtAndBrentPowellOpt, pf.p4_newtAndBrentPowellOpt) against the
reference's own optimiser on the same problems (tests/golden/opt/*.npz,
written by tests/golden/make_opt_golden.py, which runs the reference's
p4_newtAndBrentPowellOpt).

Both searches stop when a pass changes lnL by less than 1e-6, from
different algorithms (praxis there, Powell with Brent line searches here),
so they meet at the same maximum only to within their convergence: the
optimum lnL (FP64) must agree within 2e-3 and must not be worse than the
reference's by more than that; the free values must agree to the precision
that flat a maximum pins them (compositions 5e-3, gamma shapes 5 %, pInvar
0.02, branch-length sums 2 %).  p4_getFreePrams returns the free values in
the reference's wind-up order.
"""
import glob
import os

import numpy
import pytest

from conftest import GOLDEN
from p4gpu import pf, sim
from p4gpu.engine import Engine

pytestmark = pytest.mark.gpu

FIXTURES = sorted(glob.glob(os.path.join(GOLDEN, "opt", "*.npz")))


@pytest.fixture(params=FIXTURES, ids=[os.path.basename(f)[:-4] for f in FIXTURES])
def case(request, lib):
    return sim.load_problem(request.param)


def test_optimum_matches_reference(case):
    prob, z = case
    free = tuple(int(z[k]) for k in ("free_comps", "free_rmats", "free_gdasrvs", "free_pInvar"))
    e = Engine(prob, free=free)
    pf.setPrecision(e.cTree, 1)
    start = e.calcLogLike()
    assert abs(start - float(z["ref_start_lnL"])) <= 1e-9 * abs(start)
    e.optLogLike()
    lnl = e.calcLogLike()
    ref = float(z["ref_opt_lnL"])
    assert abs(lnl - ref) <= 2e-3, (lnl, ref)
    for p, sp in enumerate(prob.parts):
        if free[0]:
            numpy.testing.assert_allclose(numpy.array(e.compVals[p]), z["p%d_ref_opt_comps" % p], atol=5e-3)
        if free[2]:
            g = numpy.array([v[0] for v in e.gVals[p]])
            numpy.testing.assert_allclose(g, z["p%d_ref_opt_gamma" % p], rtol=0.05)
    bl = pf.p4_getBrLens(e.cTree, prob.tree.nNodes)
    mask = numpy.arange(prob.tree.nNodes) != prob.tree.root
    rb = z["ref_opt_brLens"]
    assert abs(bl[mask].sum() - rb[mask].sum()) <= 0.02 * rb[mask].sum()
    prams = pf.p4_getFreePrams(e.cTree)
    nExpect = sum(free[0] * sp.comps.shape[0] * (sp.dim - 1) + free[1] * sp.rmats.shape[0] * (sp.dim * (sp.dim - 1) // 2 - 1)
                  + free[2] * len(sp.gammaShapes) + free[3] for sp in prob.parts)
    assert len(prams) == nExpect
    if free[3]:
        assert abs(prams[-1] - float(z["p0_ref_opt_pInvar"])) <= 0.02
    e.free()
