"""Ancestral-state draws and simulation on the GPU against the reference's
own outputs (golden fixtures) and the oracle.

Tolerances: the draws compare FP32 root partials (the GPU) with the
reference's FP64 CLs, so a site's draw may differ only where its uniform
falls within ~1e-6 (relative) of a picker boundary: at most 2 sites per
part.  The simulation compares the GPU's FP64 P decks with the
reference's (agreement ~1e-15): at most 1 differing site per part.  With
uniforms given by value or drawn from the Philox stream on the GPU the
draws must be identical.
"""
import numpy
import pytest

from conftest import golden_files, golden_ids
from p4gpu import pf, sim
from p4gpu.engine import Engine

pytestmark = pytest.mark.gpu

SIM_SEED = 5


@pytest.fixture(params=golden_files(), ids=golden_ids())
def golden(request, lib):
    return sim.load_problem(request.param)


def test_draws_match_reference(golden):
    prob, z = golden
    if "p0_ref_ancDraws" not in z.files:
        pytest.skip("leaf root: the reference draws need an internal root")
    e = Engine(prob)
    for p, sp in enumerate(prob.parts):
        d = pf.drawAncStates(e.cTree, p, sp.nChar, z["p%d_ref_ancUniforms" % p])
        ref = z["p%d_ref_ancDraws" % p].astype(numpy.int32)
        assert (d != ref).any(axis=1).sum() <= 2, p
        # a draw is either a variable-site (state, category) or an invariant state
        ok = ((d[:, 1] >= 0) & (d[:, 0] >= 0) & (d[:, 2] == 0)) | ((d[:, 2] == 1) & (d[:, 3] >= 0))
        assert ok.all()
    e.free()


def test_philox_draws_are_the_stream(golden, port):
    """Uniforms drawn on the GPU (Philox, seed 77) give the draws of the same
    values passed by value: the device generator is the oracle's, bit for
    bit, and sites of later parts continue the stream."""
    prob, z = golden
    if prob.tree.isLeaf[prob.tree.root]:
        pytest.skip("leaf root")
    e = Engine(prob)
    off = 0
    for p, sp in enumerate(prob.parts):
        u = port.philox_uniforms(77, off, sp.nChar)
        a = pf.drawAncStates(e.cTree, p, sp.nChar, None, 77)
        b = pf.drawAncStates(e.cTree, p, sp.nChar, u)
        assert numpy.array_equal(a, b), p
        off += sp.nChar
    s = e.ancestralStateDraw(seed=77)
    assert len(s) == sum(sp.nChar for sp in prob.parts)
    e.free()


def test_simulation_matches_reference(golden):
    prob, z = golden
    e = Engine(prob)
    nStates = sum(prob.tree.nNodes * sp.nChar for sp in prob.parts)
    states = pf.simulate(e.cTree, SIM_SEED, None, nStates)
    o = 0
    for p, sp in enumerate(prob.parts):
        st = states[o:o + prob.tree.nNodes * sp.nChar].reshape(prob.tree.nNodes, sp.nChar)
        o += prob.tree.nNodes * sp.nChar
        ref = z["p%d_ref_simSeqs" % p].astype(int)
        got = numpy.zeros_like(ref)
        for v in range(prob.tree.nNodes):
            if prob.tree.isLeaf[v]:
                got[prob.tree.seqNum[v]] = st[v]
        assert (got != ref).any(axis=0).sum() <= 1, p
    e.free()


def test_simulated_alignment_evaluates(port):
    """simulate -> makePatterns -> lnL on the same tree: the GPU's FP32 lnL
    of the new alignment agrees with the FP64 oracle on the same sequences."""
    prob, z = sim.load_problem(golden_files()[0])
    e = Engine(prob)
    before = e.calcLogLike()
    seqs = e.simulate(seed=3)
    after = e.calcLogLike()
    parts = []
    for p, sp in enumerate(prob.parts):
        q = sim.PartSpec(sp.dataType, list(seqs[p]), sp.comps, sp.rmats, sp.gammaShapes, sp.nCat,
                         sp.compNums, sp.rMatrixNums, sp.gdasrvNums, sp.pInvar, sp.relRate)
        parts.append(q)
    ref, _ = port.port_loglike64(sim.Problem(prob.tree, parts, "simulated"))
    assert after != before
    assert abs(after - ref) <= 1e-6 * abs(ref), (after, ref)
    e.free()


@pytest.mark.parametrize("name", ["dna_ambig_pinv", "dna_2part_relrate", "prot48het_small"])
def test_simulation_with_reference_tree(port, name):
    """Tree.simulate(refTree=...) (Pf/p4_treeSim.c:223-284): every site's root
    state and category (or invariant state) drawn from the reference tree's
    root posterior given its data, then mutated down the tree.  The
    reference core's own run, given the same random numbers (the libc draws
    of its root loop passed by value, its GSL stream as the Philox stream of
    the same seed), gives the same leaf alignment except at sites whose root
    draw falls within FP32 rounding of a picker boundary, or whose mutation
    uniform does within FP64 rounding: at most 2 differing sites per part."""
    import os
    from conftest import REPO
    if not port.have_ref():
        pytest.skip("reference core not built")
    path = os.path.join(REPO, "tests", "golden", name + ".npz")
    probR, _ = sim.load_problem(path)
    probS, _ = sim.load_problem(path)
    rR, rS = port.RefTree(probR), port.RefTree(probS)
    rR.logLike()
    rS.logLike()
    refSeqs, libcU, nGsl = rS.simulateRef(rR, 11, SIM_SEED)
    assert nGsl > 0
    eR, eS = Engine(probR), Engine(probS)
    eR.calcLogLike()
    nStates = sum(probS.tree.nNodes * sp.nChar for sp in probS.parts)
    states = pf.simulateRef(eS.cTree, eR.cTree, SIM_SEED, None, 0, libcU, nStates)
    o = 0
    for p, sp in enumerate(probS.parts):
        st = states[o:o + probS.tree.nNodes * sp.nChar].reshape(probS.tree.nNodes, sp.nChar)
        o += probS.tree.nNodes * sp.nChar
        got = numpy.zeros_like(refSeqs[p])
        for v in range(probS.tree.nNodes):
            if probS.tree.isLeaf[v]:
                got[probS.tree.seqNum[v]] = st[v]
        assert (got != refSeqs[p]).any(axis=0).sum() <= 2, (name, p)
    # the reference tree's own data is untouched; the simulated tree evaluates
    before = eR.calcLogLike()
    assert before == eR.calcLogLike()
    eS.free()
    eR.free()
