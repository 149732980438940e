"""GPU parity: libp4gpu (through its C ABI) against the reference's outputs
(golden fixtures) and the CPU oracle.

Tolerances:
  - lnL: |dlnL| <= 1e-6 |lnL| (the FP32-pruning target), FP64 setPrams
    outputs (gamma rates, P decks) <= 1e-12;
  - the FP32 kernel arithmetic is checked bit-exactly: given the GPU's own
    FP32 P decks, the oracle's FP32 mirror must reproduce every pattern's
    scaled root likelihood and integer scaler exponent exactly.
"""
import numpy
import pytest

from conftest import golden_files, golden_ids
from p4gpu import P4Error, pf, sim
from p4gpu.engine import Engine

pytestmark = pytest.mark.gpu

LNL_RTOL = 1e-6
TENSOR_SHAPE = 3      # protein tile shape served by the tcgen05 kernel


@pytest.fixture(params=golden_files(), ids=golden_ids())
def golden(request, lib):
    return sim.load_problem(request.param)


def test_lnl_matches_reference(golden):
    prob, z = golden
    e = Engine(prob)
    lnl = e.calcLogLike()
    ref = float(z["ref_lnL"])
    assert abs(lnl - ref) <= LNL_RTOL * abs(ref), (lnl, ref)
    numpy.testing.assert_allclose(e.partLikes, z["ref_partLikes"], rtol=LNL_RTOL)
    e.free()


def test_plain_fp64_path_matches_reference(golden):
    """Precision mode 1 (the per-node FP64 restatement) agrees with the
    reference FP64 core to rounding."""
    prob, z = golden
    e = Engine(prob)
    pf.setPrecision(e.cTree, 1)
    lnl = e.calcLogLike()
    ref = float(z["ref_lnL"])
    assert abs(lnl - ref) <= 1e-11 * abs(ref), (lnl, ref)
    numpy.testing.assert_allclose(e.partLikes, z["ref_partLikes"], rtol=1e-11)
    pf.setPrecision(e.cTree, 0)
    assert abs(e.calcLogLike() - ref) <= LNL_RTOL * abs(ref)
    e.free()


def test_gpu_gamma_rates_match_reference(golden):
    prob, z = golden
    e = Engine(prob)
    e.setPrams()
    for p, sp in enumerate(prob.parts):
        for g in range(len(sp.gammaShapes)):
            r = pf.getGammaRates(e.cTree, p, g, sp.nCat)
            numpy.testing.assert_allclose(r, z["p%d_ref_gammaRates" % p][g], rtol=1e-12)
    e.free()


def test_gpu_pdecks_match_reference(golden):
    prob, z = golden
    e = Engine(prob)
    e.setPrams()
    for p, sp in enumerate(prob.parts):
        k = "p%d_" % p
        for i, v in enumerate(z[k + "ref_deckNodes"]):
            for c in range(sp.nCat):
                d = pf.getPDeck(e.cNodes[v], p, c, sp.dim)
                numpy.testing.assert_allclose(d, z[k + "ref_decks"][i][c], rtol=0, atol=1e-12)
    e.free()


def groups_of(prob):
    """The library's pruning groups: distinct (dim, nCat) in part order."""
    out = []
    for sp in prob.parts:
        if (sp.dim, sp.nCat) not in out:
            out.append((sp.dim, sp.nCat))
    return out


def force_cuda_core_shapes(e, prob):
    """Pin 20-state groups to the FP32 CUDA-core kernel (the autotuner may
    pick the split-TF32 tensor-core kernel, which the FP32 mirror does not
    follow bit for bit), and the clade size, so that the clade-table
    launches keep their default CUDA-core shapes too."""
    pf.setCladeSize(e.cTree, 6)
    for g, (dim, nCat) in enumerate(groups_of(prob)):
        if dim == 20:
            pf.setPruneShape(e.cTree, g, 0)


def test_fp32_kernel_bitexact_vs_mirror(golden, port):
    prob, z = golden
    e = Engine(prob)
    e.setPrams()
    force_cuda_core_shapes(e, prob)
    e.logLike(getSiteLikes=1)
    for p, sp in enumerate(prob.parts):
        nPat = e.nPatterns(p)
        decks, eq = pf.getDecks32(e.cTree, p, prob.tree.nNodes, sp.nCat, sp.dim)
        codes, masks = pf.getCompactCodes(e.cParts[p], prob.nTax, nPat)
        pats, cnt, spi = pf.getPatterns(e.cParts[p], prob.nTax, sp.nChar)
        vec, arr = pf.getInvarSites(e.cParts[p], sp.dim, nPat)
        inv = numpy.zeros(nPat, numpy.uint32)
        for j in range(sp.dim):
            inv |= (arr[j].astype(numpy.uint32) << j)
        # a single tree's program reads clade tables, never cherry tables
        tot, like, exps, lnl = port.port_prune32(prob, p, decks, eq, codes, masks, cnt.astype(float), inv,
                                                 cherries=False)
        g_like, g_exps, g_lnl = pf.getPatternLikes(e.cTree, p, nPat)
        assert numpy.array_equal(g_exps, exps), "scaler exponents differ"
        assert numpy.array_equal(g_like.view(numpy.uint32), like.view(numpy.uint32)), "FP32 root likes differ"
        # logf of the mantissa differs by at most a few ulps between CUDA and
        # the host libm: 1e-6 per pattern, summed over the site weights
        numpy.testing.assert_allclose(g_lnl, lnl, rtol=0, atol=1e-6)
        assert abs(e.partLikes[p] - tot) <= 1e-6 * cnt.sum()
    e.free()


def test_site_likes_match_reference(golden):
    prob, z = golden
    e = Engine(prob)
    e.setPrams()
    e.logLike(getSiteLikes=1)
    for p, sp in enumerate(prob.parts):
        s = pf.getSiteLikes(e.cParts[p], sp.nChar)
        numpy.testing.assert_allclose(s, z["p%d_ref_siteLikes" % p], rtol=5e-5)
    e.free()


@pytest.mark.parametrize("name", ["dna64het", "prot48het", "mcmcmc32", "dna32het6"])
def test_full_size_configs_vs_oracle(name, port):
    """Full-size workloads against the FP64 oracle (the port is pinned to the
    reference at 1e-12 by the CPU tests)."""
    prob = sim.make_config(name)
    e = Engine(prob)
    lnl = e.calcLogLike()
    ref, parts = port.port_loglike64(prob)
    assert abs(lnl - ref) <= LNL_RTOL * abs(ref), (name, lnl, ref, (lnl - ref) / ref)
    numpy.testing.assert_allclose(e.partLikes, parts, rtol=LNL_RTOL)
    e.free()


def test_deep_tree_needs_scaling(port):
    """200 taxa with long branches: FP32 without rescaling would underflow."""
    rng = numpy.random.default_rng(11)
    t = sim.yule_tree(200, rng, meanBrLen=0.4)
    prob = sim.Problem(t, [sim.make_part(t, rng, "dna", 400, nComps=2, gammaShape=0.3)], "deep")
    e = Engine(prob)
    lnl = e.calcLogLike()
    ref, _ = port.port_loglike64(prob)
    assert abs(lnl - ref) <= LNL_RTOL * abs(ref)
    e.logLike(getSiteLikes=1)
    _, exps, _ = pf.getPatternLikes(e.cTree, 0, e.nPatterns())
    assert exps.max() > 100          # scaling was exercised
    e.free()


def test_caterpillar_and_multifurcation(port):
    """Unbalanced (caterpillar) tree whose root is a 4-way polytomy."""
    rng = numpy.random.default_rng(5)
    kids = {"r": ["L0", "L1", "L2", "I1"]}
    for k in range(1, 37):
        kids["I%d" % k] = ["M%d" % k, "I%d" % (k + 1)]
    kids["I37"] = ["M37", "M38"]
    t = sim.tree_from_children(kids, "r", rng=rng)
    prob = sim.Problem(t, [sim.make_part(t, rng, "dna", 500, nComps=1, gammaShape=0.6, ambiguity=0.05)],
                       "cat")
    e = Engine(prob)
    lnl = e.calcLogLike()
    ref, _ = port.port_loglike64(prob)
    assert abs(lnl - ref) <= LNL_RTOL * abs(ref)
    e.free()


def test_branch_length_change_and_determinism(port):
    prob, z = sim.load_problem(golden_files()[0])
    e = Engine(prob)
    a = e.calcLogLike()
    assert e.calcLogLike() == a                 # bitwise repeatable
    bl = prob.tree.brLen.copy()
    bl[1:] *= 1.3
    e.setBrLens(bl)
    b = e.calcLogLike()
    ref, _ = port.port_loglike64(prob, brLen=bl)
    assert b != a and abs(b - ref) <= LNL_RTOL * abs(ref)
    e.free()


def test_batch_matches_single(port):
    probs = [sim.load_problem(f)[0] for f in golden_files()[:4]]
    engines = [Engine(p) for p in probs]
    single = [x.calcLogLike() for x in engines]
    batch = pf.treeLogLikeBatch([x.cTree for x in engines], 1)
    assert list(batch) == single
    for x in engines:
        x.free()


def test_topology_change_rebuilds_program(port):
    """An NNI applied through setNodeRelation on the same tree object."""
    prob, z = sim.load_problem(golden_files()[0])
    e = Engine(prob)
    a0 = e.calcLogLike()
    t = prob.tree
    # an internal edge u -> v (v internal, u internal): swap a child of v with a sibling of v
    v = next(x for x in range(t.nNodes) if not t.isLeaf[x] and x != t.root)
    u = int(t.parent[v])
    sibOfV = next(c for c in t.children(u) if c != v)
    childOfV = next(iter(t.children(v)))
    t2 = t.swapped(sibOfV, childOfV)
    e.setTopology(t2)
    lnl2 = e.calcLogLike()
    prob2 = sim.Problem(t2, prob.parts, "nni")
    ref, _ = port.port_loglike64(prob2)
    assert lnl2 != a0 and abs(lnl2 - ref) <= LNL_RTOL * abs(ref)
    e.free()


@pytest.mark.parametrize("name,scale", [("dna64het", 0.05), ("prot48het", 0.1), ("mcmcmc32", 0.1)])
def test_every_tile_shape_gives_the_same_pattern_values(name, scale, port):
    """Tile shapes differ in threads per block, patterns per thread, where the
    P decks live and how many lanes share a pattern's categories; the
    per-pattern scaled likelihoods and scaler exponents must be bitwise the
    same for all of them (only the FP64 block sums are grouped differently)."""
    from p4gpu._lib import P4Error
    prob = sim.make_config(name, scale=scale)
    e = Engine(prob)
    e.setPrams()
    groups = groups_of(prob)
    for g in range(len(groups)):
        pf.setPruneShape(e.cTree, g, 0)
    lnl0 = e.logLike(1)
    ref, _ = port.port_loglike64(prob)
    assert abs(lnl0 - ref) <= LNL_RTOL * abs(ref)
    base = [pf.getPatternLikes(e.cTree, p, e.nPatterns(p)) for p in range(len(prob.parts))]
    tried = 0
    for grp in range(len(groups)):
        for sh in range(13):
            if groups[grp][0] == 20 and sh == TENSOR_SHAPE:
                continue        # the tensor-core kernel has its own test below
            try:
                pf.setPruneShape(e.cTree, grp, sh)
            except P4Error:
                continue
            tried += 1
            lnl = e.logLike(1)
            assert abs(lnl - lnl0) <= 1e-12 * abs(lnl0), (grp, sh, lnl, lnl0)
            for p in range(len(prob.parts)):
                ls, ex, ln = pf.getPatternLikes(e.cTree, p, e.nPatterns(p))
                assert numpy.array_equal(ls, base[p][0]) and numpy.array_equal(ex, base[p][1]), (grp, sh, p)
    assert tried >= 3
    e.free()


@pytest.mark.parametrize("name,scale", [("prot48het", 0.25), ("mcmcmc32", 0.2)])
def test_protein_tensor_core_kernel(name, scale, port):
    """20-state parts through the split-precision TF32 tcgen05 kernel: lnL
    within 1e-6 relative of the reference FP64 algorithm, and every pattern's
    log likelihood within 5e-5 of the FP64 value (the hi + lo TF32 split and
    the tensor core's FP32 accumulation give a few 2^-23 per product, about
    4x the FP32 CUDA-core kernel's per-pattern error)."""
    prob = sim.make_config(name, scale=scale)
    e = Engine(prob)
    e.setPrams()
    g = groups_of(prob).index((20, 4))
    pf.setPruneShape(e.cTree, g, 0)
    lnlCore = e.logLike(1)
    core = [pf.getPatternLikes(e.cTree, p, e.nPatterns(p)) for p in range(len(prob.parts))]
    pf.setPruneShape(e.cTree, g, TENSOR_SHAPE)
    assert pf.getPruneShape(e.cTree, g) == (TENSOR_SHAPE, 128)
    lnl = e.logLike(1)
    ref, _ = port.port_loglike64(prob)
    assert abs(lnl - ref) <= LNL_RTOL * abs(ref), (lnl, ref, lnlCore)
    for p, sp in enumerate(prob.parts):
        ls, ex, ln = pf.getPatternLikes(e.cTree, p, e.nPatterns(p))
        if sp.dim == 20:
            _, pl64, _ = port.port_part_loglike64(prob, p, patLikes=True)
            errTc = numpy.abs(ln - numpy.log(pl64)).max()
            errCore = numpy.abs(core[p][2] - numpy.log(pl64)).max()
            assert errTc <= max(8.0 * errCore, 5e-5), (p, errTc, errCore)
        else:
            assert numpy.array_equal(ls, core[p][0]) and numpy.array_equal(ex, core[p][1])
    assert e.logLike(1) == lnl             # bitwise repeatable
    e.free()


def test_site_rates_match_reference(golden, port):
    """pf.getSiteRates restated (Pf/p4_tree.c:1383-1627): the reference's own
    per-site rates and Gamma categories from the fixtures.  Rates within 2e-5
    relative (1e-4 for 20 states, where the tensor-core kernel may serve the
    part); a category may differ only where the two best categories' root
    sums tie to 1e-5."""
    prob, z = golden
    if prob.tree.isLeaf[prob.tree.root]:
        pytest.skip("the reference routine reads an internal root's CLs only")
    if not any(k.endswith("_ref_siteRates") for k in z.files):
        pytest.skip("no Gamma categories: no site rates")
    e = Engine(prob)
    n = 0
    for p, sp in enumerate(prob.parts):
        k = "p%d_ref_siteRates" % p
        if k not in z.files:
            continue
        rates, cats = pf.getSiteRates(e.cTree, e.cParts[p], p, sp.nChar)
        numpy.testing.assert_allclose(rates, z[k], rtol=1e-4 if sp.dim == 20 else 2e-5, atol=0)
        bad = numpy.nonzero(cats != z["p%d_ref_gammaCats" % p])[0]
        if len(bad):
            _, _, spi, cw = port.port_part_loglike64(prob, p, catWork=True)
            w = numpy.sort(cw[spi[bad]], axis=1)
            assert numpy.all(w[:, -1] - w[:, -2] <= 1e-5 * w[:, -1]), (p, len(bad))
        n += 1
    e.free()
    assert n >= 1


@pytest.mark.parametrize("name,scale", [("dna64het", 0.05), ("prot48het", 0.1), ("mcmcmc32", 0.1),
                                        ("dna16", 1.0)])
def test_clade_tables_leave_every_pattern_unchanged(name, scale, port):
    """Clade tables (each small subtree evaluated once per distinct leaf-code
    combination) against the same tree without them: every pattern's log
    likelihood bitwise equal, for maximal clades of up to 2, 4, 6 and 8
    leaves, with the pruning shape pinned (CUDA-core kernels)."""
    prob = sim.make_config(name, scale=scale)
    e = Engine(prob)
    e.setPrams()
    groups = groups_of(prob)
    for g in range(len(groups)):
        pf.setPruneShape(e.cTree, g, 0)
    out = {}
    for L in (0, 2, 4, 6, 8):
        pf.setCladeSize(e.cTree, L)
        lnl = e.logLike(1)
        pats = [pf.getPatternLikes(e.cTree, p, e.nPatterns(p))[2] for p in range(len(prob.parts))]
        out[L] = (lnl, pats, pf.treeInfo(e.cTree)["nProg"])
    ref, _ = port.port_loglike64(prob)
    assert abs(out[0][0] - ref) <= LNL_RTOL * abs(ref)
    for L in (2, 4, 6, 8):
        assert out[L][0] == out[0][0], (L, out[L][0], out[0][0])
        for p in range(len(prob.parts)):
            assert numpy.array_equal(out[L][1][p], out[0][1][p]), (L, p)
        assert out[L][2] < out[0][2]          # a shorter whole-tree program
    e.free()


@pytest.mark.parametrize("name,scale", [("dna64het", 0.05), ("mcmcmc32", 0.1)])
def test_clade_tables_follow_topology_changes(name, scale):
    """Clade tables are renumbered on the GPU at every topology change: a run
    of evaluations that alternates between trees related by subtree swaps
    gives, with clades of up to 6 leaves, bitwise the same log likelihoods
    and per-pattern values as the same run without clade tables."""
    prob = sim.make_config(name, scale=scale)
    t0 = prob.tree
    leaves = [v for v in range(t0.nNodes) if t0.isLeaf[v] and v != t0.root]
    trees = [t0, t0.swapped(leaves[0], leaves[-1]), t0.swapped(leaves[1], leaves[len(leaves) // 2])]
    runs = {}
    for L in (0, 6):
        e = Engine(prob)
        e.setPrams()
        for g in range(len(groups_of(prob))):
            pf.setPruneShape(e.cTree, g, 0)
        pf.setCladeSize(e.cTree, L)
        seq = []
        for i in range(7):
            tt = trees[i % 3]
            e.setTopologyArrays(tt.parent, tt.leftChild, tt.sibling, tt.root)
            lnl = e.logLike(1)
            pats = [pf.getPatternLikes(e.cTree, p, e.nPatterns(p))[2] for p in range(len(prob.parts))]
            seq.append((lnl, pats))
        runs[L] = seq
        e.free()
    for (a, pa), (b, pb) in zip(runs[0], runs[6]):
        assert a == b
        for x, y in zip(pa, pb):
            assert numpy.array_equal(x, y)
    assert runs[0][0][0] != runs[0][1][0]   # the topologies differ


@pytest.mark.parametrize("name,scale", [("dna64het", 0.05), ("prot48het", 0.1), ("mcmcmc32", 0.1)])
def test_graph_replay_is_bitwise_the_plain_launches(name, scale):
    """The setPrams and pruning sequences replayed from CUDA graphs give the
    plain launches' results bit for bit, through branch-length, composition
    and topology changes (each of which may change the captured sequence)."""
    prob = sim.make_config(name, scale=scale)
    t0 = prob.tree
    leaves = [v for v in range(t0.nNodes) if t0.isLeaf[v] and v != t0.root]
    t1 = t0.swapped(leaves[0], leaves[-1])
    rng = numpy.random.default_rng(3)
    bls = [t0.brLen * numpy.exp(rng.normal(0, 0.1, t0.nNodes)) for _ in range(4)]
    out = {}
    for graphs in (0, 1):
        e = Engine(prob)
        pf.setGraphs(e.cTree, graphs)
        pf.setCladeSize(e.cTree, 6)   # the same clade tables in both runs (no timed choice)
        seq = [e.calcLogLike()]
        for i in range(6):
            e.setBrLensFast(bls[i % 4])
            if i == 2:
                c = prob.parts[0].comps[0] * numpy.exp(rng.normal(0, 0.01, prob.parts[0].dim))
                e.setComp(0, 0, c / c.sum())
            if i == 4:
                e.setTopologyArrays(t1.parent, t1.leftChild, t1.sibling, t1.root)
            pf.treeLogLikeAsync(e.cTree, 1)
            seq.append(pf.treeLogLikeWait(e.cTree))
        out[graphs] = seq
        e.free()
        rng = numpy.random.default_rng(3)
        bls = [t0.brLen * numpy.exp(rng.normal(0, 0.1, t0.nNodes)) for _ in range(4)]
    assert out[0] == out[1], (out[0], out[1])


@pytest.mark.parametrize("nTax,dtype,nSites,brLen", [(1000, "dna", 600, 0.005), (600, "dna", 1000, 0.02),
                                                     (400, "protein", 300, 0.05)])
def test_large_trees_vs_oracle(nTax, dtype, nSites, brLen, port):
    """Trees far larger than the workloads: the tile shape falls back to one
    whose shared-memory footprint fits (every taxon's codes, the program's
    stack), clade tables included, and lnL still agrees with the FP64 oracle
    (branch lengths short enough that the unscaled FP64 oracle does not
    underflow)."""
    rng = numpy.random.default_rng(nTax)
    t = sim.yule_tree(nTax, rng, meanBrLen=brLen)
    prob = sim.Problem(t, [sim.make_part(t, rng, dtype, nSites, nComps=2, gammaShape=0.7)], "large")
    e = Engine(prob)
    lnl = e.calcLogLike()
    ref, _ = port.port_loglike64(prob)
    assert abs(lnl - ref) <= LNL_RTOL * abs(ref), (lnl, ref)
    e.free()


def test_clade_tables_on_every_fixture(golden):
    """Clade tables of up to 6 leaves against none on every golden case
    (ambiguity codes, invariant sites, several parts, relative rates, a
    leaf root, no Gamma): per-pattern values bitwise equal."""
    prob, z = golden
    out = {}
    for L in (0, 6):
        e = Engine(prob)
        e.setPrams()
        for g in range(len(groups_of(prob))):
            pf.setPruneShape(e.cTree, g, 0)
        pf.setCladeSize(e.cTree, L)
        lnl = e.logLike(1)
        out[L] = (lnl, [pf.getPatternLikes(e.cTree, p, e.nPatterns(p))[2] for p in range(len(prob.parts))])
        e.free()
    assert out[0][0] == out[6][0]
    for a, b in zip(out[0][1], out[6][1]):
        assert numpy.array_equal(a, b)


def test_tensor_core_clade_tables(port):
    """Protein clade tables computed by the tensor-core kernel (split TF32)
    against the CUDA-core clade kernel: lnL within the FP32 target of the
    FP64 oracle, per-pattern log likelihoods within the tensor-core
    kernel's tolerance."""
    prob = sim.make_config("prot48het", scale=0.1)
    out = {}
    for shape in (0, TENSOR_SHAPE):
        e = Engine(prob)
        e.setPrams()
        pf.setPruneShape(e.cTree, 0, TENSOR_SHAPE)
        pf.setCladeSize(e.cTree, 6)
        pf.setCladeShape(e.cTree, 0, shape)
        lnl = e.logLike(1)
        assert pf.treeInfo(e.cTree)["nClade"] > 0
        out[shape] = (lnl, pf.getPatternLikes(e.cTree, 0, e.nPatterns(0))[2])
        e.free()
    ref, _ = port.port_loglike64(prob)
    for shape in out:
        assert abs(out[shape][0] - ref) <= LNL_RTOL * abs(ref), (shape, out[shape][0], ref)
    numpy.testing.assert_allclose(out[TENSOR_SHAPE][1], out[0][1], rtol=0, atol=5e-5)


def test_batch_with_clade_tables_matches_single(port):
    """Batches with clade tables: every tree's lnL bitwise that of the same
    tree evaluated alone with the same clade size, with new branch lengths
    for every tree at every step (the clade tables are refilled each step)
    and through a topology change of one tree (its clades are renumbered and
    the batch graph captured again)."""
    prob = sim.make_config("dna64het", scale=0.05)
    t0 = prob.tree
    leaves = [v for v in range(t0.nNodes) if t0.isLeaf[v] and v != t0.root]
    t1 = t0.swapped(leaves[0], leaves[-1])
    first = Engine(prob)
    engines = [first] + [Engine(prob, shared=(first.cData, first.cParts)) for _ in range(2)]   # one data object
    singles = [Engine(prob) for _ in range(3)]
    rng = numpy.random.default_rng(7)
    bls = [t0.brLen * numpy.exp(rng.normal(0, 0.1, t0.nNodes)) for _ in range(3)]
    for e, s, bl in zip(engines, singles, bls):
        pf.setCladeSize(e.cTree, 6)
        pf.setCladeSize(s.cTree, 6)
        e.setBrLensFast(bl)
        s.setBrLensFast(bl)
    batch = pf.Batch([e.cTree for e in engines], clades=True)
    batch.logLike()   # the batch's tile shape (timed on the batch): the lone trees use it too,
    shape, _ = pf.getPruneShape(engines[0].cTree, 0)   # since the per-block sums follow the tile
    for s in singles:
        s.calcLogLike()
        pf.setPruneShape(s.cTree, 0, shape)
    for step in range(4):
        if step >= 1:   # every tree's branch lengths move
            for i, (e, s) in enumerate(zip(engines, singles)):
                bl = bls[(i + step) % 3] * (1.0 + 0.05 * step)
                e.setBrLensFast(bl)
                s.setBrLensFast(bl)
        if step == 2:
            for x in (engines[1], singles[1]):
                x.setTopologyArrays(t1.parent, t1.leftChild, t1.sibling, t1.root)
        got = batch.logLike()
        want = [s.calcLogLike() for s in singles]
        assert list(got) == want, (step, got, want)
    batch.free()
    for x in engines[::-1] + singles:   # the data's owner last
        x.free()


@pytest.mark.parametrize("name", ["dna64het_small", "dna_2part_relrate"])
def test_programmatic_launch_same_results(lib, name):
    """Programmatic dependent launch changes when kernels start, not what they
    compute: lnL and part lnLs bitwise equal with it on and off (new trees,
    so that no graph captured in the other mode is replayed)."""
    prob, _ = sim.load_problem([f for f in golden_files() if f.endswith(name + ".npz")][0])
    out = []
    pf.setAutotune(False)     # the same tile shapes in both modes (the timing could differ)
    try:
        for on in (False, True):
            pf.setProgrammaticLaunch(on)
            e = Engine(prob)
            vals = []
            for _ in range(3):
                vals.append((e.calcLogLike(), tuple(e.partLikes)))
            out.append(vals)
            e.free()
    finally:
        pf.setProgrammaticLaunch(True)
        pf.setAutotune(True)
    assert out[0] == out[1]


def test_branch_lengths_read_from_pinned_image(port):
    """An evaluation whose only change is branch lengths copies no parameter
    image (the P-deck kernel reads them from the pinned host image): a
    sequence of branch-length-only changes, composition changes, returns to
    earlier values and a batch evaluation in between gives the oracle's lnL
    at every step."""
    prob, _ = sim.load_problem(golden_files()[0])
    e = Engine(prob)
    e.calcLogLike()
    sp = prob.parts[0]
    base = prob.tree.brLen.copy()
    c0 = sp.comps[0].copy()
    c1 = sim._fix(c0 * (1.0 + 0.05 * numpy.cos(numpy.arange(sp.dim))))
    steps = [(1.0, c0), (1.2, c0), (1.2, c1), (0.8, c1), (0.8, c0), (1.0, c0), (1.2, c0), (1.2, c0)]
    for k, (scale, comp) in enumerate(steps):
        bl = base * scale
        e.setBrLens(bl)
        sp.comps[0][:] = comp
        e.setComp(0, 0, comp)
        lnl = e.calcLogLike()
        ref, _ = port.port_loglike64(prob, brLen=bl)
        assert abs(lnl - ref) <= LNL_RTOL * abs(ref), (k, lnl, ref)
        if k == 3:   # the batch copies the image itself
            b = pf.Batch([e.cTree])
            assert abs(b.logLike()[0] - lnl) <= 1e-9 * abs(lnl)
            b.free()
    sp.comps[0][:] = c0
    e.free()


@pytest.mark.parametrize("spec", [103, 106, 113, 105])   # JTT, WAG, LG, mtMam (zeros in its table)
def test_empirical_protein_matrix(port, spec):
    """An empirical protein rate matrix chosen by its spec number
    (p4_newRMatrix fills it from the library's table; no values are poked
    in) gives the lnL the reference core computes with its own matrix for
    that spec, on the 48-taxon protein fixture with 3 compositions + G4, on
    every protein tile shape (the tensor-core kernel included)."""
    import os
    from conftest import REPO
    prob, _ = sim.load_problem(os.path.join(REPO, "tests", "golden", "prot48het_small.npz"))
    sp = prob.parts[0]
    R = port.ref_bigR(spec) if port.have_ref() else None
    if R is None:
        R = numpy.zeros((20, 20))
        pf.getBigR(spec, R)
    sp.rmats = numpy.ascontiguousarray(numpy.stack([R] * sp.rmats.shape[0]))
    sp.rSpecs = [spec] * sp.rmats.shape[0]
    ref = port.RefTree(prob).logLike()[0] if port.have_ref() else port.port_loglike64(prob)[0]
    e = Engine(prob)
    try:
        lnl = e.calcLogLike()
        assert abs(lnl - ref) <= LNL_RTOL * abs(ref), (spec, lnl, ref)
        for shape in range(4):
            pf.setPruneShape(e.cTree, 0, shape)
            lnl = e.calcLogLike()
            assert abs(lnl - ref) <= LNL_RTOL * abs(ref), (spec, shape, lnl, ref)
    finally:
        e.free()


def test_batch_reevaluates_only_changed_parts(port):
    """Part-granular batches (p4's Chain re-evaluates only the part a per-part
    proposal changed): after one part's composition, Gamma shape, R matrix
    or pInvar changes in one tree, or one tree's branch lengths, only those
    (tree, part) units are evaluated again and the others keep their lnL;
    every tree's lnL stays bitwise that of the same tree evaluated alone at
    the batch's tile shape, through changes, returns to earlier values and
    unchanged steps, and matches the oracle."""
    prob = sim.make_config("mcmcmc32", scale=0.1)
    first = Engine(prob)
    engines = [first] + [Engine(prob, shared=(first.cData, first.cParts)) for _ in range(2)]
    singles = [Engine(prob) for _ in range(3)]
    batch = pf.Batch([e.cTree for e in engines])
    batch.logLike()
    for s in singles:
        s.calcLogLike()
    nGroups = 0
    while True:   # the batch's tile shape of every (dim, nCat) group, for the lone trees too
        try:
            pf.getPruneShape(engines[0].cTree, nGroups)
            nGroups += 1
        except P4Error:
            break
    for g in range(nGroups):
        sh, _ = pf.getPruneShape(engines[0].cTree, g)
        for s in singles:
            pf.setPruneShape(s.cTree, g, sh)
    rng = numpy.random.default_rng(3)
    parts = prob.parts
    dnaP = next(p for p, sp in enumerate(parts) if sp.dim == 4)
    protP = next(p for p, sp in enumerate(parts) if sp.dim == 20)

    def comp_change(e, p, k):
        return sim._fix(parts[p].comps[0] * numpy.exp(rng.normal(0, 0.05, parts[p].dim)))

    saved = parts[dnaP].comps[0].copy()
    steps = []
    for step in range(7):
        i = step % 3
        e, s = engines[i], singles[i]
        if step == 0:     # one DNA part's composition in tree 0
            c = comp_change(e, dnaP, step)
            e.setComp(dnaP, 0, c)
            s.setComp(dnaP, 0, c)
        elif step == 1:   # one protein part's Gamma shape in tree 1
            a = parts[protP].gammaShapes[0] * 1.3
            e.setGamma(protP, 0, a)
            s.setGamma(protP, 0, a)
        elif step == 2:   # tree 2's branch lengths (every part)
            bl = prob.tree.brLen * numpy.exp(rng.normal(0, 0.1, prob.tree.nNodes))
            e.setBrLensFast(bl)
            s.setBrLensFast(bl)
        elif step == 3:   # back to tree 0's first composition
            e.setComp(dnaP, 0, saved)
            s.setComp(dnaP, 0, saved)
        elif step == 4:   # a protein R matrix in tree 1
            rv = sim.upper_of(parts[protP].rmats[0]) * numpy.exp(rng.normal(0, 0.05, 190))
            e.setRMatrix(protP, 0, rv / rv.sum())
            s.setRMatrix(protP, 0, rv / rv.sum())
        # steps 5, 6: nothing changes
        got = batch.logLike()
        want = [x.calcLogLike() for x in singles]
        assert list(got) == want, (step, list(got), want)
        steps.append(list(got))
    assert steps[5] == steps[4] == steps[6]
    # the oracle, for the last state of tree 0 (its composition restored)
    ref, _ = port.port_loglike64(prob)
    assert abs(steps[-1][0] - ref) <= LNL_RTOL * abs(ref)
    batch.free()
    for x in engines + singles:
        x.free()


@pytest.mark.parametrize("kind", ["poisson", "f81", "neardeg9", "neardeg5", "wag_skewed"])
def test_protein_eigensystems_degenerate_spectra(port, kind):
    """20-state eigensystems take the FP32-start + FP64-refinement path when
    the spectrum is separated or exactly degenerate, and fall back to FP64
    Jacobi sweeps when eigenvalues are close but unequal (gaps of 1e-9 and
    1e-5 relative): either way every FP64 P deck equals the reference core's
    within 1e-12, and the lnL agrees."""
    import os
    from conftest import REPO
    if not port.have_ref():
        pytest.skip("reference core not built")
    prob, _ = sim.load_problem(os.path.join(REPO, "tests", "golden", "prot48het_small.npz"))
    sp = prob.parts[0]
    rng = numpy.random.default_rng(17)
    nC = sp.comps.shape[0]
    R = numpy.ones((20, 20))
    comps = numpy.full((nC, 20), 0.05)
    if kind == "f81":
        comps = rng.dirichlet(numpy.full(20, 50.0), nC)
    elif kind.startswith("neardeg"):
        eps = 1e-9 if kind == "neardeg9" else 1e-5
        N = rng.standard_normal((20, 20))
        R = 1.0 + eps * (N + N.T) / 2
    elif kind == "wag_skewed":
        R = numpy.zeros((20, 20))
        pf.getBigR(106, R)
        comps = rng.dirichlet(numpy.full(20, 0.3), nC)
        comps = numpy.maximum(comps, 1e-6)
        comps /= comps.sum(1)[:, None]
    numpy.fill_diagonal(R, 0.0)
    sp.rmats = numpy.ascontiguousarray(numpy.stack([R] * sp.rmats.shape[0]))
    sp.comps[:] = comps
    ref = port.RefTree(prob)
    e = Engine(prob)
    try:
        lnl = e.calcLogLike()
        r = ref.logLike()[0]
        assert abs(lnl - r) <= LNL_RTOL * abs(r), (kind, lnl, r)
        nodes = [v for v in range(len(prob.tree.brLen)) if v != prob.tree.root][::7]
        for v in nodes:
            for c in range(sp.nCat):
                d = pf.getPDeck(e.cNodes[v], 0, c, 20)
                numpy.testing.assert_allclose(d, ref.pdeck(v, 0, c), rtol=0, atol=1e-12, err_msg=kind)
    finally:
        e.free()


@pytest.mark.parametrize("fixture,seed", [("prot48het_small.npz", 3), ("prot48het_small.npz", 4),
                                          ("dna64het_small.npz", 5), ("dna64het_small.npz", 6)])
def test_decks_random_skewed_models(port, fixture, seed):
    """P decks computed in FP32-pair arithmetic (per-lane for DNA, one block per
    deck for protein) on random models with strongly skewed compositions
    (Dirichlet(0.3), floor 1e-6) and log-normal exchangeabilities spanning
    about four orders of magnitude: every FP64 deck of every fourth node and
    every category equals the reference core's within 1e-12, and the lnL
    agrees within the FP32 tolerance."""
    import os
    from conftest import REPO
    if not port.have_ref():
        pytest.skip("reference core not built")
    prob, _ = sim.load_problem(os.path.join(REPO, "tests", "golden", fixture))
    rng = numpy.random.default_rng(seed)
    for sp in prob.parts:
        d = sp.dim
        for r in range(sp.rmats.shape[0]):
            R = numpy.exp(rng.normal(0.0, 1.5, (d, d)))
            R = (R + R.T) / 2
            numpy.fill_diagonal(R, 0.0)
            sp.rmats[r] = R
        for c in range(sp.comps.shape[0]):
            x = numpy.maximum(rng.dirichlet(numpy.full(d, 0.3)), 1e-6)
            sp.comps[c] = x / x.sum()
    ref = port.RefTree(prob)
    e = Engine(prob)
    try:
        lnl = e.calcLogLike()
        r = ref.logLike()[0]
        assert abs(lnl - r) <= LNL_RTOL * abs(r), (lnl, r)
        for p, sp in enumerate(prob.parts):
            for v in range(0, len(prob.tree.brLen), 4):
                if v == prob.tree.root:
                    continue
                for c in range(sp.nCat):
                    numpy.testing.assert_allclose(pf.getPDeck(e.cNodes[v], p, c, sp.dim), ref.pdeck(v, p, c),
                                                  rtol=0, atol=1e-12, err_msg="node %d cat %d" % (v, c))
    finally:
        e.free()
