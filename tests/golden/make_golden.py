"""Generate tests/golden/*.npz from the reference p4 likelihood core.

Each fixture holds a complete problem (tree, model, alignment) and the
reference's own outputs for it: lnL, per-part lnL, per-site likelihoods,
discrete-gamma rates, P decks of a few nodes, and the compressed patterns
with their counts, site->pattern index and invariant-site tables.  The
reference core (Pf/*.c) is compiled by oracle/Makefile; this script runs
in the development container, where the reference sources exist.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "p4-phylogenetics_gb300"))
sys.path.insert(0, REPO)

from p4gpu import sim  # noqa: E402
from oracle import oracle  # noqa: E402


def root_leaf_problem(rng):
    # A(root, leaf) -> 1 -> {B, 3 -> {C, D}}: p4 allows rooting on a leaf
    parent = [-1, 0, 1, 1, 3, 3]
    left = [1, 2, -1, 4, -1, -1]
    sib = [-1, -1, 3, -1, 5, -1]
    isLeaf = [1, 0, 1, 0, 1, 1]
    seqNum = [0, -1, 1, -1, 2, 3]
    brLen = [0.0, 0.15, 0.05, 0.2, 0.08, 0.12]
    tree = sim.TreeSpec(parent, left, sib, isLeaf, seqNum, brLen, root=0)
    part = sim.make_part(tree, rng, "dna", 300, nComps=1, gammaShape=0.7, ambiguity=0.08)
    return sim.Problem(tree, [part], "rootleaf")


def cases():
    out = {}
    out["dna16"] = sim.make_config("dna16")
    out["dna64het_small"] = sim.make_config("dna64het", scale=0.02)
    out["prot48het_small"] = sim.make_config("prot48het", scale=0.05)
    out["mcmcmc32_small"] = sim.make_config("mcmcmc32", scale=0.02)
    rng = numpy.random.default_rng(7)
    t = sim.yule_tree(12, rng)
    out["dna_ambig_pinv"] = sim.Problem(t, [sim.make_part(t, rng, "dna", 600, nComps=2, gammaShape=0.4,
                                                          pInvar=0.25, ambiguity=0.12)], "dna_ambig_pinv")
    t = sim.yule_tree(10, rng)
    out["prot_ambig_nocat"] = sim.Problem(t, [sim.make_part(t, rng, "protein", 400, nComps=1, nCat=1,
                                                            ambiguity=0.1)], "prot_ambig_nocat")
    t = sim.yule_tree(20, rng, meanBrLen=0.3)
    parts = [sim.make_part(t, rng, "dna", 500, nComps=3, gammaShape=1.3, nCat=4, nR=2, relRate=0.6),
             sim.make_part(t, rng, "dna", 300, nComps=1, nCat=1, relRate=1.8, pInvar=0.1)]
    out["dna_2part_relrate"] = sim.Problem(t, parts, "dna_2part_relrate")
    t = sim.yule_tree(3, rng)
    out["dna3_minimal"] = sim.Problem(t, [sim.make_part(t, rng, "dna", 50, nComps=1, gammaShape=2.0)],
                                      "dna3_minimal")
    out["rootleaf"] = root_leaf_problem(rng)
    return out


SIM_SEED = 5   # Philox stream of the simulation fixtures


def main():
    refdir = sys.argv[1] if len(sys.argv) > 1 else os.environ.get(oracle.REF_ENV)
    if not refdir:
        sys.exit("usage: make_golden.py REFERENCE_PF_DIR (or set %s)" % oracle.REF_ENV)
    oracle.build(ref=True, refdir=refdir)
    for name, prob in cases().items():
        ref = oracle.RefTree(prob)
        lnl, pl = ref.logLike()
        extra = dict(ref_lnL=lnl, ref_partLikes=pl)
        for p, sp in enumerate(prob.parts):
            k = "p%d_" % p
            pats, cnt, spi, iv, ia = ref.patterns(p)
            extra[k + "ref_patterns"] = pats
            extra[k + "ref_counts"] = cnt
            extra[k + "ref_seqPosIdx"] = spi
            extra[k + "ref_invVec"] = iv
            extra[k + "ref_invArr"] = ia
            extra[k + "ref_gammaRates"] = ref.gammaRates(p)
            nodes = [v for v in range(prob.tree.nNodes) if v != prob.tree.root]
            pick = sorted(set([nodes[0], nodes[len(nodes) // 2], nodes[-1]]))
            extra[k + "ref_deckNodes"] = numpy.array(pick, numpy.int32)
            extra[k + "ref_decks"] = numpy.stack([numpy.stack([ref.pdeck(v, p, c) for c in range(sp.nCat)])
                                                  for v in pick])
        # site likes last: p4_partLogLike with getSiteLikes recomputes the root sum only
        for p in range(len(prob.parts)):
            extra["p%d_ref_siteLikes" % p] = ref.siteLikes(p)
            if prob.parts[p].nCat > 1 and len(prob.parts[p].gammaShapes) == 1:
                r, c = ref.siteRates(p)
                extra["p%d_ref_siteRates" % p] = r
                extra["p%d_ref_gammaCats" % p] = c
        # ancestral-state draws on the same root CLs (libc random seeded per
        # part; the uniforms it used are stored with the draws)
        if not prob.tree.isLeaf[prob.tree.root]:
            for p in range(len(prob.parts)):
                u, d = ref.drawAncStates(p, 11 + p)
                extra["p%d_ref_ancUniforms" % p] = u
                extra["p%d_ref_ancDraws" % p] = d.astype(numpy.int8)
        # Newton branch-length optimisation on a fresh copy (it moves the
        # branch lengths); the reference's cl2 needs an internal root
        if not prob.tree.isLeaf[prob.tree.root]:
            opt = oracle.RefTree(prob)
            opt.logLike()
            nl, nb = opt.newtOptimize()
            extra["ref_newtLnL"] = nl
            extra["ref_newtBrLens"] = nb
        # simulation last: it replaces the reference's alignment
        seqs, nDrawn = ref.simulate(SIM_SEED)
        extra["ref_simUniforms"] = numpy.int64(nDrawn)
        for p, sq in enumerate(seqs):
            extra["p%d_ref_simSeqs" % p] = sq.astype(numpy.int8)
        path = os.path.join(HERE, name + ".npz")
        sim.save_problem(prob, path, **extra)
        print("%-20s lnL %.6f  parts %s  %d bytes" % (name, lnl, numpy.round(pl, 4), os.path.getsize(path)))


if __name__ == "__main__":
    main()
