"""Maximum-likelihood fixtures: the reference's own model-parameter optimiser
(Pf/p4_treeOpt.c p4_newtAndBrentPowellOpt: Newton branch lengths alternating
with praxis over the free parameters, after p4_newtSetup as Tree.optLogLike
calls it, p4/tree.py:9467-9470) run on small seeded problems.

    python tests/golden/make_opt_golden.py [REFERENCE_PF_DIR]

Each fixture holds the problem (sim.save_problem), which values are free
(free_comps, free_rmats, free_gdasrvs, free_pInvar: per part 0/1), the
starting lnL, and the reference's optimum: lnL, branch lengths, comps,
R-matrix upper triangles, gamma shapes and pInvar per part.
"""
import ctypes
import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "p4-phylogenetics_gb300"))
sys.path.insert(0, REPO)

from p4gpu import sim  # noqa: E402
from oracle import oracle  # noqa: E402

OUT = os.path.join(HERE, "opt")


def cases():
    rng = numpy.random.default_rng(3)
    out = {}
    t = sim.yule_tree(16, rng)
    base = sim.Problem(t, [sim.make_part(t, rng, "dna", 300, nComps=1, gammaShape=0.5)], "opt16")
    out["opt16_gamma"] = (base, (0, 0, 1, 0))                 # one parameter: 1D Brent in the reference
    out["opt16_comp_gamma"] = (base, (1, 0, 1, 0))
    out["opt16_gtr_gamma"] = (base, (1, 1, 1, 0))
    t = sim.yule_tree(12, rng)
    pinv = sim.Problem(t, [sim.make_part(t, rng, "dna", 400, nComps=1, gammaShape=0.8, pInvar=0.2)],
                       "opt12_pinv")
    out["opt12_gtr_gamma_pinv"] = (pinv, (1, 1, 1, 1))
    t = sim.yule_tree(10, rng)
    het = sim.Problem(t, [sim.make_part(t, rng, "dna", 500, nComps=2, compAlpha=5.0, gammaShape=0.6)],
                      "opt10_het")
    out["opt10_twocomps_gamma"] = (het, (1, 0, 1, 0))
    return out


def run(prob, free):
    lib = oracle.ref_lib()
    lib.ref_setFree.restype = None
    lib.ref_setFree.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 5
    lib.ref_optimize.restype = ctypes.c_double
    lib.ref_optimize.argtypes = [ctypes.c_void_p, oracle.D, oracle.D]
    lib.ref_pInvar.restype = ctypes.c_double
    lib.ref_pInvar.argtypes = [ctypes.c_void_p, ctypes.c_int]
    r = oracle.RefTree(prob)
    lnl0, _ = r.logLike()
    for p in range(len(prob.parts)):
        lib.ref_setFree(r.h, p, *free)
    bl = numpy.zeros(prob.tree.nNodes)
    ru = numpy.zeros(sum(sp.rmats.shape[0] * sp.dim * (sp.dim - 1) // 2 for sp in prob.parts))
    lnl = lib.ref_optimize(r.h, oracle._d(bl), oracle._d(ru))
    res = dict(ref_start_lnL=lnl0, ref_opt_lnL=lnl, ref_opt_brLens=bl, ref_opt_rUpper=ru)
    # comps, gamma shapes (aliased buffers) and pInvar as the reference left them
    for p, sp in enumerate(prob.parts):
        comps, gv = r._keep[5 * p], r._keep[5 * p + 2]
        res["p%d_ref_opt_comps" % p] = comps.copy()
        res["p%d_ref_opt_gamma" % p] = gv[: len(sp.gammaShapes)].copy()
        res["p%d_ref_opt_pInvar" % p] = lib.ref_pInvar(r.h, p)
    return res


def main():
    refdir = sys.argv[1] if len(sys.argv) > 1 else os.environ.get(oracle.REF_ENV)
    if refdir:
        oracle.build(ref=True, refdir=refdir)
    if not oracle.have_ref():
        sys.exit("usage: make_opt_golden.py REFERENCE_PF_DIR (or set %s)" % oracle.REF_ENV)
    os.makedirs(OUT, exist_ok=True)
    for name, (prob, free) in cases().items():
        res = run(prob, free)
        extra = dict(free_comps=free[0], free_rmats=free[1], free_gdasrvs=free[2], free_pInvar=free[3], **res)
        sim.save_problem(prob, os.path.join(OUT, name + ".npz"), **extra)
        print("%-24s start %.6f -> reference optimum %.6f" % (name, res["ref_start_lnL"], res["ref_opt_lnL"]))


if __name__ == "__main__":
    main()
