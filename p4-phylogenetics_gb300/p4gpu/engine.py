"""Wire a synthetic Problem into libp4gpu through the pf calls.

The sequence of calls is the one p4 makes: Alignment -> Part
(p4/alignment.py:5830-5877), Data._setCStuff (p4/data.py:269-277),
Model.allocCStuff / setCStuff (p4/model.py:735-833), Tree._allocCStuff /
setCStuff (p4/tree.py:9255-9377), then p4_setPrams + p4_treeLogLike
(p4/tree.py:9400-9412).
"""
import numpy

from . import pf
from .var import var


def make_data(problem):
    """pf data objects for a Problem's alignment: (cData, [cPart])."""
    nTax = problem.tree.nLeaves
    cData = pf.newData(nTax, len(problem.parts))
    cParts = []
    for pNum, sp in enumerate(problem.parts):
        eq = sp.equateSymbols()
        cp = pf.newPart(nTax, sp.nChar, eq, len(eq), sp.symbols, sp.dim)
        if eq:
            pf.pokeEquatesTable(cp, sp.equatesTable())
        pf.pokeSequences(cp, "".join(sp.sequences))
        pf.makePatterns(cp)
        pf.setGlobalInvarSitesVec(cp)
        pf.pokePartInData(cp, cData, pNum)
        cParts.append(cp)
    return cData, cParts


class Engine(object):
    """One library tree (with its own model) for a Problem.  Several engines
    may share one data object (`shared=(cData, cParts)`), as the chains of
    an MCMC share p4's Data."""

    def __init__(self, problem, shared=None, free=None):
        """free: (comps, rMatrices, gdasrvs, pInvar) flags, the same for every
        part, marking which model values the ML optimiser may move (the
        model's nFreePrams counted from them as p4's Model does); None: the
        flags p4's MCMC uses, with nFreePrams 0 (branch lengths only)."""
        self.problem = problem
        tree = problem.tree
        self.nParts = len(problem.parts)
        self.ownsData = shared is None
        self.cData, self.cParts = make_data(problem) if shared is None else shared
        # model
        nFree = 0
        if free is not None:
            fc, fr, fg, fp = (int(bool(x)) for x in free)
            for sp in problem.parts:
                nFree += fc * sp.comps.shape[0] * (sp.dim - 1)
                nFree += fr * sum(1 for x in getattr(sp, "rSpecs", [20] * sp.rmats.shape[0]) if x == 20) * \
                    (sp.dim * (sp.dim - 1) // 2 - 1)
                nFree += fg * len(sp.gammaShapes) + fp
        self.cModel = pf.p4_newModel(self.nParts, int(self.nParts > 1), 0, nFree, 1,
                                     var._rMatrixNormalizeTo1, *var.bounds())
        self.compVals, self.gVals, self.gFreqs, self.gRates, self.bqet = [], [], [], [], []
        for pNum, sp in enumerate(problem.parts):
            nG = len(sp.gammaShapes)
            bq = numpy.ones((sp.comps.shape[0], sp.rmats.shape[0]), numpy.int32)
            self.bqet.append(bq)
            # a model with invariant sites has its pInvar free, as p4's
            # defaults make it (the ancestral-state draw reads the flag)
            fc, fr, fg, fp = (1, 1, 1, int(sp.pInvar > 0.0)) if free is None else (int(bool(x)) for x in free)
            pf.p4_newModelPart(self.cModel, pNum, sp.dim, sp.comps.shape[0], sp.rmats.shape[0], nG,
                               sp.nCat, fp, bq)
            cv = [numpy.array(c, numpy.double) for c in sp.comps]
            for m, c in enumerate(cv):
                pf.p4_newComp(self.cModel, pNum, m, fc, c)
            self.compVals.append(cv)
            for r in range(sp.rmats.shape[0]):
                spec = sp.rSpecs[r] if hasattr(sp, "rSpecs") else 20
                if spec != 20:   # an empirical matrix: the library fills its values, and it is fixed
                    pf.p4_newRMatrix(self.cModel, pNum, r, 0, spec)
                    continue
                pf.p4_newRMatrix(self.cModel, pNum, r, fr, 20)
                for i in range(sp.dim - 1):
                    for j in range(i + 1, sp.dim):
                        pf.p4_setRMatrixBigR(self.cModel, pNum, r, i, j, sp.rmats[r, i, j])
            gv, gf, gr = [], [], []
            for g in range(nG):
                v = numpy.array([sp.gammaShapes[g]], numpy.double)
                f = numpy.zeros(sp.nCat, numpy.double)
                rt = numpy.zeros(sp.nCat, numpy.double)
                h = pf.p4_newGdasrv(self.cModel, pNum, g, sp.nCat, fg, v, f, rt)
                pf.gdasrvCalcRates(h)
                gv.append(v)
                gf.append(f)
                gr.append(rt)
            self.gVals.append(gv)
            self.gFreqs.append(gf)
            self.gRates.append(gr)
            pf.p4_setPInvarVal(self.cModel, pNum, sp.pInvar)
            pf.p4_setRelRateVal(self.cModel, pNum, sp.relRate)
        # tree
        self.preOrder = tree.preOrder.astype(numpy.int32).copy()
        self.postOrder = tree.postOrder.astype(numpy.int32).copy()
        self.partLikes = numpy.zeros(self.nParts, numpy.double)
        self.cTree = pf.p4_newTree(tree.nNodes, tree.nLeaves, self.preOrder, self.postOrder,
                                   var._newtAndBrentPowellOptPassLimit, self.partLikes,
                                   self.cData, self.cModel)
        self.cNodes = [pf.p4_newNode(v, self.cTree, int(tree.seqNum[v]), int(tree.isLeaf[v]), 1)
                       for v in range(tree.nNodes)]
        self.setTopology(tree)
        self.setBrLens(tree.brLen)
        for pNum, sp in enumerate(problem.parts):
            for v in range(tree.nNodes):
                pf.p4_setCompNum(self.cNodes[v], pNum, int(sp.compNums[v]))
                if v != tree.root:
                    pf.p4_setRMatrixNum(self.cNodes[v], pNum, int(sp.rMatrixNums[v]))
                    pf.p4_setGdasrvNum(self.cNodes[v], pNum, int(sp.gdasrvNums[v]))

    def setTopology(self, tree):
        for v in range(tree.nNodes):
            pf.p4_setNodeRelation(self.cNodes[v], 0, int(tree.parent[v]))
            pf.p4_setNodeRelation(self.cNodes[v], 1, int(tree.leftChild[v]))
            pf.p4_setNodeRelation(self.cNodes[v], 2, int(tree.sibling[v]))
        pf.p4_setTreeRoot(self.cTree, self.cNodes[tree.root])

    def setBrLens(self, brLen):
        root = self.problem.tree.root
        for v, L in enumerate(brLen):
            if v != root:
                pf.p4_setBrLen(self.cNodes[v], float(L))

    def setPrams(self, pNum=-1):
        pf.p4_setPrams(self.cTree, pNum)

    def logLike(self, getSiteLikes=0):
        return pf.p4_treeLogLike(self.cTree, getSiteLikes)

    def calcLogLike(self):
        self.setPrams(-1)
        return self.logLike(0)

    def nPatterns(self, pNum=0):
        return pf.partPatternCount(self.cParts[pNum])

    # ---- vectorised state setters (one call each)
    def setTopologyArrays(self, parent, leftChild, sibling, root):
        pf.setTopology(self.cTree, numpy.ascontiguousarray(parent, numpy.int32),
                       numpy.ascontiguousarray(leftChild, numpy.int32),
                       numpy.ascontiguousarray(sibling, numpy.int32), int(root))

    def setBrLensFast(self, brLen):
        pf.setBrLens(self.cTree, numpy.ascontiguousarray(brLen, numpy.double))

    def setComp(self, pNum, cNum, val):
        self.compVals[pNum][cNum][:] = val

    def setRMatrix(self, pNum, rNum, upper):
        pf.setRMatrixUpper(self.cModel, pNum, rNum, numpy.ascontiguousarray(upper, numpy.double))

    def setGamma(self, pNum, gNum, alpha):
        self.gVals[pNum][gNum][0] = alpha

    def setPInvar(self, pNum, val):
        pf.p4_setPInvarVal(self.cModel, pNum, val)

    def setRelRate(self, pNum, val):
        pf.p4_setRelRateVal(self.cModel, pNum, val)

    def setCompNums(self, pNum, compNums):
        for v, c in enumerate(compNums):
            pf.p4_setCompNum(self.cNodes[v], pNum, int(c))

    # ---- draws (Pf/p4_treeSim.c)
    def ancestralStateDraw(self, seed=0, uniforms=None):
        """Tree.ancestralStateDraw (p4/tree.py:9640-9670): one draw of the
        root's states (or invariant states) from their posterior, every part
        in turn, as one string of symbols.  uniforms: per part, the sites'
        random numbers (None: the Philox stream of seed)."""
        out = []
        for pNum, sp in enumerate(self.problem.parts):
            u = None if uniforms is None else uniforms[pNum]
            d = pf.drawAncStates(self.cTree, pNum, sp.nChar, u, seed)
            st = numpy.where(d[:, 1] >= 0, d[:, 0], d[:, 3])
            out.append("".join(sp.symbols[s] for s in st))
        return "".join(out)

    def simulate(self, seed=0, uniforms=None, calculatePatterns=True, refTree=None, refSeed=0, refUniforms=None):
        """Tree.simulate (p4/tree.py:9527-9636): new sequences for every part
        of the data, drawn down the tree; with calculatePatterns the parts are
        compressed again (makePatterns + setGlobalInvarSitesVec).  refTree
        (another Engine on the same tree shape and model, with data): the
        root's states and categories are drawn from refTree's root posterior
        given its data (refUniforms / refSeed), as p4's refTree mode.
        Returns the new sequences, per part a list of nTax strings."""
        if refTree is None:
            pf.simulate(self.cTree, seed, uniforms)
        else:
            pf.simulateRef(self.cTree, refTree.cTree, seed, uniforms, refSeed, refUniforms)
        seqs = []
        nTax = self.problem.tree.nLeaves
        for pNum, sp in enumerate(self.problem.parts):
            if calculatePatterns:
                pf.makePatterns(self.cParts[pNum])
                pf.setGlobalInvarSitesVec(self.cParts[pNum])
            s = pf.symbolSequences(self.cParts[pNum], nTax, sp.nChar)
            seqs.append([s[i * sp.nChar:(i + 1) * sp.nChar] for i in range(nTax)])
        return seqs

    # ---- ML branch lengths (Pf/p4_treeNewt.c)
    def optLogLike(self):
        """Tree.optLogLike(method="newtAndBrentPowell") (p4/tree.py:9467-9490):
        Newton on the branch lengths alternating with a search over the
        model's free parameters, a final lnL, the new branch lengths back
        into the problem's tree (the comps and gamma shapes the optimiser
        moved are in compVals / gVals, which the library aliases)."""
        pf.p4_newtSetup(self.cTree)
        pf.p4_newtAndBrentPowellOpt(self.cTree)
        lnl = self.calcLogLike()
        bl = pf.p4_getBrLens(self.cTree, self.problem.tree.nNodes)
        self.problem.tree.brLen[:] = bl
        return lnl

    def free(self):
        pf.p4_freeTree(self.cTree)
        pf.p4_freeModel(self.cModel)
        if self.ownsData:
            for cp in self.cParts:
                pf.freePart(cp)
            pf.freeData(self.cData)
