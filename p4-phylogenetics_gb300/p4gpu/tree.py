"""p4's Tree with its Data and Model attached, as the MCMC and the likelihood
entry take them.

In p4 a Tree (p4/tree.py) carries `data` (p4/data.py: alignment parts) and
`model` (p4/model.py: per part the compositions, rate matrices, discrete-gamma
shapes, pInvar, relative rate and which of them each node uses), and
Tree.calcLogLike (p4/tree.py:9406) pushes both through pf into the C core;
Mcmc(aTree, ...) (p4/mcmc.py:672) runs on such a tree.  These classes hold the
same information in the form the GPU library's pf calls take; the data can be
detached and re-attached (checkpoints store the tree and model, never the
alignment, as p4's do).

Node numbering, relations and branch lengths are p4's: parent / leftChild /
sibling per node, the length on the node at the branch's lower end, leaves
numbered by their taxon (seqNum).
"""
import numpy

from . import sim
from .p4exceptions import P4Error


class DataPart(object):
    """One alignment part: data type, symbols, equates, one sequence per taxon."""

    def __init__(self, dataType, sequences, equates=None):
        if dataType not in ("dna", "protein"):
            raise P4Error("data type %r is not supported (dna or protein)" % dataType)
        self.dataType = dataType
        self.sequences = list(sequences)
        self.equates = (dict(sim.DNA_EQUATES if dataType == "dna" else sim.PROTEIN_EQUATES)
                        if equates is None else dict(equates))

    @property
    def dim(self):
        return 4 if self.dataType == "dna" else 20

    @property
    def nChar(self):
        return len(self.sequences[0])


class Data(object):
    """The alignment parts of a Tree (p4/data.py: Data.parts, nParts, nTax)."""

    def __init__(self, parts, taxNames=None):
        self.parts = list(parts)
        nTax = len(self.parts[0].sequences)
        if any(len(p.sequences) != nTax for p in self.parts):
            raise P4Error("every data part needs one sequence per taxon")
        self.taxNames = list(taxNames) if taxNames is not None else ["t%d" % i for i in range(nTax)]

    @property
    def nParts(self):
        return len(self.parts)

    @property
    def nTax(self):
        return len(self.parts[0].sequences)


class ModelPart(object):
    """Model of one part (p4/model.py ModelPart): comps [nComps][dim], R
    matrices [nR][dim][dim] (symmetric), gamma shapes [nGdasrvs], nCat,
    pInvar (and whether it is free), relRate, and per node the comp, rMatrix
    and gdasrv numbers."""

    def __init__(self, dim, comps, rMatrices, gammaShapes, nCat, compNums, rMatrixNums, gdasrvNums,
                 pInvar=0.0, pInvarFree=None, relRate=1.0):
        self.dim = int(dim)
        self.comps = numpy.array(comps, numpy.double, ndmin=2)
        self.rMatrices = numpy.array(rMatrices, numpy.double, ndmin=3)
        self.gammaShapes = numpy.array(gammaShapes, numpy.double).reshape(-1)
        self.nCat = int(nCat)
        self.compNums = numpy.array(compNums, numpy.int32)
        self.rMatrixNums = numpy.array(rMatrixNums, numpy.int32)
        self.gdasrvNums = numpy.array(gdasrvNums, numpy.int32)
        self.pInvar = float(pInvar)
        self.pInvarFree = (self.pInvar > 0.0) if pInvarFree is None else bool(pInvarFree)
        self.relRate = float(relRate)

    @property
    def nComps(self):
        return self.comps.shape[0]

    @property
    def nRMatrices(self):
        return self.rMatrices.shape[0]

    @property
    def nGdasrvs(self):
        return len(self.gammaShapes)


class Model(object):
    """The model parts of a Tree (p4/model.py: Model.parts, nParts, isHet)."""

    def __init__(self, parts, relRatesAreFree=False):
        self.parts = list(parts)
        self.relRatesAreFree = bool(relRatesAreFree)

    @property
    def nParts(self):
        return len(self.parts)

    @property
    def isHet(self):
        return any(mp.nComps > 1 or mp.nRMatrices > 1 or mp.nGdasrvs > 1 for mp in self.parts)


class Tree(object):
    """A tree (topology, branch lengths, taxon names) with data and model."""

    def __init__(self, spec, taxNames=None, data=None, model=None, name=None):
        self.spec = spec
        self.taxNames = list(taxNames) if taxNames is not None else ["t%d" % i for i in range(spec.nLeaves)]
        if len(self.taxNames) != spec.nLeaves:
            raise P4Error("%d taxon names for %d leaves" % (len(self.taxNames), spec.nLeaves))
        self.data = data
        self.model = model
        self.name = name
        self.logLike = None

    # ------------------------------------------------------------ builders
    @classmethod
    def fromProblem(cls, problem, taxNames=None):
        """A Tree, Data and Model holding a synthetic Problem's values."""
        spec = problem.tree
        data = Data([DataPart(sp.dataType, sp.sequences, sp.equates) for sp in problem.parts], taxNames)
        mparts = [ModelPart(sp.dim, sp.comps, sp.rmats, sp.gammaShapes, sp.nCat, sp.compNums, sp.rMatrixNums,
                            sp.gdasrvNums, sp.pInvar, None, sp.relRate) for sp in problem.parts]
        return cls(spec.copy(), data.taxNames, data, Model(mparts), getattr(problem, "name", None))

    def toProblem(self):
        """The same tree, data and model as one synthetic-problem object, the
        form the library engine (p4gpu.engine.Engine) pushes through pf."""
        if self.data is None or self.model is None:
            raise P4Error("the tree needs a model and data attached")
        if self.data.nParts != self.model.nParts:
            raise P4Error("data has %d parts, model %d" % (self.data.nParts, self.model.nParts))
        if self.data.nTax != self.spec.nLeaves:
            raise P4Error("data has %d taxa, the tree %d leaves" % (self.data.nTax, self.spec.nLeaves))
        parts = []
        for dp, mp in zip(self.data.parts, self.model.parts):
            if dp.dim != mp.dim:
                raise P4Error("data part dim %d, model part dim %d" % (dp.dim, mp.dim))
            parts.append(sim.PartSpec(dp.dataType, dp.sequences, mp.comps, mp.rMatrices, mp.gammaShapes, mp.nCat,
                                      mp.compNums, mp.rMatrixNums, mp.gdasrvNums, mp.pInvar, mp.relRate,
                                      dp.equates))
        return sim.Problem(self.spec, parts, self.name or "tree")

    # ------------------------------------------------------------ queries
    @property
    def nTax(self):
        return self.spec.nLeaves

    @property
    def nNodes(self):
        return self.spec.nNodes

    @property
    def root(self):
        return self.spec.root

    def calcLogLike(self, verbose=False):
        """Tree.calcLogLike (p4/tree.py:9406-9414): push the tree, data and
        model through pf (p4_setPrams + p4_treeLogLike on the GPU library);
        sets and returns self.logLike."""
        from .engine import Engine
        e = Engine(self.toProblem())
        try:
            self.logLike = e.calcLogLike()
        finally:
            e.free()
        if verbose:
            print("Tree.calcLogLike. %f" % self.logLike)
        return self.logLike

    def writeNewick(self, flob, translationHash=None, doMcmcCommandComments=False, brLen=None, parent=None,
                    leftChild=None, sibling=None, root=None):
        """Newick of the tree (or of the given topology arrays and branch
        lengths) as p4's Tree.writeNewick writes it (p4/tree.py:6276-6402):
        taxa by translation number when a translationHash is given, ', '
        between siblings, ':%g' branch lengths (unless every one is 0.1), with
        doMcmcCommandComments the per-node model numbers ' [& c0.1 r0.0 g0.0]'
        of the parts with more than one comp / rMatrix / gdasrv
        (p4/tree.py:6404-6433), terminated by ';' and a newline."""
        par = self.spec.parent if parent is None else parent
        lc = self.spec.leftChild if leftChild is None else leftChild
        sib = self.spec.sibling if sibling is None else sibling
        rt = self.spec.root if root is None else root
        bl = self.spec.brLen if brLen is None else brLen
        isLeaf = self.spec.isLeaf
        seqNum = self.spec.seqNum
        writeBrLens = any(bl[v] != 0.1 for v in range(len(par)) if v != rt)

        def label(v):
            name = self.taxNames[int(seqNum[v])]
            return str(translationHash[name]) if translationHash else name

        def comment(v):
            out = []
            for pNum, mp in enumerate(self.model.parts):
                if mp.nComps > 1:
                    out.append(" c%i.%i" % (pNum, mp.compNums[v]))
                if v != rt:
                    if mp.nRMatrices > 1:
                        out.append(" r%i.%i" % (pNum, mp.rMatrixNums[v]))
                    if mp.nGdasrvs > 1:
                        out.append(" g%i.%i" % (pNum, mp.gdasrvNums[v]))
            return " [&" + "".join(out) + "]" if out else ""

        out = []

        def walk(v):
            kids = []
            c = lc[v]
            while c >= 0:
                kids.append(int(c))
                c = sib[c]
            if kids:
                out.append("(")
                for i, c in enumerate(kids):
                    if i:
                        out.append(", ")
                    walk(c)
                out.append(")")
                if isLeaf[v]:          # a leaf at the root (tree on a stick)
                    out.append(label(v))
            else:
                out.append(label(v))
            if writeBrLens and v != rt:
                out.append(":%g" % bl[v])
            if doMcmcCommandComments:
                out.append(comment(v))

        walk(rt)
        out.append(";\n")
        flob.write("".join(out))
