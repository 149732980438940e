"""Drop-in stand-in for the likelihood-path functions of p4's ``p4.pf``.

Same function names, argument order and meaning as the reference's CPython
extension (Pf/pfmodule.c, method table Pf/pfmodule.c:2873-3018); handles are
Python ints as there.  numpy buffers that the reference aliases (comp
values, gdasrv val/freqs/rates, pre/postOrder, partLikes, bounds) are
aliased here too: this module keeps a reference to each array for as long
as the C object that points at it lives.  Errors raise P4Error instead of
the reference's exit(1).
"""
import ctypes

import numpy

from . import _lib
from ._lib import check, dptr, handle, iptr
from .p4exceptions import P4Error

_keep = {}   # handle -> list of arrays the C side aliases


def _L():
    return _lib.load()


def _hold(h, *arrays):
    _keep.setdefault(h, []).extend(arrays)


def _b(s):
    return s.encode() if isinstance(s, str) else s


def _require(a, dtype, name):
    if not isinstance(a, numpy.ndarray) or a.dtype != dtype or not a.flags.c_contiguous:
        raise TypeError("%s must be a C-contiguous numpy %s array" % (name, numpy.dtype(dtype)))
    return a


# ------------------------------------------------------------------- data
def newData(nTax, nParts):
    return handle(_L().p4g_newData(nTax, nParts), "newData")


def freeData(cData):
    check(_L().p4g_freeData(cData), "freeData")


def pokePartInData(cPart, cData, partNum):
    check(_L().p4g_pokePartInData(cPart, cData, partNum), "pokePartInData")


def newPart(nTax, nChar, equateSymbols, nEquates, symbols, dim):
    return handle(_L().p4g_newPart(nTax, nChar, _b(equateSymbols), nEquates, _b(symbols), dim),
                  "newPart")


def freePart(cPart):
    check(_L().p4g_freePart(cPart), "freePart")


def pokeEquatesTable(cPart, table):
    check(_L().p4g_pokeEquatesTable(cPart, _b(table)), "pokeEquatesTable")


def pokeSequences(cPart, seqs):
    check(_L().p4g_pokeSequences(cPart, _b(seqs)), "pokeSequences")


def makePatterns(cPart):
    check(_L().p4g_makePatterns(cPart), "makePatterns")


def getSiteRates(cTree, cPart, pNum, nChar):
    """Per-site posterior mean rates and most likely Gamma categories
    (pf.getSiteRates, Pf/p4_tree.c:1383-1627)."""
    rates = numpy.zeros(nChar, numpy.double)
    cats = numpy.zeros(nChar, numpy.int32)
    check(_L().p4g_getSiteRates(cTree, cPart, int(pNum), dptr(rates), iptr(cats)), "getSiteRates")
    return rates, cats


def p4_newtSetup(cTree):
    """pf.p4_newtSetup (Pf/pfmodule.c:2274, Pf/p4_treeNewt.c:11)."""
    check(_L().p4g_newtSetup(cTree), "p4_newtSetup")


def p4_newtAround(cTree, epsilon, likeDelta):
    """p4_newtAround (Pf/p4_treeNewt.c:79): Newton on every branch length,
    rounds until the lnL changes by less than likeDelta."""
    check(_L().p4g_newtAround(cTree, float(epsilon), float(likeDelta)), "p4_newtAround")


def p4_newtAndBrentPowellOpt(cTree):
    """pf.p4_newtAndBrentPowellOpt (Pf/pfmodule.c:2259, Pf/p4_treeOpt.c:1182):
    branch lengths by Newton alternating with a Powell search over the
    model's free parameters, FP64 on the GPU."""
    check(_L().p4g_newtAndBrentPowellOpt(cTree), "p4_newtAndBrentPowellOpt")


def p4_getFreePrams(cTree, cap=4096):
    """pf.p4_getFreePrams (Pf/pfmodule.c:2304): the free parameters in
    p4_windUpParameters order, as a list."""
    out = numpy.zeros(cap, numpy.double)
    n = ctypes.c_int(0)
    check(_L().p4g_getFreePrams(cTree, dptr(out), cap, ctypes.byref(n)), "p4_getFreePrams")
    return [float(x) for x in out[:n.value]]


def p4_getBrLens(cTree, nNodes):
    """pf.p4_getBrLens (Pf/pfmodule.c:2289): every node's branch length."""
    out = numpy.zeros(nNodes, numpy.double)
    check(_L().p4g_getBrLens(cTree, dptr(out)), "p4_getBrLens")
    return out


def symbolSequences(cPart, nTax, nChar):
    """pf.symbolSequences (Pf/part.c:604): the part's sequences, one string."""
    buf = ctypes.create_string_buffer(nTax * nChar + 1)
    check(_L().p4g_symbolSequences(cPart, buf), "symbolSequences")
    return buf.value.decode("ascii")


def drawAncStates(cTree, pNum, nChar, uniforms=None, seed=0):
    """pf.p4_drawAncState for every site of part pNum (Pf/p4_treeSim.c:591-857):
    an nChar x 4 int array of (chState, cat, isInvar, invarState).  uniforms:
    the sites' random numbers in [0, 1), or None for the Philox stream of
    seed."""
    draws = numpy.zeros((nChar, 4), numpy.int32)
    u = None
    if uniforms is not None:
        u = numpy.ascontiguousarray(uniforms, numpy.double)
        if u.shape != (nChar,):
            raise P4Error("drawAncStates: %d uniforms for %d sites" % (u.size, nChar))
    check(_L().p4g_drawAncStates(cTree, int(pNum), dptr(u) if u is not None else None,
                                 int(seed) & 0xffffffffffffffff, iptr(draws)), "drawAncStates")
    return draws


def simulate(cTree, seed=0, uniforms=None, nStates=0):
    """pf.p4_simulate(cTree, 0, rng) (Pf/p4_treeSim.c:14-590): new sequences
    for every part of the tree's data.  uniforms: the random numbers in the
    reference's draw order, or None for the Philox stream of seed.  With
    nStates (sum over parts of nNodes * nChar) the states of every node are
    returned as an int8 array (parts concatenated, node-major)."""
    u = None
    if uniforms is not None:
        u = numpy.ascontiguousarray(uniforms, numpy.double)
    states = numpy.zeros(max(int(nStates), 1), numpy.int8) if nStates else None
    check(_L().p4g_simulate(cTree, dptr(u) if u is not None else None, int(u.size) if u is not None else 0,
                            int(seed) & 0xffffffffffffffff,
                            states.ctypes.data if states is not None else None), "simulate")
    return states


def simulateRef(cTree, refTree, seed=0, uniforms=None, refSeed=0, refUniforms=None, nStates=0):
    """pf.p4_simulate(cTree, refTree, rng) (Pf/p4_treeSim.c:223-284): new
    sequences whose root states and categories are drawn from refTree's root
    posterior (one random number per site, parts in order: refUniforms, or
    the Philox stream of refSeed), mutated down cTree with the mutation
    loop's random numbers (uniforms, or the Philox stream of seed)."""
    u = None if uniforms is None else numpy.ascontiguousarray(uniforms, numpy.double)
    ru = None if refUniforms is None else numpy.ascontiguousarray(refUniforms, numpy.double)
    states = numpy.zeros(max(int(nStates), 1), numpy.int8) if nStates else None
    check(_L().p4g_simulateRef(cTree, refTree, dptr(ru) if ru is not None else None,
                               int(refSeed) & 0xffffffffffffffff, dptr(u) if u is not None else None,
                               int(u.size) if u is not None else 0, int(seed) & 0xffffffffffffffff,
                               states.ctypes.data if states is not None else None), "simulateRef")
    return states


def makePatternsDevice(cPart):
    """makePatterns computed on the GPU (identical output)."""
    check(_L().p4g_makePatternsDevice(cPart), "makePatternsDevice")


def setGlobalInvarSitesVec(cPart):
    check(_L().p4g_setGlobalInvarSitesVec(cPart), "setGlobalInvarSitesVec")


def partPatternCount(cPart):
    n = ctypes.c_int(0)
    check(_L().p4g_partPatternCount(cPart, ctypes.byref(n)), "partPatternCount")
    return n.value


def getSiteLikes(cPart, nChar):
    out = numpy.zeros(nChar, numpy.double)
    check(_L().p4g_getSiteLikes(cPart, dptr(out)), "getSiteLikes")
    return out


# ------------------------------------------------------------------- model
def p4_newModel(nParts, doRelRates, relRatesAreFree, nFreePrams, isHet, rMatrixNormalizeTo1,
                *bounds):
    if len(bounds) != 14:
        raise TypeError("p4_newModel needs the 14 bound arrays of var.py")
    _require(rMatrixNormalizeTo1, numpy.int32, "rMatrixNormalizeTo1")
    for b in bounds:
        _require(b, numpy.double, "bound")
    h = handle(_L().p4g_newModel(nParts, doRelRates, relRatesAreFree, int(nFreePrams), isHet,
                                 iptr(rMatrixNormalizeTo1), *[dptr(b) for b in bounds]),
               "p4_newModel")
    _hold(h, rMatrixNormalizeTo1, *bounds)
    return h


def p4_freeModel(cModel):
    check(_L().p4g_freeModel(cModel), "p4_freeModel")
    _keep.pop(cModel, None)


def p4_newModelPart(cModel, pNum, dim, nComps, nRMatrices, nGdasrvs, nCat, pInvarFree,
                    bQETneedsReset):
    _require(bQETneedsReset, numpy.int32, "bQETneedsReset")
    check(_L().p4g_newModelPart(cModel, pNum, dim, nComps, nRMatrices, nGdasrvs, nCat, pInvarFree,
                                iptr(bQETneedsReset)), "p4_newModelPart")
    _hold(cModel, bQETneedsReset)


def p4_newComp(cModel, pNum, mNum, free, val):
    _require(val, numpy.double, "comp val")
    check(_L().p4g_newComp(cModel, pNum, mNum, free, dptr(val)), "p4_newComp")
    _hold(cModel, val)


# spec names -> numbers as Model.allocCStuff maps them (p4/model.py:790-806)
RMATRIX_SPEC = {"ones": 100, "specified": 20, "optimized": 20, "2p": 5}


def p4_newRMatrix(cModel, pNum, mNum, free, spec):
    check(_L().p4g_newRMatrix(cModel, pNum, mNum, free, spec), "p4_newRMatrix")


def getBigR(spec, a):
    """pf.getBigR(specNum, a) (Pf/pfmodule.c:1271): fill the 20x20 float64
    array a with the exchangeabilities of an empirical protein spec."""
    if a.shape != (20, 20) or a.dtype != numpy.double or not a.flags.c_contiguous:
        raise P4Error("getBigR: a must be a C-contiguous 20x20 float64 array")
    check(_L().p4g_getBigR(int(spec), dptr(a)), "getBigR")


def p4_newGdasrv(cModel, pNum, mNum, nCat, free, val, freqs, rates):
    for a, n in ((val, "val"), (freqs, "freqs"), (rates, "rates")):
        _require(a, numpy.double, "gdasrv " + n)
    h = handle(_L().p4g_newGdasrv(cModel, pNum, mNum, nCat, free, dptr(val), dptr(freqs),
                                  dptr(rates)), "p4_newGdasrv")
    _hold(cModel, val, freqs, rates)
    return h


def gdasrvCalcRates(cGdasrv):
    check(_L().p4g_gdasrvCalcRates(cGdasrv), "gdasrvCalcRates")


def gdasrvCalcRates_np(nCat, val, freqs, rates):
    check(_L().p4g_gdasrvCalcRates_np(nCat, float(val), dptr(freqs), dptr(rates)),
          "gdasrvCalcRates_np")


def p4_setRMatrixBigR(cModel, pNum, rNum, i, j, val):
    check(_L().p4g_setRMatrixBigR(cModel, pNum, rNum, i, j, float(val)), "p4_setRMatrixBigR")


def p4_setKappa(cModel, pNum, rNum, val):
    check(_L().p4g_setKappa(cModel, pNum, rNum, float(val)), "p4_setKappa")


def p4_setPInvarVal(cModel, pNum, val):
    check(_L().p4g_setPInvarVal(cModel, pNum, float(numpy.asarray(val).reshape(-1)[0])),
          "p4_setPInvarVal")


def p4_setRelRateVal(cModel, pNum, val):
    check(_L().p4g_setRelRateVal(cModel, pNum, float(numpy.asarray(val).reshape(-1)[0])),
          "p4_setRelRateVal")


# ------------------------------------------------------------------- tree
def p4_newTree(nNodes, nLeaves, preOrder, postOrder, passLimit, partLikes, cData, cModel):
    _require(preOrder, numpy.int32, "preOrder")
    _require(postOrder, numpy.int32, "postOrder")
    _require(partLikes, numpy.double, "partLikes")
    pl = iptr(passLimit) if isinstance(passLimit, numpy.ndarray) else None
    h = handle(_L().p4g_newTree(nNodes, nLeaves, iptr(preOrder), iptr(postOrder), pl,
                                dptr(partLikes), cData, cModel), "p4_newTree")
    _hold(h, preOrder, postOrder, partLikes, passLimit)
    return h


def p4_freeTree(cTree):
    check(_L().p4g_freeTree(cTree), "p4_freeTree")
    _keep.pop(cTree, None)


def p4_newNode(nodeNum, cTree, seqNum, isLeaf, inTree):
    return handle(_L().p4g_newNode(nodeNum, cTree, seqNum, isLeaf, inTree), "p4_newNode")


def p4_setNodeRelation(cNode, relation, relNum):
    check(_L().p4g_setNodeRelation(cNode, relation, relNum), "p4_setNodeRelation")


def p4_setTreeRoot(cTree, cNode):
    check(_L().p4g_setTreeRoot(cTree, cNode), "p4_setTreeRoot")


def p4_setBrLen(cNode, brLen):
    check(_L().p4g_setBrLen(cNode, float(brLen)), "p4_setBrLen")


def p4_setCompNum(cNode, pNum, num):
    check(_L().p4g_setCompNum(cNode, pNum, num), "p4_setCompNum")


def p4_setRMatrixNum(cNode, pNum, num):
    check(_L().p4g_setRMatrixNum(cNode, pNum, num), "p4_setRMatrixNum")


def p4_setGdasrvNum(cNode, pNum, num):
    check(_L().p4g_setGdasrvNum(cNode, pNum, num), "p4_setGdasrvNum")


def p4_setPrams(cTree, pNum):
    check(_L().p4g_setPrams(cTree, pNum), "p4_setPrams")


def p4_treeLogLike(cTree, getSiteLikes):
    out = ctypes.c_double(0.0)
    check(_L().p4g_treeLogLike(cTree, int(getSiteLikes), ctypes.byref(out)), "p4_treeLogLike")
    return out.value


def p4_partLogLike(cTree, cPart, pNum, getSiteLikes):
    out = ctypes.c_double(0.0)
    check(_L().p4g_partLogLike(cTree, cPart, pNum, int(getSiteLikes), ctypes.byref(out)),
          "p4_partLogLike")
    return out.value


def p4_calculateBigPDecks(cNode):
    check(_L().p4g_calculateBigPDecks(cNode), "p4_calculateBigPDecks")


def p4_calculateAllBigPDecksAllParts(cTree):
    check(_L().p4g_calculateAllBigPDecksAllParts(cTree), "p4_calculateAllBigPDecksAllParts")


def p4_copyCondLikes(a, b, doAll):
    check(_L().p4g_copyCondLikes(a, b, doAll), "p4_copyCondLikes")


def p4_copyBigPDecks(a, b, doAll):
    check(_L().p4g_copyBigPDecks(a, b, doAll), "p4_copyBigPDecks")


def p4_copyModelPrams(a, b):
    check(_L().p4g_copyModelPrams(a, b), "p4_copyModelPrams")


# --------------------------------------------------------- batched / extras
def treeLogLikeBatch(cTrees, doSetPrams=1):
    n = len(cTrees)
    arr = (ctypes.c_void_p * n)(*cTrees)
    out = numpy.zeros(n, numpy.double)
    check(_L().p4g_treeLogLikeBatch(arr, n, int(doSetPrams), dptr(out)), "treeLogLikeBatch")
    return out


def setPrecision(cTree, mode):
    """0 = fused FP32 pruning (default), 1 = plain FP64 per-node path."""
    check(_L().p4g_setPrecision(cTree, int(mode)), "setPrecision")


def setBrLens(cTree, brLens):
    _require(brLens, numpy.double, "brLens")
    check(_L().p4g_setBrLens(cTree, dptr(brLens)), "setBrLens")


class Batch(object):
    """Several trees evaluated with one launch sequence (a CUDA graph after
    the first call); the chains of an MCMCMC."""

    def __init__(self, cTrees, graph=True, clades=False):
        n = len(cTrees)
        self.n = n
        self._arr = (ctypes.c_void_p * n)(*cTrees)
        self.h = handle(_L().p4g_newBatch(self._arr, n), "newBatch")
        check(_L().p4g_batchSetGraph(self.h, int(graph)), "batchSetGraph")
        if clades:   # clade tables: for trees whose topologies stay fixed
            check(_L().p4g_batchSetClades(self.h, 1), "batchSetClades")
        self.out = numpy.zeros(n, numpy.double)

    def logLike(self):
        check(_L().p4g_batchLogLike(self.h, dptr(self.out)), "batchLogLike")
        return self.out.copy()

    def free(self):
        if self.h:
            _L().p4g_freeBatch(self.h)
            self.h = None


def setAutotune(on):
    check(_L().p4g_setAutotune(int(on)), "setAutotune")


def getPruneShape(cTree, group=0):
    sh, tile = ctypes.c_int(0), ctypes.c_int(0)
    check(_L().p4g_getPruneShape(cTree, group, ctypes.byref(sh), ctypes.byref(tile)), "getPruneShape")
    return sh.value, tile.value


def setPruneShape(cTree, group, shape):
    check(_L().p4g_setPruneShape(cTree, int(group), int(shape)), "setPruneShape")


def setGraphs(cTree, on):
    """Replay the tree's launch sequences from CUDA graphs (default on)."""
    check(_L().p4g_setGraphs(cTree, int(on)), "setGraphs")


def setCladeShape(cTree, group, shape):
    """Tile shape of a pruning group's clade-table launches."""
    check(_L().p4g_setCladeShape(cTree, int(group), int(shape)), "setCladeShape")


def setCladeSize(cTree, maxLeaves):
    check(_L().p4g_setCladeSize(cTree, int(maxLeaves)), "setCladeSize")


def setTopology(cTree, parent, leftChild, sibling, root):
    for a, n in ((parent, "parent"), (leftChild, "leftChild"), (sibling, "sibling")):
        _require(a, numpy.int32, n)
    check(_L().p4g_setTopology(cTree, iptr(parent), iptr(leftChild), iptr(sibling), int(root)),
          "setTopology")


def setRMatrixUpper(cModel, pNum, rNum, vals):
    _require(vals, numpy.double, "rMatrix values")
    check(_L().p4g_setRMatrixUpper(cModel, pNum, rNum, dptr(vals)), "setRMatrixUpper")


def treeLogLikeAsync(cTree, doSetPrams=1):
    check(_L().p4g_treeLogLikeAsync(cTree, int(doSetPrams)), "treeLogLikeAsync")


def treeLogLikeWait(cTree):
    out = ctypes.c_double(0.0)
    check(_L().p4g_treeLogLikeWait(cTree, ctypes.byref(out)), "treeLogLikeWait")
    return out.value


def treeInfo(cTree):
    info = (ctypes.c_longlong * 7)()
    check(_L().p4g_treeInfo(cTree, info), "treeInfo")
    keys = ("h2dBytes", "launches", "nPatterns", "nSlots", "nProg", "d2hBytes", "nClade")
    return dict(zip(keys, [int(x) for x in info]))


def setProgrammaticLaunch(on):
    """Programmatic dependent launch of the P-deck and pruning kernels (default on)."""
    check(_L().p4g_setProgrammaticLaunch(int(bool(on))), "setProgrammaticLaunch")


def treeDeviceBytes(cTree):
    """(bytes of the tree's own device state, bytes of its data's device
    copies), as allocated so far; allocates nothing."""
    tb, db = ctypes.c_longlong(0), ctypes.c_longlong(0)
    check(_L().p4g_treeDeviceBytes(cTree, ctypes.byref(tb), ctypes.byref(db)), "treeDeviceBytes")
    return tb.value, db.value


def fp32FmaPeak(iters=20000):
    """Measured FP32 FMA throughput: (TFLOP/s, ms of the timed launch)."""
    tf, ms = ctypes.c_double(0.0), ctypes.c_double(0.0)
    check(_L().p4g_fp32FmaPeak(int(iters), ctypes.byref(tf), ctypes.byref(ms)), "fp32FmaPeak")
    return tf.value, ms.value


def getPDeck(cNode, pNum, cat, dim):
    out = numpy.zeros((dim, dim), numpy.double)
    check(_L().p4g_getPDeck(cNode, pNum, cat, dptr(out)), "getPDeck")
    return out


def getDecks32(cTree, pNum, nNodes, nCat, dim, maxPartial=64):
    decks = numpy.zeros((nNodes, nCat, dim, dim), numpy.float32)
    eq = numpy.zeros((nNodes, maxPartial, nCat, dim), numpy.float32)
    npart = ctypes.c_int(0)
    check(_L().p4g_getDecks32(cTree, pNum, _lib.fptr(decks), _lib.fptr(eq), ctypes.byref(npart)),
          "getDecks32")
    k = npart.value
    flat = eq.reshape(-1)[: nNodes * k * nCat * dim].reshape(nNodes, k, nCat, dim).copy()
    return decks, flat


def getCompactCodes(cPart, nTax, nPatterns, maxPartial=64):
    codes = numpy.zeros((nTax, nPatterns), numpy.uint8)
    masks = numpy.zeros(maxPartial, numpy.uint32)
    check(_L().p4g_getCompactCodes(cPart, _lib.ucptr(codes), _lib.uptr(masks)), "getCompactCodes")
    return codes, masks


def getPatternLikes(cTree, pNum, nPatterns):
    like = numpy.zeros(nPatterns, numpy.float32)
    exps = numpy.zeros(nPatterns, numpy.int32)
    lnl = numpy.zeros(nPatterns, numpy.double)
    check(_L().p4g_getPatternLikes(cTree, pNum, _lib.fptr(like), iptr(exps), dptr(lnl)),
          "getPatternLikes")
    return like, exps, lnl


def getGammaRates(cTree, pNum, gNum, nCat):
    out = numpy.zeros(nCat, numpy.double)
    check(_L().p4g_getGammaRates(cTree, pNum, gNum, dptr(out)), "getGammaRates")
    return out


def getPatterns(cPart, nTax, nChar):
    n = partPatternCount(cPart)
    pats = numpy.zeros((nTax, n), numpy.int32)
    counts = numpy.zeros(n, numpy.int32)
    spi = numpy.zeros(nChar, numpy.int32)
    check(_L().p4g_getPatterns(cPart, iptr(pats), iptr(counts), iptr(spi)), "getPatterns")
    return pats, counts, spi


def getInvarSites(cPart, dim, nPatterns):
    vec = numpy.zeros(nPatterns, numpy.int32)
    arr = numpy.zeros((dim, nPatterns), numpy.int32)
    check(_L().p4g_getInvarSites(cPart, iptr(vec), iptr(arr)), "getInvarSites")
    return vec, arr


def getStream():
    return _L().p4g_getStream()
