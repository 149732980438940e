"""Metropolis-coupled MCMC over the GPU likelihood, with p4's semantics.

Reference: Mcmc (p4/mcmc.py: proposal probabilities :110-200, tunings
:48-107, weights _makeProposals :1300-1953, run :2496-3208, swaps
:3299-3421, Proposal.tune :250-284) and Chain (p4/chain.py: gen
:1138-1705 with the heated MH test :1100-1118,1310-1318; proposals
proposeLocal :3199, proposeAllBrLens :3143, proposeBrLen :3091,
proposeETBR_Blaise :4128 (in p4gpu/topology.py), proposeAllCompsDir :2259,
proposeAllRMatricesDir :2291, proposeGdasrv :2051, proposePInvar :2107,
proposeRelRate :2127).

What differs is where time goes.  p4 evaluates chains one after another,
re-prunes changed nodes with one FFI call per node and part, and copies
every conditional-likelihood buffer between its cur and prop trees after
every generation.  Here every chain's proposal of a generation is
evaluated in one batched library call (all chains x all parts on one
stream, one host synchronisation), each evaluation is a full fused pass
(no per-node CL state exists to keep in sync), and accept/reject only
swaps host-side parameter records.
"""
import math

import numpy

from . import pf
from .engine import Engine, make_data
from .p4exceptions import P4Error
from .topology import LinkedTree, propose_etbr
from .var import var

# p4's tuned proposals (Mcmc.tunableProps, p4/mcmc.py:2923-2929); eTBR keeps
# its default lambda (p4/mcmc.py:2931)
TUNABLE = frozenset("allBrLens allCompsDir brLen gdasrv local pInvar allRMatricesDir relRate learned".split())
ETBR_LAMBDA = 2.0 * math.log(1.6)     # p4/mcmc.py:97
ETBR_PEXT = 0.8                       # p4/mcmc.py:98


# --------------------------------------------------------------------- state
class PartState(object):
    __slots__ = ("comps", "rvals", "gamma", "pInvar", "relRate")

    def __init__(self, comps, rvals, gamma, pInvar, relRate):
        self.comps = comps
        self.rvals = rvals
        self.gamma = gamma
        self.pInvar = pInvar
        self.relRate = relRate

    def copy(self):
        return PartState(self.comps.copy(), self.rvals.copy(), self.gamma.copy(), self.pInvar,
                         self.relRate)


class State(object):
    """One chain's parameters: topology arrays, branch lengths, model values."""

    def __init__(self, parent, leftChild, sibling, root, brLen, parts):
        self.parent = parent
        self.leftChild = leftChild
        self.sibling = sibling
        self.root = root
        self.brLen = brLen
        self.parts = parts

    def copy(self):
        return State(self.parent.copy(), self.leftChild.copy(), self.sibling.copy(), self.root,
                     self.brLen.copy(), [p.copy() for p in self.parts])

    def shallow(self):
        """A new State sharing every array and part with this one; a proposal
        copies what it changes first (own_brLen, own_topology, own_part)."""
        return State(self.parent, self.leftChild, self.sibling, self.root, self.brLen, list(self.parts))

    def own_brLen(self):
        self.brLen = self.brLen.copy()

    def own_topology(self):
        self.parent = self.parent.copy()
        self.leftChild = self.leftChild.copy()
        self.sibling = self.sibling.copy()

    def own_part(self, p):
        self.parts[p] = self.parts[p].copy()
        return self.parts[p]

    def children(self, v):
        c = int(self.leftChild[v])
        sib = self.sibling
        while c >= 0:
            yield c
            c = int(sib[c])

    def kids(self):
        """Every node's children in sibling order (lists of ints)."""
        lc, sib = self.leftChild.tolist(), self.sibling.tolist()
        out = []
        for v in range(len(lc)):
            ch = []
            c = lc[v]
            while c >= 0:
                ch.append(c)
                c = sib[c]
            out.append(ch)
        return out

    def set_kids(self, kids):
        n = len(self.parent)
        parent, leftChild, sibling = [-1] * n, [-1] * n, [-1] * n
        for v in range(n):
            ch = kids[v]
            if ch:
                leftChild[v] = ch[0]
                for a, b in zip(ch[:-1], ch[1:]):
                    sibling[a] = b
                for c in ch:
                    parent[c] = v
        self.parent[:] = parent
        self.leftChild[:] = leftChild
        self.sibling[:] = sibling

    def tree_length(self):
        return float(self.brLen.sum() - self.brLen[self.root])


def upper(R):
    d = R.shape[0]
    return numpy.array([R[i, j] for i in range(d - 1) for j in range(i + 1, d)])


try:
    from scipy.special import gammaln as _gammaln
except ImportError:          # the same values from math.lgamma, one at a time
    def _gammaln(a):
        return numpy.array([math.lgamma(float(v)) for v in numpy.ravel(a)])


def dirichlet_lnpdf(alpha, x):
    """ln Dirichlet(x | alpha), the closed form (as gsl_ran_dirichlet_lnpdf):
    term by term in Python floats for short vectors (compositions, DNA rate
    matrices), vectorised for long ones (protein rate matrices)."""
    if len(alpha) <= 32:
        lg, lnx = math.lgamma, math.log
        tot = 0.0
        s = 0.0
        for a, xi in zip(alpha.tolist(), x.tolist()):
            tot += a
            s += (a - 1.0) * lnx(xi) - lg(a)
        return lg(tot) + s
    return (math.lgamma(float(alpha.sum())) - float(_gammaln(alpha).sum())
            + float(((alpha - 1.0) * numpy.log(x)).sum()))


# --------------------------------------------------------------------- proposals
class Proposal(object):
    """A proposal kind with per-temperature tuning and p4's tuner."""

    def __init__(self, name, weight, tuning, nChains, pNum=-1, acc=(0.7, 0.6, 0.1, 0.05),
                 factor=(1.6, 1.2, 0.8, 0.7), tuningLimitHi=None):
        self.name = name
        self.weight = float(weight)
        self.pNum = pNum
        self.tuning = [float(tuning)] * nChains
        self.tnAccVeryHi, self.tnAccHi, self.tnAccLo, self.tnAccVeryLo = acc
        self.tnFactorVeryHi, self.tnFactorHi, self.tnFactorLo, self.tnFactorVeryLo = factor
        self.tuningLimitHi = tuningLimitHi
        self.tnSampleSize = 250
        self.tnNSamples = [0] * nChains
        self.tnNAccepts = [0] * nChains
        self.nProposals = [0] * nChains
        self.nAcceptances = [0] * nChains
        self.nAborts = [0] * nChains
        self.nTopologyChanges = [0] * nChains

    def tune(self, tempNum):
        """p4/mcmc.py:250-284."""
        acc = self.tnNAccepts[tempNum] / float(self.tnNSamples[tempNum])
        changed = False
        if acc > self.tnAccHi:
            self.tuning[tempNum] *= self.tnFactorVeryHi if acc > self.tnAccVeryHi else self.tnFactorHi
            changed = True
        elif acc < self.tnAccLo:
            self.tuning[tempNum] *= self.tnFactorVeryLo if acc < self.tnAccVeryLo else self.tnFactorLo
            changed = True
        if changed and self.tuningLimitHi and self.tuning[tempNum] > self.tuningLimitHi:
            self.tuning[tempNum] = self.tuningLimitHi
        self.tnNSamples[tempNum] = 0
        self.tnNAccepts[tempNum] = 0


class McmcProposalProbs(dict):
    """Relative proposal probabilities (p4/mcmc.py:110-200)."""

    DEFAULTS = dict(allCompsDir=1.0, allRMatricesDir=1.0, gdasrv=1.0, pInvar=1.0, local=1.0,
                    brLen=0.0, allBrLens=1.0, eTBR=1.0, relRate=1.0, learned=0.0)

    def __init__(self, **kw):
        dict.__init__(self, self.DEFAULTS)
        for k, v in kw.items():
            if k not in self.DEFAULTS:
                raise P4Error("no such proposal '%s'" % k)
            self[k] = float(v)

    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError:
            raise AttributeError(k)

    def __setattr__(self, k, v):
        if k not in self.DEFAULTS:
            raise P4Error("no such proposal '%s'" % k)
        self[k] = float(v)


# --------------------------------------------------------------------- chain
class PriorEvaluator(object):
    """lnL = 0 for every state: the chain samples the prior (tests of the
    proposals' Hastings ratios)."""

    def evaluate(self, states):
        return [0.0] * len(states)


class Chain(object):
    def __init__(self, mcmc, tempNum, state, shared):
        self.mcmc = mcmc
        self.tempNum = tempNum
        self.cur = state
        self.engine = Engine(mcmc.problem, shared=shared) if shared is not None else None
        self.loaded = None            # State the engine currently holds
        self.dirty = set(["all"])
        self.curLogLike = None
        self.prop = None
        self.proposal = None
        self.logPriorRatio = 0.0
        self.logProposalRatio = 0.0
        self.learnedJump = 0.0        # squared whitened jump of the last learned proposal
        self.changed = set()

    def load(self, st, fields):
        """Write the given fields of state `st` into the library tree."""
        e = self.engine
        full = "all" in fields
        if full or "topo" in fields:
            e.setTopologyArrays(st.parent, st.leftChild, st.sibling, st.root)
        if full or "brLen" in fields or "topo" in fields:
            e.setBrLensFast(st.brLen)
        for p, ps in enumerate(st.parts):
            if full or ("comps", p) in fields:
                for c in range(ps.comps.shape[0]):
                    e.setComp(p, c, ps.comps[c])
            if full or ("rmats", p) in fields:
                for r in range(ps.rvals.shape[0]):
                    e.setRMatrix(p, r, ps.rvals[r])
            if full or ("gamma", p) in fields:
                for g in range(len(ps.gamma)):
                    e.setGamma(p, g, ps.gamma[g])
            if full or ("pInvar", p) in fields:
                e.setPInvar(p, ps.pInvar)
            if full or ("relRate", p) in fields:
                e.setRelRate(p, ps.relRate)


# --------------------------------------------------------------------- mcmc
class Mcmc(object):
    """p4's Mcmc (p4/mcmc.py:672): MCMCMC over a Tree with its data and model.

    nChains chains at cumulative temperatures chainTemps = [0, t, 2t, ...]
    (the swap vector, p4/mcmc.py:2636-2641; the temperatures are fixed, p4's
    swap tuner is not rebuilt); one swap attempt between adjacent
    temperatures per generation; heat beta = 1/(1+T) on the likelihood and
    prior ratios (p4/chain.py:1100-1118).  With files on (the default for a
    Tree), every sampleInterval generations the cold chain is written to
    mcmc_likes_<runNum>, mcmc_trees_<runNum>.nex and mcmc_prams_<runNum>, and
    every checkPointInterval generations the run is pickled to
    mcmc_checkPoint_<runNum>.<gen+1> (p4gpu.mcmcio; resume with
    p4gpu.func.unPickleMcmc), in p4's formats.
    """

    def __init__(self, aTree, nChains=4, runNum=0, sampleInterval=100, checkPointInterval=10000,
                 simulate=None, writePrams=True, constraints=None, verbose=True,
                 chainTemp=0.1, seed=0, prob=None, startState=None, brLenPriorLambda=10.0, tune=True,
                 freeRelRates=None, freePInvar=None, evaluator="graph", writeFiles=None, _restart=False):
        """aTree: a p4gpu.tree.Tree with data and model attached (or a
        synthetic-problem object, for which files are off by default).

        evaluator: 'graph' (all chains in one captured launch sequence),
        'batch' (the same without the graph), 'sequential' (one library call
        and one host synchronisation per chain, as p4 loops over chains), or
        an object whose evaluate(states) returns the lnL of each given chain
        state (a host-side likelihood, e.g. PriorEvaluator), or a callable
        that makes such an object from the run's problem."""
        from .tree import Tree
        if constraints is not None:
            raise P4Error("Mcmc: topology constraints are not supported")
        if simulate:
            raise P4Error("Mcmc: posterior-predictive simulation during the run is not supported")
        try:
            nChains = int(nChains)
            runNum = int(runNum)
        except (TypeError, ValueError):
            raise P4Error("Mcmc: nChains and runNum must be ints")
        if nChains < 1 or runNum < 0:
            raise P4Error("Mcmc: nChains >= 1 and runNum >= 0 required")
        if isinstance(aTree, Tree):
            self.tree = aTree
            problem = aTree.toProblem()
            if freeRelRates is None:
                freeRelRates = aTree.model.relRatesAreFree
            if freePInvar is None:
                freePInvar = [mp.pInvarFree for mp in aTree.model.parts]
            if writeFiles is None:
                writeFiles = True
        else:
            problem = aTree
            self.tree = Tree.fromProblem(problem)
        self.problem = problem
        self.nChains = nChains
        self.runNum = runNum
        self.verbose = verbose
        self.chainTemp = chainTemp
        self.chainTemps = [i * chainTemp for i in range(nChains)]
        self.rng = numpy.random.default_rng(seed)
        self.sampleInterval = sampleInterval
        self.checkPointInterval = checkPointInterval
        self.writePrams = writePrams
        self.writeFiles = bool(writeFiles)
        self.prob = prob if prob is not None else McmcProposalProbs()
        self.brLenPriorLambda = brLenPriorLambda
        self.doTuning = tune
        self.gen = -1
        t = problem.tree
        self.nTax = t.nLeaves
        self.isLeaf = t.isLeaf.copy()
        self.seqNum = t.seqNum.copy()
        self.freePInvar = [sp.pInvar > 0 for sp in problem.parts] if freePInvar is None else list(freePInvar)
        self.freeRelRates = bool(freeRelRates) and len(problem.parts) > 1
        self.samples = {"gen": [], "lnL": [], "treeLength": [], "alpha": [], "splits": []}
        self.learned = None
        self.nEvals = 0
        self.files = None
        if self.writeFiles and not _restart:
            from . import mcmcio
            mcmcio.check_new_run(self)
        self._attach(evaluator, [startState if startState is not None else state_from_problem(problem)] * nChains)
        self._makeProposals()
        self.swapAttempts = [0] * max(nChains - 1, 1)
        self.swapAccepts = [0] * max(nChains - 1, 1)
        lnls = self._evaluate(self.chains, [ch.cur for ch in self.chains])
        for ch, l in zip(self.chains, lnls):
            ch.curLogLike = float(l)

    def _attach(self, evaluator, states):
        """Chains at the given states, and the likelihood machinery they use
        (library engines and the batch, or a host evaluator)."""
        if isinstance(evaluator, type) or (callable(evaluator) and not hasattr(evaluator, "evaluate")):
            evaluator = evaluator(self.problem)      # a class or factory of host evaluators
        self.hostEval = None if isinstance(evaluator, str) else evaluator
        if self.hostEval is None and evaluator not in ("graph", "batch", "sequential"):
            raise P4Error("unknown evaluator %r" % (evaluator,))
        self.evaluator = evaluator
        self.shared = make_data(self.problem) if self.hostEval is None else None
        self.chains = [Chain(self, i, st.copy(), self.shared) for i, st in enumerate(states)]
        self.batch = None
        if evaluator in ("graph", "batch"):
            self.batch = pf.Batch([ch.engine.cTree for ch in self.chains], graph=(evaluator == "graph"))
        for ch in self.chains:
            if ch.engine is not None:
                ch.load(ch.cur, {"all"})
            ch.dirty = set()

    def recomputeLogLikes(self):
        """Every chain's lnL evaluated afresh at its current state (what p4's
        checkpoint and restart do with calcLogLike)."""
        for ch in self.chains:
            if ch.engine is not None:
                ch.load(ch.cur, {"all"})
            ch.dirty = set()
        return [float(x) for x in self._evaluate(self.chains, [ch.cur for ch in self.chains])]

    def _evaluate(self, active, states):
        """lnL of every chain in `active` at `states` (with the library, the
        chains' engines already hold those values)."""
        self.nEvals += len(active)
        if self.hostEval is not None:
            if getattr(self.hostEval, "wantsIds", False):     # per-chain state kept by the evaluator
                return self.hostEval.evaluate(states, [self.chains.index(ch) for ch in active])
            return self.hostEval.evaluate(states)
        if self.batch is not None:
            allL = self.batch.logLike()
            return [allL[self.chains.index(ch)] for ch in active]
        out = []
        for ch in active:
            pf.p4_setPrams(ch.engine.cTree, -1)
            out.append(pf.p4_treeLogLike(ch.engine.cTree, 0))
        return out

    # ---------------------------------------------------------- proposals
    def _makeProposals(self):
        nN = self.problem.tree.nNodes
        n = self.nChains
        P = []
        pr = self.prob
        if pr.brLen:
            P.append(Proposal("brLen", pr.brLen * (nN - 1), 2.0 * math.log(2.0), n))
        if pr.allBrLens:
            P.append(Proposal("allBrLens", pr.allBrLens * (nN - 1), 2.0 * math.log(1.02), n,
                              acc=(0.4, 0.15, 0.05, 0.03), tuningLimitHi=0.2))
        if pr.local:
            P.append(Proposal("local", pr.local * (nN - 1), 2.0 * math.log(1.1), n,
                              acc=(0.7, 0.6, 0.05, 0.03)))
        if pr.eTBR:
            P.append(Proposal("eTBR", pr.eTBR * (nN - 1), ETBR_LAMBDA, n))
        for p, sp in enumerate(self.problem.parts):
            dirAcc, dirFac = (0.4, 0.15, 0.05, 0.03), (0.7, 0.8, 1.2, 1.4)
            if pr.allCompsDir and sp.comps.shape[0]:
                P.append(Proposal("allCompsDir", pr.allCompsDir * (sp.dim - 1) * sp.comps.shape[0], 500.0,
                                  n, pNum=p, acc=dirAcc, factor=dirFac))
            nFreeR = sum(1 for x in getattr(sp, "rSpecs", [20] * sp.rmats.shape[0]) if x == 20)
            if pr.allRMatricesDir and nFreeR:   # empirical matrices are fixed
                k = (sp.dim * sp.dim - sp.dim) / 2 - 1
                P.append(Proposal("allRMatricesDir", pr.allRMatricesDir * nFreeR * k, 500.0,
                                  n, pNum=p, acc=dirAcc, factor=dirFac))
            if pr.gdasrv and sp.nCat > 1 and len(sp.gammaShapes):
                P.append(Proposal("gdasrv", pr.gdasrv, 2.0 * math.log(1.5), n, pNum=p,
                                  acc=(0.7, 0.6, 0.15, 0.10), factor=(2.0, 1.5, 0.75, 0.5)))
            if pr.pInvar and self.freePInvar[p]:
                P.append(Proposal("pInvar", pr.pInvar, 0.5, n, pNum=p, acc=(0.7, 0.6, 0.1, 0.06)))
        if pr.relRate and self.freeRelRates:
            P.append(Proposal("relRate", pr.relRate, 0.5, n))
        if pr.learned:
            P.append(Proposal("learned", pr.learned * (nN - 1), 1.0, n))
        if not P:
            raise P4Error("no proposals")
        self.proposals = P
        w = numpy.array([p.weight for p in P])
        self.cumWeights = numpy.cumsum(w)
        self.totalWeight = float(w.sum())

    def chooseProposal(self):
        r = self.rng.uniform(0.0, self.totalWeight)
        i = int(numpy.searchsorted(self.cumWeights, r, side="right"))
        return self.proposals[min(i, len(self.proposals) - 1)]

    def _reflect(self, v, lo, hi, mult):
        """p4's reflection back into [lo, hi] (multiplicative or additive)."""
        for _ in range(1000):
            if v < lo:
                v = lo * lo / v if mult else (lo - v) + lo
            elif v > hi:
                v = hi * hi / v if mult else hi - (v - hi)
            else:
                return v
        return min(max(v, lo), hi)

    def propose(self, ch, prop):
        """Apply `prop` to a copy of ch.cur; sets ch.prop, ratios, changed
        fields.  Returns False if the proposal aborts (doAbort in p4)."""
        name = prop.name
        st = ch.cur.copy() if name == "learned" else ch.cur.shallow()
        rng = self.rng
        tn = prop.tuning[ch.tempNum]
        lam = self.brLenPriorLambda
        ch.logPriorRatio = 0.0
        ch.logProposalRatio = 0.0
        ch.changed = set()
        if name == "brLen":
            st.own_brLen()
            nodes = [v for v in range(len(st.brLen)) if v != st.root]
            v = nodes[int(rng.integers(len(nodes)))]
            old = st.brLen[v]
            new = self._reflect(old * math.exp(tn * (rng.random() - 0.5)), var.BRLEN_MIN, var.BRLEN_MAX, True)
            st.brLen[v] = new
            ch.logProposalRatio = math.log(new / old)
            ch.logPriorRatio = lam * (old - new)
            ch.changed.add("brLen")
        elif name == "allBrLens":
            # sliding window on every branch (p4/chain.py:3143-3197)
            st.own_brLen()
            sel = numpy.arange(len(st.brLen)) != st.root
            old = st.brLen[sel]
            new = old + tn * (rng.random(len(old)) - 0.5)
            lo, hi = var.BRLEN_MIN, var.BRLEN_MAX
            for _ in range(1000):           # additive reflection into [lo, hi], as _reflect
                below, above = new < lo, new > hi
                if not (below.any() or above.any()):
                    break
                new[below] = (lo - new[below]) + lo
                new[above] = hi - (new[above] - hi)
            new = numpy.clip(new, lo, hi)
            st.brLen[sel] = new
            ch.logPriorRatio = lam * float((old - new).sum())
            ch.changed.add("brLen")
        elif name == "local":
            st.own_brLen()
            st.own_topology()
            ok = self._proposeLocal(st, tn, ch)
            if not ok:
                return False
        elif name == "eTBR":
            st.own_brLen()
            st.own_topology()
            t = LinkedTree(st.parent, st.leftChild, st.sibling, st.root, st.brLen, self.isLeaf)
            ch.logPriorRatio, ch.logProposalRatio, changed = propose_etbr(t, rng, tn, ETBR_PEXT, lam)
            st.parent[:] = t.parent
            st.leftChild[:] = t.leftChild
            st.sibling[:] = t.sibling
            st.brLen[:] = t.brLens()
            ch.changed.add("brLen")
            if changed:
                ch.changed.add("topo")
                self._topoChanged = True
        elif name == "allCompsDir":
            p = prop.pNum
            ps = st.own_part(p)
            for c in range(ps.comps.shape[0]):
                cur = ch.cur.parts[p].comps[c]
                new = rng.dirichlet(tn * cur)
                for _ in range(1000):
                    if new.min() >= var.PIVEC_MIN:
                        break
                    low = new < var.PIVEC_MIN
                    new[low] += (1.0 + rng.random(int(low.sum()))) * var.PIVEC_MIN
                    new /= new.sum()
                new = _fix_sum(new)
                ps.comps[c] = new
                ch.logProposalRatio += dirichlet_lnpdf(tn * new, cur) - dirichlet_lnpdf(tn * cur, new)
            ch.changed.add(("comps", p))
        elif name == "allRMatricesDir":
            p = prop.pNum
            ps = st.own_part(p)
            specs = getattr(self.problem.parts[p], "rSpecs", None)
            for r in range(ps.rvals.shape[0]):
                if specs is not None and specs[r] != 20:
                    continue
                cur = ch.cur.parts[p].rvals[r]
                new = rng.dirichlet(tn * cur)
                for _ in range(1000):
                    if new.min() >= var.RATE_MIN and new.max() <= var.RATE_MAX:
                        break
                    lo = new < var.RATE_MIN
                    new[lo] += (1.0 + rng.random(int(lo.sum()))) * var.RATE_MIN
                    hi = new > var.RATE_MAX
                    new[hi] = var.RATE_MAX - (1.0 + rng.random(int(hi.sum()))) * var.RATE_MIN
                    new /= new.sum()
                ps.rvals[r] = new
                ch.logProposalRatio += dirichlet_lnpdf(tn * new, cur) - dirichlet_lnpdf(tn * cur, new)
            ch.changed.add(("rmats", p))
        elif name == "gdasrv":
            p = prop.pNum
            ps = st.own_part(p)
            old = float(ps.gamma[0])
            new = self._reflect(old * math.exp(tn * (rng.random() - 0.5)), var.GAMMA_SHAPE_MIN,
                                var.GAMMA_SHAPE_MAX, True)
            ps.gamma[0] = new
            ch.logProposalRatio = math.log(new / old)
            ch.logPriorRatio = old - new          # exponential(1) prior on the shape
            ch.changed.add(("gamma", p))
        elif name == "pInvar":
            p = prop.pNum
            ps = st.own_part(p)
            ps.pInvar = self._reflect(ps.pInvar + (rng.random() - 0.5) * tn, var.PINVAR_MIN, var.PINVAR_MAX,
                                      False)
            ch.changed.add(("pInvar", p))
        elif name == "relRate":
            tot = 0.0
            fact = 0.0
            for p in range(len(st.parts)):
                ps = st.own_part(p)
                ps.relRate = self._reflect(ps.relRate + (rng.random() - 0.5) * tn, var.RELRATE_MIN,
                                           var.RELRATE_MAX, False)
            for p, ps in enumerate(st.parts):
                n = self.problem.parts[p].nChar
                tot += n
                fact += ps.relRate * n
            for p, ps in enumerate(st.parts):
                ps.relRate *= tot / fact
                ch.changed.add(("relRate", p))
        elif name == "learned":
            if self.learned is None:
                return False
            ok = self.learned.propose(self, ch, st, tn)
            if not ok:
                return False
        else:
            raise P4Error("unknown proposal %s" % name)
        ch.prop = st
        return True

    def _reroot_to_child(self, st, newRoot):
        kids = st.kids()
        old = st.root
        kids[old].remove(newRoot)
        kids[newRoot].append(old)
        st.brLen[old] = st.brLen[newRoot]
        st.brLen[newRoot] = 0.0
        st.root = newRoot
        st.set_kids(kids)

    def _proposeLocal(self, st, tn, ch):
        """Larget-Simon LOCAL on the path a-u-v-c (p4/chain.py:3199-3960)."""
        rng = self.rng
        n = len(st.parent)
        for _ in range(100):
            c = int(rng.integers(n))
            if st.parent[c] >= 0 and st.parent[st.parent[c]] >= 0:
                break
        else:
            return False
        v = int(st.parent[c])
        u = int(st.parent[v])
        if st.parent[u] < 0:       # u is the root: re-root on another child of it
            cands = [x for x in st.children(u) if x != v]
            if not cands:
                return False
            self._reroot_to_child(st, cands[int(rng.integers(len(cands)))])
            ch.changed.add("topo")
        a = int(st.parent[u])
        kids = st.kids()
        # rotate so that c leads v's children, v leads u's: d, b = next siblings
        kv = kids[v]
        i = kv.index(c)
        kv[:] = kv[i:] + kv[:i]
        ku = kids[u]
        i = ku.index(v)
        ku[:] = ku[i:] + ku[:i]
        d = kv[1]
        b = ku[1]
        m = st.brLen[c] + st.brLen[v] + st.brLen[u]
        x = st.brLen[u]
        y = x + st.brLen[v]
        ratio = math.exp(tn * (rng.random() - 0.5))
        newM = m * ratio
        if rng.random() < 0.5:
            newY = y * ratio
            newX = rng.random() * newM
            for _ in range(101):
                if abs(newY - newX) >= var.BRLEN_MIN:
                    break
                newX = rng.random() * newM
            else:
                return False
        else:
            newX = x * ratio
            newY = rng.random() * newM
            for _ in range(101):
                if abs(newY - newX) >= var.BRLEN_MIN:
                    break
                newY = rng.random() * newM
            else:
                return False
        if newX < newY:        # same topology
            st.brLen[u] = newX
            st.brLen[v] = newY - newX
            st.brLen[c] = newM - newY
            st.set_kids(kids)
        else:                  # v takes u's place under a; u goes under v with c and b
            ia = kids[a].index(u)
            kids[a][ia] = v
            kv_rest = [x2 for x2 in kv if x2 != c]          # d and any further children of v
            ku_rest = [x2 for x2 in ku if x2 not in (v, b)]  # further children of u
            kids[v] = [u] + kv_rest
            kids[u] = [c, b] + ku_rest
            st.brLen[v] = newY
            st.brLen[u] = newX - newY
            st.brLen[c] = newM - newX
            st.set_kids(kids)
            ch.changed.add("topo")
            self._topoChanged = True
        for x2 in (c, v, u):
            if not (var.BRLEN_MIN <= st.brLen[x2] <= var.BRLEN_MAX):
                return False
        ch.logProposalRatio = 3.0 * math.log(ratio)
        ch.logPriorRatio = self.brLenPriorLambda * (m - newM)
        ch.changed.add("brLen")
        return True

    # ---------------------------------------------------------- loop
    def step(self):
        """One generation: a proposal per chain, one batched lnL call, MH
        per chain, one swap attempt, tuning."""
        self.gen += 1
        active = []
        for ch in self.chains:
            prop = self.chooseProposal()
            ch.proposal = prop
            self._topoChanged = False
            ok = self.propose(ch, prop)
            if not ok:
                prop.nAborts[ch.tempNum] += 1
                continue
            if self._topoChanged:
                prop.nTopologyChanges[ch.tempNum] += 1
            if ch.engine is not None:
                ch.load(ch.prop, ch.changed | ch.dirty)
            ch.dirty = set()
            active.append(ch)
        lnls = self._evaluate(active, [ch.prop for ch in active]) if active else []
        for ch, propLnL in zip(active, lnls):
            prop = ch.proposal
            beta = 1.0 / (1.0 + self.chainTemps[ch.tempNum])
            llr = (float(propLnL) - ch.curLogLike) * beta
            pRet = llr + ch.logProposalRatio + ch.logPriorRatio * beta
            if pRet < -100.0:
                r = 0.0
            elif pRet >= 0.0:
                r = 1.0
            else:
                r = math.exp(pRet)
            accept = r == 1.0 or self.rng.random() < r
            prop.nProposals[ch.tempNum] += 1
            prop.tnNSamples[ch.tempNum] += 1
            if accept:
                prop.nAcceptances[ch.tempNum] += 1
                prop.tnNAccepts[ch.tempNum] += 1
                if prop.name == "learned" and self.learned is not None:
                    self.learned.nAccepted += 1
                    self.learned.sumJump += ch.learnedJump
                ch.cur = ch.prop
                ch.curLogLike = float(propLnL)
            else:
                ch.dirty = set(ch.changed)      # engine holds the rejected values
            if self.doTuning and prop.name in TUNABLE and prop.tnNSamples[ch.tempNum] >= prop.tnSampleSize:
                prop.tune(ch.tempNum)
        if self.nChains > 1:
            self._swap()
        if self.sampleInterval and (self.gen + 1) % self.sampleInterval == 0:   # p4/mcmc.py:2991
            self._sample()
            if self.files is not None:
                self.files.sample(self)
        if self.files is not None and self.checkPointInterval and (self.gen + 1) % self.checkPointInterval == 0:
            self.checkPoint()

    def _swap(self):
        """Swap vector between adjacent temperatures (p4/mcmc.py:3299-3341)."""
        t1 = int(self.rng.integers(self.nChains - 1))
        t2 = t1 + 1
        c1 = next(ch for ch in self.chains if ch.tempNum == t1)
        c2 = next(ch for ch in self.chains if ch.tempNum == t2)
        b1 = 1.0 / (1.0 + self.chainTemps[t1])
        b2 = 1.0 / (1.0 + self.chainTemps[t2])
        lnR = b1 * c2.curLogLike + b2 * c1.curLogLike - b1 * c1.curLogLike - b2 * c2.curLogLike
        r = 0.0 if lnR < -100.0 else (1.0 if lnR >= 0.0 else math.exp(lnR))
        self.swapAttempts[t1] += 1
        if self.rng.random() < r:
            self.swapAccepts[t1] += 1
            c1.tempNum, c2.tempNum = c2.tempNum, c1.tempNum

    def coldChain(self):
        return next(ch for ch in self.chains if ch.tempNum == 0)

    def _sample(self):
        ch = self.coldChain()
        s = self.samples
        s["gen"].append(self.gen + 1)
        s["lnL"].append(ch.curLogLike)
        s["treeLength"].append(ch.cur.tree_length())
        ps = ch.cur.parts[0]
        s["alpha"].append(float(ps.gamma[0]) if len(ps.gamma) else float("nan"))
        s["splits"].append(splits_of(ch.cur, self.isLeaf, self.seqNum, self.nTax))

    def run(self, nGensToDo, callback=None):
        """Mcmc.run (p4/mcmc.py:2496): nGensToDo generations.  A run after the
        first (or after a restart from a checkpoint) zeroes the proposal and
        swap counts, as p4 does; the tuner's counts and the tunings carry on."""
        if self.gen > -1:
            for p in self.proposals:
                p.nProposals = [0] * self.nChains
                p.nAcceptances = [0] * self.nChains
                p.nTopologyChanges = [0] * self.nChains
                p.nAborts = [0] * self.nChains
            self.swapAttempts = [0] * max(self.nChains - 1, 1)
            self.swapAccepts = [0] * max(self.nChains - 1, 1)
        if self.writeFiles:
            from . import mcmcio
            if self.checkPointInterval and self.sampleInterval and self.checkPointInterval % self.sampleInterval:
                raise P4Error("the checkPointInterval (%d) should be evenly divisible by the sampleInterval (%d)"
                              % (self.checkPointInterval, self.sampleInterval))
            self.files = mcmcio.SampleFiles(self)
        try:
            for _ in range(nGensToDo):
                self.step()
                if callback:
                    callback(self)
        finally:
            if self.files is not None:
                self.files.finish()
                self.files = None

    def checkPoint(self):
        """Mcmc.checkPoint (p4/mcmc.py:3516): every chain's lnL recomputed and
        checked against the running value (within 0.01), then the run's host
        state -- tree and model without the data, chain states, tunings,
        counts, random-number state -- pickled to
        mcmc_checkPoint_<runNum>.<gen+1>."""
        from . import mcmcio
        return mcmcio.check_point(self)

    def acceptance(self):
        out = {}
        for p in self.proposals:
            n = sum(p.nProposals)
            out[p.name + ("" if p.pNum < 0 else ".%d" % p.pNum)] = (sum(p.nAcceptances) / n) if n else None
        return out


def _fix_sum(c):
    c = c / c.sum()
    c[numpy.argmax(c)] += 1.0 - c.sum()
    return c


def state_from_problem(problem):
    t = problem.tree
    parts = []
    for sp in problem.parts:
        parts.append(PartState(sp.comps.copy(), numpy.stack([upper(R) for R in sp.rmats]),
                               numpy.array(sp.gammaShapes, numpy.double), sp.pInvar, sp.relRate))
    return State(t.parent.copy(), t.leftChild.copy(), t.sibling.copy(), t.root, t.brLen.copy(), parts)


def splits_of(st, isLeaf, seqNum, nTax):
    """Non-trivial splits of the tree as bitmasks over taxa, each normalised
    so that taxon 0 is outside the set."""
    kids = st.kids()
    n = len(kids)
    masks = [0] * n
    order = []
    stack = [int(st.root)]
    while stack:
        v = stack.pop()
        order.append(v)
        stack.extend(kids[v])
    full = (1 << nTax) - 1
    out = set()
    for v in reversed(order):
        if isLeaf[v]:
            masks[v] = 1 << int(seqNum[v])
        m = masks[v]
        for c in kids[v]:
            m |= masks[c]
        masks[v] = m
        if v != st.root:
            k = bin(m).count("1")
            if 1 < k < nTax - 1:
                out.add(m if not (m & 1) else (full ^ m))
    return frozenset(out)


# --------------------------------------------------------------------- diagnostics
def effective_sample_size(data):
    """Tracer's autocorrelation ESS as p4 computes it (p4/func.py:2953,
    Pf/pfmodule.c:2631-2698): lags up to min(n/3, 1000), pairwise sums of
    adjacent autocovariances until one is non-positive."""
    x = numpy.asarray(data, numpy.double)
    n = len(x)
    if n < 2:
        return 0.0
    mean = x.mean()
    d = x - mean
    maxLag = min(int(n / 3), 1000)
    prev = 0.0
    var0 = 0.0
    varStat = 0.0
    for lag in range(maxLag):
        g = float(numpy.dot(d[: n - lag], d[lag:])) / (n - lag)
        if lag == 0:
            varStat = g
            var0 = g
        elif lag % 2 == 0:
            if prev + g > 0.0:
                varStat += 2.0 * (prev + g)
            else:
                break
        prev = g
    if varStat == 0.0:
        return 0.0
    return n * (var0 / varStat)


def split_frequencies(splitSets):
    counts = {}
    for s in splitSets:
        for m in s:
            counts[m] = counts.get(m, 0) + 1
    n = float(len(splitSets))
    return {m: c / n for m, c in counts.items()}


def asdsf(splitSets1, splitSets2, minimumProportion=0.1):
    """Average standard deviation of split frequencies between two runs
    (p4/func.py:3428-3468: splits with support >= minimumProportion in
    either run; n-1 weighted standard deviation of the two supports)."""
    return asdsf_of_frequencies(split_frequencies(splitSets1), split_frequencies(splitSets2),
                                minimumProportion)


def asdsf_of_frequencies(f1, f2, minimumProportion=0.1):
    """ASDSF of two runs given as {split: frequency} maps."""
    keys = [k for k in set(f1) | set(f2)
            if f1.get(k, 0.0) >= minimumProportion or f2.get(k, 0.0) >= minimumProportion]
    if not keys:
        return 0.0
    sds = [abs(f1.get(k, 0.0) - f2.get(k, 0.0)) / math.sqrt(2.0) for k in keys]
    return sum(sds) / len(sds)
