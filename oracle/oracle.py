"""TEST INFRASTRUCTURE: Python access to the two CPU oracles.

  - libp4ref.so: the reference p4 FP64 likelihood core (Pf/*.c), compiled
    from the reference sources by oracle/Makefile, driven through
    ref_driver.c.  Outputs of the reference itself.
  - libp4port.so: the project's CPU restatement (p4port.c): reference-
    semantics FP64 pruning, the published discrete-gamma algorithms, and a
    bit-exact FP32 mirror of the GPU kernel's arithmetic.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module; the product never imports it.
"""
import ctypes
import os
import subprocess

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SO = os.path.join(HERE, "_ref", "libp4ref.so")
PORT_SO = os.path.join(HERE, "_ref", "libp4port.so")
# The reference's Pf sources: staged into _ref/src (git-ignored) from the
# directory named by P4_REFERENCE_PF (or given to build()), then built there.
REF_ENV = "P4_REFERENCE_PF"
REF_COPY = os.path.join(HERE, "_ref", "src")
REF_SOURCES = ("p4_tree.c p4_node.c eig.c linalg.c pcomplex.c gamma.c util.c pmatrices.c part.c p4_model.c "
               "proteinModels.c p4_treeCopyVerify.c p4_treeSim.c p4_treeNewt.c p4_treeOpt.c brent.c").split()

D = ctypes.POINTER(ctypes.c_double)
I = ctypes.POINTER(ctypes.c_int)
F = ctypes.POINTER(ctypes.c_float)
U8 = ctypes.POINTER(ctypes.c_uint8)
U32 = ctypes.POINTER(ctypes.c_uint32)
VP = ctypes.c_void_p


def _d(a):
    return a.ctypes.data_as(D)


def _i(a):
    return a.ctypes.data_as(I)


def stage_reference(refdir):
    """Copy the reference sources the oracle compiles (and every header of
    that directory) into _ref/src; files already identical are left alone."""
    import filecmp
    import shutil
    os.makedirs(REF_COPY, exist_ok=True)
    names = list(REF_SOURCES) + sorted(f for f in os.listdir(refdir) if f.endswith(".h"))
    for f in names:
        src, dst = os.path.join(refdir, f), os.path.join(REF_COPY, f)
        if not (os.path.exists(dst) and filecmp.cmp(src, dst, shallow=False)):
            shutil.copyfile(src, dst)


def have_ref_sources():
    return all(os.path.exists(os.path.join(REF_COPY, f)) for f in REF_SOURCES)


def build(ref=True, refdir=None):
    """make -C oracle: the port always; the reference core where its sources
    are given (refdir or $P4_REFERENCE_PF, staged into _ref/src first) or were
    staged before.  A reference build that fails where only the staged copy
    exists (a host without Python headers) is reported, not raised."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    if not ref:
        return
    refdir = refdir or os.environ.get(REF_ENV)
    if refdir and os.path.isdir(refdir):
        stage_reference(refdir)
    elif not have_ref_sources():
        return
    r = subprocess.run(["make", "-s", "-C", HERE, "REF=" + REF_COPY, "ref"], capture_output=True, text=True)
    if r.returncode != 0:
        msg = "oracle: reference core did not build (%s)" % (r.stderr.strip().splitlines() or ["?"])[-1]
        if refdir:
            raise RuntimeError(msg + "\n" + r.stderr)
        print(msg)


def have_ref():
    return os.path.exists(REF_SO)


_ref = None
_port = None


def ref_lib():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            build(ref=True)
        lib = ctypes.CDLL(REF_SO)
        lib.ref_new.restype = VP
        lib.ref_new.argtypes = [ctypes.c_int, ctypes.c_int]
        lib.ref_part.restype = ctypes.c_int
        lib.ref_part.argtypes = [VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p,
                                 ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p]
        lib.ref_nPatterns.restype = ctypes.c_int
        lib.ref_nPatterns.argtypes = [VP, ctypes.c_int]
        lib.ref_getPatterns.restype = None
        lib.ref_getPatterns.argtypes = [VP, ctypes.c_int, I, I, I, I, I]
        lib.ref_modelPart.restype = ctypes.c_int
        lib.ref_modelPart.argtypes = [VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, D, ctypes.c_int,
                                      D, ctypes.c_int, D, D, D, ctypes.c_int, ctypes.c_double,
                                      ctypes.c_double]
        lib.ref_tree.restype = ctypes.c_int
        lib.ref_tree.argtypes = [VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, I, I, I, I, I, D, I,
                                 I, I, I, I]
        lib.ref_setBrLen.restype = None
        lib.ref_setBrLen.argtypes = [VP, ctypes.c_int, ctypes.c_double]
        lib.ref_logLike.restype = ctypes.c_double
        lib.ref_logLike.argtypes = [VP, D]
        lib.ref_logLikeNoSetPrams.restype = ctypes.c_double
        lib.ref_logLikeNoSetPrams.argtypes = [VP]
        lib.ref_siteLikes.restype = ctypes.c_double
        lib.ref_siteLikes.argtypes = [VP, ctypes.c_int, D]
        lib.ref_siteRates.restype = ctypes.c_double
        lib.ref_siteRates.argtypes = [VP, ctypes.c_int, D, I]
        lib.ref_getPDeck.restype = None
        lib.ref_getPDeck.argtypes = [VP, ctypes.c_int, ctypes.c_int, ctypes.c_int, D]
        lib.ref_simulate.restype = ctypes.c_longlong
        lib.ref_simulate.argtypes = [VP, ctypes.c_ulonglong, D, I]
        lib.ref_drawAncStates.restype = None
        lib.ref_drawAncStates.argtypes = [VP, ctypes.c_int, ctypes.c_uint, D, I]
        lib.ref_setTopology.restype = None
        lib.ref_setTopology.argtypes = [VP, I, I, I, ctypes.c_int, I, I]
        lib.ref_setBrLens.restype = None
        lib.ref_setBrLens.argtypes = [VP, D]
        lib.ref_setModelValues.restype = None
        lib.ref_setModelValues.argtypes = [VP, ctypes.c_int, D, D, D, ctypes.c_double, ctypes.c_double]
        lib.ref_partUpdate.restype = ctypes.c_double
        lib.ref_partUpdate.argtypes = [VP, ctypes.c_int]
        lib.ref_allBrLensLogLike.restype = ctypes.c_double
        lib.ref_allBrLensLogLike.argtypes = [VP, D]
        lib.ref_newtOptimize.restype = ctypes.c_double
        lib.ref_newtOptimize.argtypes = [VP, ctypes.c_int, D, D, D]
        lib.ref_philoxUniform.restype = ctypes.c_double
        lib.ref_philoxUniform.argtypes = [ctypes.c_ulonglong, ctypes.c_ulonglong]
        lib.ref_getBigR.restype = ctypes.c_int
        lib.ref_getBigR.argtypes = [ctypes.c_int, D]
        lib.ref_simulateRef.restype = ctypes.c_longlong
        lib.ref_simulateRef.argtypes = [VP, VP, ctypes.c_uint, D, ctypes.c_ulonglong, D, I]
        _ref = lib
    return _ref


def ref_bigR(spec):
    """The reference's 20x20 exchangeability matrix for an RMatrix spec, as its
    p4_newRMatrix fills it (Pf/p4_model.c:345-450)."""
    out = numpy.zeros((20, 20), numpy.double)
    ref_lib().ref_getBigR(int(spec), _d(out))
    return out


def port_lib():
    global _port
    if _port is None:
        if not os.path.exists(PORT_SO):
            build(ref=False)
        lib = ctypes.CDLL(PORT_SO)
        lib.port_discreteGamma.restype = ctypes.c_int
        lib.port_discreteGamma.argtypes = [ctypes.c_double, ctypes.c_int, D]
        lib.port_bigQ.restype = ctypes.c_int
        lib.port_bigQ.argtypes = [ctypes.c_int, D, D, D]
        lib.port_eigSym.restype = ctypes.c_int
        lib.port_eigSym.argtypes = [ctypes.c_int, D, D, D, D]
        lib.port_pmatrix.restype = None
        lib.port_pmatrix.argtypes = [ctypes.c_int, D, D, D, ctypes.c_double, D]
        lib.port_encode.restype = ctypes.c_int
        lib.port_encode.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p,
                                    ctypes.c_int, ctypes.c_char_p, ctypes.c_int, I]
        lib.port_makePatterns.restype = ctypes.c_int
        lib.port_makePatterns.argtypes = [ctypes.c_int, ctypes.c_int, I, I, I, I]
        lib.port_invarSites.restype = None
        lib.port_invarSites.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, I, I,
                                        I, I]
        lib.port_setRootCLOut.restype = None
        lib.port_setRootCLOut.argtypes = [D]
        lib.port_partLogLike64.restype = ctypes.c_double
        lib.port_partLogLike64.argtypes = [ctypes.c_int, ctypes.c_int, I, I, I, I, I, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_int, I, I, I, D, D,
                                           ctypes.c_double, I, I, D, D]
        lib.port_partPrune32.restype = ctypes.c_double
        lib.port_partPrune32.argtypes = [ctypes.c_int, ctypes.c_int, I, I, I, I, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_int, F, F, U8, D,
                                         ctypes.c_double, U32, U32, D, F, I, D, ctypes.c_int]
        _port = lib
    return _port


# ----------------------------------------------------------------- reference
class RefTree(object):
    """The reference likelihood core holding one Problem."""

    def __init__(self, problem):
        lib = ref_lib()
        tree = problem.tree
        nP = len(problem.parts)
        self.lib = lib
        self.problem = problem
        self.h = lib.ref_new(tree.nLeaves, nP)
        self._keep = []
        for pNum, sp in enumerate(problem.parts):
            eq = sp.equateSymbols()
            lib.ref_part(self.h, pNum, sp.dim, sp.nChar, sp.symbols.encode(), eq.encode(), len(eq),
                         sp.equatesTable().encode(), "".join(sp.sequences).encode())
            comps = numpy.ascontiguousarray(sp.comps, numpy.double).copy()
            rm = numpy.ascontiguousarray(sp.rmats, numpy.double).copy()
            nG = len(sp.gammaShapes)
            gv = numpy.array(sp.gammaShapes, numpy.double).copy() if nG else numpy.zeros(1)
            gf = numpy.zeros(max(nG, 1) * sp.nCat)
            gr = numpy.zeros(max(nG, 1) * sp.nCat)
            self._keep += [comps, rm, gv, gf, gr]
            self._rates = getattr(self, "_rates", []) + [(gr, nG, sp.nCat)]
            lib.ref_modelPart(self.h, pNum, sp.dim, comps.shape[0], _d(comps), rm.shape[0], _d(rm), nG,
                              _d(gv), _d(gf), _d(gr), sp.nCat, sp.pInvar, sp.relRate)
        n = tree.nNodes
        cn = numpy.zeros((n, nP), numpy.int32)
        rn = numpy.zeros((n, nP), numpy.int32)
        gn = numpy.zeros((n, nP), numpy.int32)
        for pNum, sp in enumerate(problem.parts):
            cn[:, pNum] = sp.compNums
            rn[:, pNum] = sp.rMatrixNums
            gn[:, pNum] = sp.gdasrvNums
        arrs = [numpy.ascontiguousarray(a, numpy.int32) for a in
                (tree.parent, tree.leftChild, tree.sibling, tree.seqNum, tree.isLeaf)]
        self._keep += arrs + [cn, rn, gn]
        bl = numpy.ascontiguousarray(tree.brLen, numpy.double)
        lib.ref_tree(self.h, n, tree.nLeaves, tree.root, _i(arrs[0]), _i(arrs[1]), _i(arrs[2]),
                     _i(arrs[3]), _i(arrs[4]), _d(bl), _i(cn), _i(rn), _i(gn),
                     _i(tree.preOrder.astype(numpy.int32)), _i(tree.postOrder.astype(numpy.int32)))

    def setBrLens(self, brLen):
        for v, L in enumerate(brLen):
            if v != self.problem.tree.root:
                self.lib.ref_setBrLen(self.h, v, float(L))

    def logLike(self):
        pl = numpy.zeros(len(self.problem.parts))
        lnL = self.lib.ref_logLike(self.h, _d(pl))
        return lnL, pl

    def allBrLensLogLike(self, brLen):
        """p4's allBrLens evaluation: new branch lengths, every node's P decks
        (eigensystems kept), full pruning and log-sum; returns lnL."""
        bl = numpy.ascontiguousarray(brLen, numpy.double)
        return self.lib.ref_allBrLensLogLike(self.h, _d(bl))

    def setState(self, st):
        """Push one MCMC chain state (p4gpu.mcmc.State: topology, branch
        lengths, per part comps / R upper triangles / gamma shapes / pInvar /
        relRate) into the reference tree, as p4's Tree.setCStuff and
        Model.setCStuff do before a p4_setPrams."""
        lib = self.lib
        par = numpy.ascontiguousarray(st.parent, numpy.int32)
        lc = numpy.ascontiguousarray(st.leftChild, numpy.int32)
        t = self.problem.tree
        if len(par) != t.nNodes or any(bool(lc[v] >= 0) == bool(t.isLeaf[v]) for v in range(t.nNodes)
                                       if v != int(st.root)):
            raise ValueError("RefTree.setState: the state's leaves are not this tree's leaves")
        sib = numpy.ascontiguousarray(st.sibling, numpy.int32)
        pre, post = linked_orders(par, lc, sib, int(st.root))
        lib.ref_setTopology(self.h, _i(par), _i(lc), _i(sib), int(st.root), _i(pre), _i(post))
        bl = numpy.ascontiguousarray(st.brLen, numpy.double)
        lib.ref_setBrLens(self.h, _d(bl))
        for pNum, ps in enumerate(st.parts):
            c = numpy.ascontiguousarray(ps.comps, numpy.double)
            r = numpy.ascontiguousarray(ps.rvals, numpy.double)
            g = numpy.ascontiguousarray(ps.gamma if len(ps.gamma) else numpy.zeros(1), numpy.double)
            lib.ref_setModelValues(self.h, pNum, _d(c), _d(r), _d(g), float(ps.pInvar), float(ps.relRate))

    def siteLikes(self, pNum):
        out = numpy.zeros(self.problem.parts[pNum].nChar)
        self.lib.ref_siteLikes(self.h, pNum, _d(out))
        return out

    def siteRates(self, pNum):
        """(siteRates, gammaCats) of the reference's p4_partLogLikeSiteRates."""
        n = self.problem.parts[pNum].nChar
        rates = numpy.zeros(n)
        cats = numpy.zeros(n, numpy.int32)
        self.lib.ref_siteRates(self.h, pNum, _d(rates), _i(cats))
        return rates, cats

    def drawAncStates(self, pNum, seed):
        """The reference's p4_drawAncStateP for every site of part pNum on the
        root CLs of the last evaluation, libc random() seeded with seed:
        (uniforms it used, draws nChar x 4)."""
        n = self.problem.parts[pNum].nChar
        u = numpy.zeros(n)
        d = numpy.zeros((n, 4), numpy.int32)
        self.lib.ref_drawAncStates(self.h, pNum, int(seed), _d(u), _i(d))
        return u, d

    def simulate(self, seed, uniforms=None):
        """The reference's p4_simulate (no reference tree) after a logLike:
        (per part the nTax x nChar simulated codes, uniforms drawn).  With
        uniforms (an array) the reference draws from it, else from the
        Philox stream of seed."""
        tot = sum(sp.nChar for sp in self.problem.parts) * self.problem.tree.nLeaves
        out = numpy.zeros(tot, numpy.int32)
        u = None if uniforms is None else numpy.ascontiguousarray(uniforms, numpy.double)
        n = self.lib.ref_simulate(self.h, int(seed), _d(u) if u is not None else None, _i(out))
        seqs, o = [], 0
        for sp in self.problem.parts:
            k = self.problem.tree.nLeaves * sp.nChar
            seqs.append(out[o:o + k].reshape(self.problem.tree.nLeaves, sp.nChar).copy())
            o += k
        return seqs, int(n)

    def simulateRef(self, refTree, libcSeed, seed, uniforms=None):
        """The reference's p4_simulate with refTree (another RefTree, on which
        logLike has run) after a logLike of this one: (per part the nTax x
        nChar simulated codes, the libc uniforms the root draws used -- one
        per site of every part --, GSL uniforms drawn)."""
        tot = sum(sp.nChar for sp in self.problem.parts) * self.problem.tree.nLeaves
        out = numpy.zeros(tot, numpy.int32)
        lu = numpy.zeros(sum(sp.nChar for sp in refTree.problem.parts))
        u = None if uniforms is None else numpy.ascontiguousarray(uniforms, numpy.double)
        n = self.lib.ref_simulateRef(self.h, refTree.h, int(libcSeed), _d(lu), int(seed),
                                     _d(u) if u is not None else None, _i(out))
        seqs, o = [], 0
        for sp in self.problem.parts:
            k = self.problem.tree.nLeaves * sp.nChar
            seqs.append(out[o:o + k].reshape(self.problem.tree.nLeaves, sp.nChar).copy())
            o += k
        return seqs, lu, int(n)

    def newtOptimize(self, calls=((1.0, 10.0), (1.0e-1, 1.0), (1.0e-2, 0.1), (1.0e-5, 1.0e-7))):
        """The reference's p4_newtSetup + p4_newtAround(eps, delta) for each
        call (default: p4_newtAndBrentPowellOpt's sequence for a model without
        free parameters), after a logLike: (final lnL, branch lengths)."""
        eps = numpy.array([c[0] for c in calls], numpy.double)
        dl = numpy.array([c[1] for c in calls], numpy.double)
        bl = numpy.zeros(self.problem.tree.nNodes)
        lnl = self.lib.ref_newtOptimize(self.h, len(calls), _d(eps), _d(dl), _d(bl))
        return lnl, bl

    def patterns(self, pNum):
        sp = self.problem.parts[pNum]
        nT = self.problem.tree.nLeaves
        n = self.lib.ref_nPatterns(self.h, pNum)
        pats = numpy.zeros((nT, n), numpy.int32)
        cnt = numpy.zeros(n, numpy.int32)
        spi = numpy.zeros(sp.nChar, numpy.int32)
        iv = numpy.zeros(n, numpy.int32)
        ia = numpy.zeros((sp.dim, n), numpy.int32)
        self.lib.ref_getPatterns(self.h, pNum, _i(pats), _i(cnt), _i(spi), _i(iv), _i(ia))
        return pats, cnt, spi, iv, ia

    def gammaRates(self, pNum):
        gr, nG, nCat = self._rates[pNum]
        return gr[: max(nG, 1) * nCat].reshape(max(nG, 1), nCat).copy()

    def pdeck(self, node, pNum, cat):
        d = self.problem.parts[pNum].dim
        out = numpy.zeros((d, d))
        self.lib.ref_getPDeck(self.h, node, pNum, cat, _d(out))
        return out


def linked_orders(parent, leftChild, sibling, root):
    """Pre- and post-order node numbers of a tree in linked form."""
    pre, post = [], []
    stack = [(root, False)]
    while stack:
        v, done = stack.pop()
        if done:
            post.append(v)
            continue
        pre.append(v)
        stack.append((v, True))
        kids = []
        c = leftChild[v]
        while c >= 0:
            kids.append(int(c))
            c = sibling[c]
        for c in reversed(kids):
            stack.append((c, False))
    return numpy.array(pre, numpy.int32), numpy.array(post, numpy.int32)


def _same_topology(a, b):
    return (a.root == b.root and numpy.array_equal(a.parent, b.parent) and numpy.array_equal(a.leftChild, b.leftChild)
            and numpy.array_equal(a.sibling, b.sibling))


def _same_part(a, b):
    return (numpy.array_equal(a.comps, b.comps) and numpy.array_equal(a.rvals, b.rvals)
            and numpy.array_equal(a.gamma, b.gamma) and a.pInvar == b.pInvar and a.relRate == b.relRate)


class RefChainEvaluator(object):
    """The lnL of MCMC chain states from the reference's own C core.  Plugged
    into p4gpu.mcmc.Mcmc as its evaluator, it turns the project's sampler
    into a CPU chain on the reference likelihood.

    Each chain (by the ids the sampler passes) has its own reference tree, and
    a state is evaluated the way p4's Chain.proposeSp evaluates a proposal at
    part granularity: when the topology or any branch length changed, every
    part is recomputed (p4_setPrams + p4_treeLogLike after the tree and model
    are pushed, as after a full setCStuff); when only some parts' model
    values changed, just those parts (p4_setPramsPart, that part's pruning
    and p4_partLogLike, p4/chain.py:316-556), the other parts' lnLs kept.
    (p4 re-prunes only the flagged nodes after local and eTBR moves and
    copies every conditional likelihood between its cur and prop trees each
    generation; this evaluator does the full pruning there and no copies.)"""

    wantsIds = True

    def __init__(self, problem):
        self.problem = problem
        self.refs = {}
        self.held = {}
        self.nEvals = 0
        self.nPartUpdates = 0

    def evaluate(self, states, ids=None):
        out = []
        for n, st in enumerate(states):
            key = ids[n] if ids is not None else None
            ref = self.refs.get(key)
            if ref is None:
                ref = self.refs[key] = RefTree(self.problem)
            prev = self.held.get(key) if key is not None else None
            if prev is None or not _same_topology(prev[0], st) or not numpy.array_equal(prev[0].brLen, st.brLen):
                ref.setState(st)
                lnl, pl = ref.logLike()
            else:
                pl = prev[1].copy()
                for p, (a, b) in enumerate(zip(prev[0].parts, st.parts)):
                    if _same_part(a, b):
                        continue
                    c = numpy.ascontiguousarray(b.comps, numpy.double)
                    r = numpy.ascontiguousarray(b.rvals, numpy.double)
                    g = numpy.ascontiguousarray(b.gamma if len(b.gamma) else numpy.zeros(1), numpy.double)
                    ref.lib.ref_setModelValues(ref.h, p, _d(c), _d(r), _d(g), float(b.pInvar), float(b.relRate))
                    pl[p] = ref.lib.ref_partUpdate(ref.h, p)
                    self.nPartUpdates += 1
                lnl = float(pl.sum())
            if key is not None:
                self.held[key] = (st.copy(), numpy.array(pl, copy=True))
            out.append(lnl)
        self.nEvals += len(states)
        return out


def _parallel_ref_worker(conn, problem, cpu):
    if cpu is not None and hasattr(os, "sched_setaffinity"):
        os.sched_setaffinity(0, {cpu})
    ev = RefChainEvaluator(problem)
    while True:
        msg = conn.recv()
        if msg is None:
            break
        try:
            conn.send(("ok", ev.evaluate(msg[0], msg[1])))
        except Exception as ex:     # reported by the parent
            conn.send(("error", repr(ex)))
    conn.close()


class ParallelRefEvaluator(object):
    """RefChainEvaluator over k processes (spawned, one per core when the
    host allows pinning): evaluate(states) hands the states round-robin to
    the workers, each holding its own reference tree of the same problem, and
    returns the lnLs in order -- the chains of a Metropolis-coupled run
    evaluated side by side on the host's cores."""

    def __init__(self, problem, k):
        import multiprocessing as mp
        ctx = mp.get_context("spawn")
        cpus = sorted(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else [None]
        self.k = k
        self.conns, self.procs = [], []
        for i in range(k):
            a, b = ctx.Pipe()
            pr = ctx.Process(target=_parallel_ref_worker, args=(b, problem, cpus[i % len(cpus)]), daemon=True)
            pr.start()
            self.conns.append(a)
            self.procs.append(pr)
        self.nEvals = 0

    wantsIds = True

    def evaluate(self, states, ids=None):
        ids = list(range(len(states))) if ids is None else list(ids)
        jobs = [(states[i::self.k], ids[i::self.k]) for i in range(self.k)]
        for c, j in zip(self.conns, jobs):
            if j[0]:
                c.send(j)
        out = [None] * len(states)
        for i, (c, j) in enumerate(zip(self.conns, jobs)):
            if not j[0]:
                continue
            kind, vals = c.recv()
            if kind != "ok":
                raise RuntimeError("reference worker: %s" % vals)
            for n, v in enumerate(vals):
                out[i + n * self.k] = v
        self.nEvals += len(states)
        return out

    def close(self):
        for c in self.conns:
            try:
                c.send(None)
            except OSError:
                pass
        for pr in self.procs:
            pr.join(timeout=10)
            if pr.is_alive():
                pr.terminate()


# ----------------------------------------------------------------- port
def discrete_gamma(alpha, K):
    out = numpy.zeros(K)
    rc = port_lib().port_discreteGamma(alpha, K, _d(out))
    assert rc == 0
    return out


def bigQ(R, pi):
    dim = len(pi)
    Q = numpy.zeros((dim, dim))
    assert port_lib().port_bigQ(dim, _d(numpy.ascontiguousarray(R, float)),
                                _d(numpy.ascontiguousarray(pi, float)), _d(Q)) == 0
    return Q


def eig_sym(Q, pi):
    dim = len(pi)
    U = numpy.zeros((dim, dim))
    lam = numpy.zeros(dim)
    rc = port_lib().port_eigSym(dim, _d(numpy.ascontiguousarray(Q, float)),
                                _d(numpy.ascontiguousarray(pi, float)), _d(U), _d(lam))
    assert rc == 0
    return U, lam


def pmatrix(U, lam, pi, t):
    dim = len(pi)
    P = numpy.zeros((dim, dim))
    port_lib().port_pmatrix(dim, _d(U), _d(lam), _d(numpy.ascontiguousarray(pi, float)), float(t),
                            _d(P))
    return P


def encode_part(sp, nTax):
    codes = numpy.zeros((nTax, sp.nChar), numpy.int32)
    eq = sp.equateSymbols()
    rc = port_lib().port_encode(nTax, sp.nChar, "".join(sp.sequences).encode(), sp.symbols.encode(),
                                sp.dim, eq.encode(), len(eq), _i(codes))
    assert rc == 0
    return codes


def make_patterns(codes):
    nTax, nChar = codes.shape
    pats = numpy.zeros((nTax, nChar), numpy.int32)
    cnt = numpy.zeros(nChar, numpy.int32)
    spi = numpy.zeros(nChar, numpy.int32)
    c = numpy.ascontiguousarray(codes, numpy.int32)
    n = port_lib().port_makePatterns(nTax, nChar, _i(c), _i(pats), _i(cnt), _i(spi))
    return numpy.ascontiguousarray(pats[:, :n]), cnt[:n].copy(), spi


def equates_matrix(sp):
    eq = sp.equateSymbols()
    m = numpy.zeros((max(len(eq), 1), sp.dim), numpy.int32)
    for k, e in enumerate(eq):
        for j, s in enumerate(sp.symbols):
            m[k, j] = 1 if s in sp.equates[e] else 0
    return m


def invar_sites(pats, sp):
    nTax, n = pats.shape
    eqm = equates_matrix(sp)
    iv = numpy.zeros(n, numpy.int32)
    ia = numpy.zeros((sp.dim, n), numpy.int32)
    port_lib().port_invarSites(nTax, n, sp.dim, eqm.shape[0], _i(eqm),
                               _i(numpy.ascontiguousarray(pats, numpy.int32)), _i(iv), _i(ia))
    return iv, ia


def port_pdecks(problem, pNum, brLen=None):
    """FP64 P decks [nNodes][nCat][dim][dim] from the port's own setPrams."""
    tree = problem.tree
    sp = problem.parts[pNum]
    bl = tree.brLen if brLen is None else brLen
    nG = len(sp.gammaShapes)
    rates = [discrete_gamma(a, sp.nCat) for a in sp.gammaShapes] if nG else [numpy.ones(1)]
    eigs = {}
    decks = numpy.zeros((tree.nNodes, sp.nCat, sp.dim, sp.dim))
    for v in range(tree.nNodes):
        if v == tree.root:
            continue
        key = (int(sp.compNums[v]), int(sp.rMatrixNums[v]))
        if key not in eigs:
            pi = sp.comps[key[0]]
            Q = bigQ(sp.rmats[key[1]], pi)
            eigs[key] = eig_sym(Q, pi) + (pi,)
        U, lam, pi = eigs[key]
        for c in range(sp.nCat):
            r = rates[sp.gdasrvNums[v]][c] if nG else 1.0
            t = bl[v] * r * sp.relRate
            if sp.pInvar != 0.0:
                t = t / (1.0 - sp.pInvar)
            decks[v, c] = pmatrix(U, lam, pi, t)
    return decks


def port_part_loglike64(problem, pNum, brLen=None, decks=None, patLikes=False, catWork=False):
    """The port's reference-semantics FP64 lnL for one part (with patLikes:
    also the pattern likelihoods and site->pattern index; with catWork: also
    the per-category root sums, nPat x nCat)."""
    tree = problem.tree
    sp = problem.parts[pNum]
    codes = encode_part(sp, tree.nLeaves)
    pats, cnt, spi = make_patterns(codes)
    iv, ia = invar_sites(pats, sp)
    if decks is None:
        decks = port_pdecks(problem, pNum, brLen)
    decks = numpy.ascontiguousarray(decks, numpy.double)
    eqm = equates_matrix(sp)
    n = pats.shape[1]
    pl = numpy.zeros(n) if (patLikes or catWork) else None
    cw = numpy.zeros((n, sp.nCat)) if catWork else None
    ints = [numpy.ascontiguousarray(a, numpy.int32) for a in
            (tree.leftChild, tree.sibling, tree.isLeaf, tree.seqNum, tree.postOrder)]
    rootComp = numpy.ascontiguousarray(sp.comps[sp.compNums[tree.root]], numpy.double)
    lnl = port_lib().port_partLogLike64(tree.nNodes, tree.root, *[_i(a) for a in ints], sp.dim,
                                        sp.nCat, n, eqm.shape[0] if sp.equates else 0, _i(eqm),
                                        _i(pats), _i(cnt), _d(decks), _d(rootComp), sp.pInvar,
                                        _i(iv), _i(ia), _d(pl) if pl is not None else None,
                                        _d(cw) if catWork else None)
    if catWork:
        return lnl, pl, spi, cw
    return (lnl, pl, spi) if patLikes else lnl


def philox_uniform(seed, n):
    """The n-th value of the Philox4x32-10 stream of seed, restated in
    Python (Salmon et al., SC 2011): the test-side copy of the generator."""
    M0, M1, W0, W1, MASK = 0xD2511F53, 0xCD9E8D57, 0x9E3779B9, 0xBB67AE85, 0xffffffff
    c = [n & MASK, (n >> 32) & MASK, 0, 0]
    k = [seed & MASK, (seed >> 32) & MASK]
    for _ in range(10):
        p0, p1 = M0 * c[0], M1 * c[2]
        c = [(p1 >> 32) ^ c[1] ^ k[0], p1 & MASK, (p0 >> 32) ^ c[3] ^ k[1], p0 & MASK]
        k = [(k[0] + W0) & MASK, (k[1] + W1) & MASK]
    return c[0] * 2.0 ** -32, c


def port_site_rates(problem, pNum):
    """Per-site posterior mean rate and most likely Gamma category, restating
    p4_partLogLikeSiteRates (Pf/p4_tree.c:1383-1627): work[c] = sum_s pi_s
    cl_root[c][s]; the category is the first argmax of work; the rate is
    sum_c work[c] * (1/nCat) * rate[c] / like, like being the site likelihood.
    The tree's root must be an internal node."""
    sp = problem.parts[pNum]
    lnl, pl, spi, cw = port_part_loglike64(problem, pNum, catWork=True)
    rates = discrete_gamma(float(sp.gammaShapes[0]), sp.nCat)
    freqs = numpy.full(sp.nCat, 1.0 / sp.nCat)
    cats = numpy.argmax(cw, axis=1).astype(numpy.int32)       # first maximum, as the reference's strict >
    rate = (cw * freqs * rates).sum(axis=1) / pl
    return rate[spi], cats[spi]


def port_loglike64(problem, brLen=None):
    parts = [port_part_loglike64(problem, p, brLen) for p in range(len(problem.parts))]
    return float(sum(parts)), parts


def port_prune32(problem, pNum, decks32, eqTab32, ccodes, partialMasks, counts, invMask, cherries=True):
    """FP32 mirror of the fused GPU kernel on the GPU's own FP32 decks
    (cherries: the GPU program's table lookups, which skip the rescale step
    at nodes whose only children are two leaves)."""
    tree = problem.tree
    sp = problem.parts[pNum]
    nT, n = ccodes.shape
    nPartial = eqTab32.shape[1] if eqTab32.ndim == 4 else 0
    ints = [numpy.ascontiguousarray(a, numpy.int32) for a in
            (tree.leftChild, tree.sibling, tree.isLeaf, tree.seqNum)]
    d32 = numpy.ascontiguousarray(decks32, numpy.float32)
    e32 = numpy.ascontiguousarray(eqTab32 if nPartial else numpy.zeros(4, numpy.float32),
                                  numpy.float32)
    cc = numpy.ascontiguousarray(ccodes, numpy.uint8)
    rootComp = numpy.ascontiguousarray(sp.comps[sp.compNums[tree.root]], numpy.double)
    pm = numpy.ascontiguousarray(partialMasks, numpy.uint32)
    im = numpy.ascontiguousarray(invMask, numpy.uint32)
    cnt = numpy.ascontiguousarray(counts, numpy.double)
    like = numpy.zeros(n, numpy.float32)
    exps = numpy.zeros(n, numpy.int32)
    lnl = numpy.zeros(n)
    tot = port_lib().port_partPrune32(tree.nNodes, tree.root, *[_i(a) for a in ints], sp.dim,
                                      sp.nCat, n, nPartial, d32.ctypes.data_as(F),
                                      e32.ctypes.data_as(F), cc.ctypes.data_as(U8), _d(rootComp),
                                      sp.pInvar, pm.ctypes.data_as(U32), im.ctypes.data_as(U32),
                                      _d(cnt), like.ctypes.data_as(F), _i(exps), _d(lnl), int(cherries))
    return tot, like, exps, lnl


# ---------------------------------------------------------------- draws
def philox_uniforms(seed, n0, count):
    """Values n0 .. n0+count-1 of the Philox4x32-10 stream of seed, numpy."""
    MASK = numpy.uint64(0xffffffff)
    n = numpy.arange(n0, n0 + count, dtype=numpy.uint64)
    c0, c1 = n & MASK, n >> numpy.uint64(32)
    c2 = numpy.zeros_like(c0)
    c3 = numpy.zeros_like(c0)
    k0, k1 = numpy.uint64(seed & 0xffffffff), numpy.uint64((seed >> 32) & 0xffffffff)
    for _ in range(10):
        p0 = numpy.uint64(0xD2511F53) * c0
        p1 = numpy.uint64(0xCD9E8D57) * c2
        c0, c1, c2, c3 = ((p1 >> numpy.uint64(32)) ^ c1 ^ k0, p1 & MASK,
                          (p0 >> numpy.uint64(32)) ^ c3 ^ k1, p0 & MASK)
        k0 = (k0 + numpy.uint64(0x9E3779B9)) & MASK
        k1 = (k1 + numpy.uint64(0xBB67AE85)) & MASK
    return c0.astype(numpy.double) * 2.0 ** -32


def preorder(tree):
    """p4's pre-order (p4/tree.py:1752-1800): a node, then its children from
    leftChild along the siblings."""
    out, st = [], [tree.root]
    while st:
        v = st.pop()
        out.append(v)
        kids, c = [], int(tree.leftChild[v])
        while c >= 0:
            kids.append(c)
            c = int(tree.sibling[c])
        st.extend(reversed(kids))
    return out


def _pick(u, cum):
    """First index whose running sum exceeds u (cum: ..., last entry 1.0)."""
    return numpy.argmax(u[:, None] < cum, axis=1)


def port_simulate(problem, seed, decks):
    """p4_simulate without a reference tree (Pf/p4_treeSim.c:14-590), by
    sites in parallel: every decision takes the value of the Philox stream the
    sequential loop would draw for it (categories per part with nCat > 1,
    root states, invariant flags per part with pInvar > 0, then per part, per
    non-root node in pre-order, per variable site).  decks[p]: the P decks,
    nNodes x nCat x dim x dim (row = parent state).  Returns per part the
    nNodes x nChar states."""
    tree = problem.tree
    parts = problem.parts
    pre = [v for v in preorder(tree) if v != tree.root]
    n = 0
    cats = []
    for sp in parts:
        if sp.nCat > 1:
            cats.append(numpy.floor(sp.nCat * philox_uniforms(seed, n, sp.nChar)).astype(int))
            n += sp.nChar
        else:
            cats.append(numpy.zeros(sp.nChar, int))
    states = []
    for sp in parts:
        pi = sp.comps[sp.compNums[tree.root]]
        cum = numpy.cumsum(pi)
        cum[-1] = 1.0
        st = numpy.zeros((tree.nNodes, sp.nChar), int)
        st[tree.root] = _pick(philox_uniforms(seed, n, sp.nChar), cum)
        n += sp.nChar
        states.append(st)
    inv = []
    for sp in parts:
        if sp.pInvar > 0.0:
            inv.append(philox_uniforms(seed, n, sp.nChar) < sp.pInvar)
            n += sp.nChar
        else:
            inv.append(numpy.zeros(sp.nChar, bool))
    for p, sp in enumerate(parts):
        var = ~inv[p]
        nVar = int(var.sum())
        for r, v in enumerate(pre):
            par = int(tree.parent[v])
            ps = states[p][par]
            st = ps.copy()
            idx = numpy.nonzero(var)[0]
            u = philox_uniforms(seed, n + r * nVar, nVar)
            rows = numpy.cumsum(decks[p][v][cats[p][idx], ps[idx]], axis=1)
            rows[:, -1] = 1.0
            st[idx] = _pick(u, rows)
            states[p][v] = st
        n += len(pre) * nVar
    return states


def port_root_cl(problem, pNum):
    """The port's FP64 root CL of part pNum, nCat x dim x nPat."""
    sp = problem.parts[pNum]
    n = make_patterns(encode_part(sp, problem.tree.nLeaves))[0].shape[1]
    out = numpy.zeros((sp.nCat, sp.dim, n))
    port_lib().port_setRootCLOut(_d(out))
    port_part_loglike64(problem, pNum)
    return out


def draw_anc_prep(problem, pNum):
    """(site -> pattern index, invariant-state array) of a part."""
    sp = problem.parts[pNum]
    pats, cnt, spi = make_patterns(encode_part(sp, problem.tree.nLeaves))
    iv, ia = invar_sites(pats, sp)
    return spi, ia


def port_draw_anc(problem, pNum, rootCL, uniforms, sites=None, prep=None):
    """p4_drawAncState (Pf/p4_treeSim.c:591-845) for every site: rootCL is
    nCat x dim x nPat (FP64, unscaled), uniforms one per site.  Returns
    nChar x 4 draws (chState, cat, isInvar, invarState)."""
    sp = problem.parts[pNum]
    tree = problem.tree
    spi, ia = prep if prep is not None else draw_anc_prep(problem, pNum)
    pi = sp.comps[sp.compNums[tree.root]]
    freq = (1.0 / sp.nCat) * (1.0 - sp.pInvar)
    out = numpy.zeros((sp.nChar, 4), numpy.int32)
    for i in (range(sp.nChar) if sites is None else sites):
        k = spi[i]
        terms = [pi[s] * rootCL[c, s, k] * freq for c in range(sp.nCat) for s in range(sp.dim)]
        inv_terms = [(s, pi[s] * sp.pInvar) for s in range(sp.dim) if sp.pInvar and ia[s, k]]
        tot = 0.0
        for x in terms:
            tot += x
        for _, x in inv_terms:
            tot += x
        x = uniforms[i] * tot
        run, got = 0.0, None
        for j, t in enumerate(terms):
            run += t
            if x < run:
                got = (j % sp.dim, j // sp.dim, 0, -1)
                break
        if got is None:
            for s, t in inv_terms:
                run += t
                if x < run:
                    got = (-1, -1, 1, s)
                    break
        out[i] = got if got is not None else (-1, -1, 0, -1)
    return out
