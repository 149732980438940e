"""Seeded synthetic phylogenetic workloads (host side, numpy).

Trees: Yule (pure-birth) random binary trees, unrooted the p4 way (a
trifurcating root), nodes numbered in pre-order from the root, leaves'
seqNum = taxon index in pre-order; branch lengths i.i.d. Exponential.

Models: GTR exchangeabilities ~ Dirichlet(1 x 6) normalised to sum 1 (as
var.rMatrixNormalizeTo1, p4/var.py:287), compositions ~ Dirichlet, protein
exchangeabilities log-normal(sigma) normalised to sum 1, discrete-Gamma
rates with equal-probability bins (bin means), components placed on nodes
the way Tree.setModelComponentsOnNodesRandomly does (p4/tree.py:7347-7420:
each component on at least `forceRepresentation` nodes, the rest random).

Sequences: states drawn from the root composition at the root and from
rows of P(t * rate_cat) down every branch, one Gamma category per site (the
semantics of Pf/p4_treeSim.c:14), then optionally sprinkled with gaps,
'?' and ambiguity codes for edge-case tests.
"""
import numpy

DNA_SYMBOLS = "acgt"
PROTEIN_SYMBOLS = "arndcqeghilkmfpstwyv"
DNA_EQUATES = {"n": "acgt", "m": "ac", "k": "gt", "h": "act", "y": "ct", "v": "acg", "w": "at",
               "d": "agt", "b": "cgt", "r": "ag", "s": "cg"}
PROTEIN_EQUATES = {"b": "dn", "x": PROTEIN_SYMBOLS, "z": "eq"}


class TreeSpec(object):
    """Topology + branch lengths as flat arrays (p4 node numbering)."""

    def __init__(self, parent, leftChild, sibling, isLeaf, seqNum, brLen, root=0):
        self.parent = numpy.asarray(parent, numpy.int32)
        self.leftChild = numpy.asarray(leftChild, numpy.int32)
        self.sibling = numpy.asarray(sibling, numpy.int32)
        self.isLeaf = numpy.asarray(isLeaf, numpy.int32)
        self.seqNum = numpy.asarray(seqNum, numpy.int32)
        self.brLen = numpy.asarray(brLen, numpy.double)
        self.root = int(root)
        self.nNodes = len(self.parent)
        self.nLeaves = int(self.isLeaf.sum())
        self.preOrder, self.postOrder = self._orders()

    def children(self, v):
        c = self.leftChild[v]
        while c >= 0:
            yield int(c)
            c = self.sibling[c]

    def _orders(self):
        pre, post = [], []
        stack = [(self.root, False)]
        while stack:
            v, done = stack.pop()
            if done:
                post.append(v)
                continue
            pre.append(v)
            stack.append((v, True))
            for c in reversed(list(self.children(v))):
                stack.append((c, False))
        return numpy.array(pre, numpy.int32), numpy.array(post, numpy.int32)

    def copy(self):
        return TreeSpec(self.parent.copy(), self.leftChild.copy(), self.sibling.copy(),
                        self.isLeaf.copy(), self.seqNum.copy(), self.brLen.copy(), self.root)

    def kids(self):
        return {v: list(self.children(v)) for v in range(self.nNodes)}

    def with_kids(self, kids):
        """Same node numbers and branch lengths, new child lists."""
        n = self.nNodes
        parent = -numpy.ones(n, numpy.int32)
        left = -numpy.ones(n, numpy.int32)
        sib = -numpy.ones(n, numpy.int32)
        for v, ch in kids.items():
            if ch:
                left[v] = ch[0]
                for a, b in zip(ch[:-1], ch[1:]):
                    sib[a] = b
                for c in ch:
                    parent[c] = v
        return TreeSpec(parent, left, sib, self.isLeaf.copy(), self.seqNum.copy(),
                        self.brLen.copy(), self.root)

    def swapped(self, a, b):
        """Exchange the positions of two disjoint subtrees (an NNI when a and
        b hang on the two ends of one internal edge)."""
        kids = self.kids()
        pa, pb = int(self.parent[a]), int(self.parent[b])
        ia, ib = kids[pa].index(a), kids[pb].index(b)
        kids[pa][ia], kids[pb][ib] = b, a
        return self.with_kids(kids)


class PartSpec(object):
    """One data partition with its model (comps, R matrices, gamma, pInvar)."""

    def __init__(self, dataType, sequences, comps, rmats, gammaShapes, nCat, compNums,
                 rMatrixNums, gdasrvNums, pInvar=0.0, relRate=1.0, equates=None, rSpecs=None):
        self.dataType = dataType
        self.symbols = DNA_SYMBOLS if dataType == "dna" else PROTEIN_SYMBOLS
        self.dim = len(self.symbols)
        self.equates = dict(DNA_EQUATES if dataType == "dna" else PROTEIN_EQUATES) \
            if equates is None else equates
        self.sequences = sequences           # list of str, one per taxon
        self.comps = numpy.ascontiguousarray(comps, numpy.double)
        self.rmats = numpy.ascontiguousarray(rmats, numpy.double)
        self.gammaShapes = numpy.asarray(gammaShapes, numpy.double).reshape(-1)
        self.nCat = int(nCat)
        self.compNums = numpy.asarray(compNums, numpy.int32)
        self.rMatrixNums = numpy.asarray(rMatrixNums, numpy.int32)
        self.gdasrvNums = numpy.asarray(gdasrvNums, numpy.int32)
        self.pInvar = float(pInvar)
        self.relRate = float(relRate)
        # per R matrix, the spec p4_newRMatrix takes: 20 (values in rmats,
        # poked in), or an empirical protein spec (the library fills its
        # values; rmats then holds the same table for the oracle)
        self.rSpecs = [20] * self.rmats.shape[0] if rSpecs is None else [int(x) for x in rSpecs]

    @property
    def nChar(self):
        return len(self.sequences[0])

    def equateSymbols(self):
        return "".join(sorted(self.equates))        # p4/alignment.py:5791-5794

    def equatesTable(self):
        rows = []
        for e in self.equateSymbols():              # p4/alignment.py:5838-5862
            members = self.equates[e]
            rows.append("".join("1" if s in members else "0" for s in self.symbols))
        return "".join(rows)


class Problem(object):
    def __init__(self, tree, parts, name=""):
        self.tree = tree
        self.parts = parts
        self.name = name

    @property
    def nTax(self):
        return self.tree.nLeaves


# ------------------------------------------------------------------ trees
def yule_tree(nTax, rng, meanBrLen=0.1):
    """Yule random tree with nTax leaves, unrooted onto a trifurcating root."""
    if nTax < 3:
        raise ValueError("need at least 3 taxa")
    # rooted binary Yule growth: children lists
    kids = {0: []}
    leaves = [0]
    nxt = 1
    while len(leaves) < nTax:
        i = int(rng.integers(len(leaves)))
        v = leaves[i]
        a, b = nxt, nxt + 1
        nxt += 2
        kids[v] = [a, b]
        kids[a] = []
        kids[b] = []
        leaves[i] = a
        leaves.append(b)
    # unroot: the first internal child of the root becomes the new root
    r = 0
    c0, c1 = kids[r]
    if kids[c0]:
        newRoot, other = c0, c1
    else:
        newRoot, other = c1, c0
    kids[newRoot] = kids[newRoot] + [other]
    del kids[r]
    # renumber in pre-order
    order = []
    stack = [newRoot]
    while stack:
        v = stack.pop()
        order.append(v)
        for c in reversed(kids[v]):
            stack.append(c)
    num = {v: i for i, v in enumerate(order)}
    n = len(order)
    parent = -numpy.ones(n, numpy.int32)
    left = -numpy.ones(n, numpy.int32)
    sib = -numpy.ones(n, numpy.int32)
    isLeaf = numpy.zeros(n, numpy.int32)
    seqNum = -numpy.ones(n, numpy.int32)
    t = 0
    for v in order:
        i = num[v]
        ch = [num[c] for c in kids[v]]
        if ch:
            left[i] = ch[0]
            for a, b in zip(ch[:-1], ch[1:]):
                sib[a] = b
            for c in ch:
                parent[c] = i
        else:
            isLeaf[i] = 1
            seqNum[i] = t
            t += 1
    brLen = rng.exponential(meanBrLen, size=n)
    brLen[0] = 0.0
    brLen = numpy.maximum(brLen, 1e-8)              # var.BRLEN_MIN
    return TreeSpec(parent, left, sib, isLeaf, seqNum, brLen, root=0)


# ------------------------------------------------------------------ models
def random_gtr(rng, dim=4):
    k = dim * (dim - 1) // 2
    vals = rng.dirichlet(numpy.ones(k))
    return sym_from_upper(vals, dim)


def random_lognormal_R(rng, dim=20, sigma=1.0):
    k = dim * (dim - 1) // 2
    vals = numpy.exp(rng.normal(0.0, sigma, size=k))
    vals /= vals.sum()
    return sym_from_upper(vals, dim)


def sym_from_upper(vals, dim):
    R = numpy.ones((dim, dim))
    k = 0
    for i in range(dim - 1):
        for j in range(i + 1, dim):
            R[i, j] = R[j, i] = vals[k]
            k += 1
    return R


def upper_of(R):
    """Upper-triangle values of a symmetric matrix, row-major (i < j)."""
    d = R.shape[0]
    return numpy.array([R[i, j] for i in range(d - 1) for j in range(i + 1, d)])


def _fix(c):
    """Renormalise a composition so |sum - 1| <= 1e-14 as p4 requires."""
    c = numpy.asarray(c, numpy.double) / numpy.sum(c)
    c[numpy.argmax(c)] += 1.0 - c.sum()
    return c


def random_comp(rng, alpha, dim, pivecMin=1e-13):
    c = rng.dirichlet(numpy.full(dim, float(alpha)))
    c = numpy.maximum(c, 10 * pivecMin)
    c /= c.sum()
    # p4 requires |sum - 1| <= 1e-14 (Pf/p4_tree.c:443-449); fix the rounding
    c[numpy.argmax(c)] += 1.0 - c.sum()
    return c


def place_components(rng, nNodes, root, nComps, forceRepresentation=2, includeRoot=True):
    """Component numbers per node as setModelComponentsOnNodesRandomly does."""
    nums = numpy.zeros(nNodes, numpy.int32)
    if nComps == 1:
        return nums
    nodes = [v for v in range(nNodes) if includeRoot or v != root]
    if nComps * forceRepresentation > len(nodes):
        raise ValueError("not enough nodes for forceRepresentation")
    rng.shuffle(nodes)
    for m in range(nComps):
        for _ in range(forceRepresentation):
            nums[nodes.pop()] = m
    for v in nodes:
        nums[v] = int(rng.integers(nComps))
    return nums


def gamma_rates(alpha, nCat):
    """Equal-probability discrete-Gamma(alpha, alpha) bin means (exact quantiles)."""
    if nCat == 1:
        return numpy.ones(1)
    from scipy import special, stats
    cuts = stats.gamma.ppf(numpy.arange(1, nCat) / nCat, a=alpha, scale=1.0 / alpha)
    cdf1 = special.gammainc(alpha + 1.0, cuts * alpha)
    edges = numpy.concatenate([[0.0], cdf1, [1.0]])
    return numpy.diff(edges) * nCat


def pmatrix(R, pi, t):
    """P(t) for the normalised reversible Q = R.diag(pi) (host FP64)."""
    dim = len(pi)
    Q = R * pi[None, :]
    numpy.fill_diagonal(Q, 0.0)
    numpy.fill_diagonal(Q, -Q.sum(axis=1))
    Q = Q / -(pi * numpy.diag(Q)).sum()
    sq = numpy.sqrt(pi)
    S = sq[:, None] * Q / sq[None, :]
    S = 0.5 * (S + S.T)
    lam, U = numpy.linalg.eigh(S)
    P = (U * numpy.exp(lam * t)[None, :]) @ U.T
    P = P / sq[:, None] * sq[None, :]
    return numpy.clip(P, 0.0, None)


# ------------------------------------------------------------------ simulation
def simulate(tree, part, nSites, rng, rates=None):
    """Simulate one partition's sequences on the tree; returns list of str."""
    dim = part.dim
    nCat = part.nCat
    if rates is None:
        rates = [gamma_rates(a, nCat) for a in part.gammaShapes] if nCat > 1 else [numpy.ones(1)]
    cats = rng.integers(nCat, size=nSites)
    states = numpy.zeros((tree.nNodes, nSites), numpy.int8)
    rootPi = part.comps[part.compNums[tree.root]]
    states[tree.root] = _draw(rng, numpy.broadcast_to(numpy.cumsum(rootPi), (nSites, dim)))
    for v in tree.preOrder[1:]:
        v = int(v)
        par = int(tree.parent[v])
        R = part.rmats[part.rMatrixNums[v]]
        pi = part.comps[part.compNums[v]]
        g = part.gdasrvNums[v] if nCat > 1 else 0
        t = tree.brLen[v] * part.relRate
        if part.pInvar:
            t /= 1.0 - part.pInvar
        cum = numpy.stack([numpy.cumsum(pmatrix(R, pi, t * rates[g][c]), axis=1)
                           for c in range(nCat)])            # (nCat, dim, dim)
        states[v] = _draw(rng, cum[cats, states[par]])
    if part.pInvar:
        inv = rng.random(nSites) < part.pInvar
        if inv.any():
            fixed = _draw(rng, numpy.broadcast_to(numpy.cumsum(rootPi), (int(inv.sum()), dim)))
            states[:, inv] = fixed[None, :]
    syms = numpy.frombuffer(part.symbols.encode(), numpy.uint8)
    seqs = [""] * tree.nLeaves
    for v in range(tree.nNodes):
        if tree.isLeaf[v]:
            seqs[tree.seqNum[v]] = syms[states[v]].tobytes().decode()
    return seqs


def _draw(rng, cum):
    u = rng.random(cum.shape[0])[:, None]
    return numpy.minimum((u >= cum).sum(axis=1), cum.shape[1] - 1).astype(numpy.int8)


def sprinkle(seqs, rng, frac, chars):
    """Replace a fraction of characters with gaps / '?' / ambiguity codes."""
    out = []
    pool = numpy.frombuffer(chars.encode(), numpy.uint8)
    for s in seqs:
        a = numpy.frombuffer(s.encode(), numpy.uint8).copy()
        m = rng.random(len(a)) < frac
        a[m] = pool[rng.integers(len(pool), size=int(m.sum()))]
        out.append(a.tobytes().decode())
    return out


# ------------------------------------------------------------------ named workloads
def make_part(tree, rng, dataType, nSites, nComps=1, compAlpha=10.0, gammaShape=0.5, nCat=4,
              nR=1, proteinSigma=1.0, pInvar=0.0, relRate=1.0, ambiguity=0.0):
    dim = 4 if dataType == "dna" else 20
    comps = numpy.stack([random_comp(rng, compAlpha, dim) for _ in range(nComps)])
    if dataType == "dna":
        rmats = numpy.stack([random_gtr(rng, 4) for _ in range(nR)])
    else:
        rmats = numpy.stack([random_lognormal_R(rng, 20, proteinSigma) for _ in range(nR)])
    compNums = place_components(rng, tree.nNodes, tree.root, nComps)
    rNums = place_components(rng, tree.nNodes, tree.root, nR, includeRoot=False)
    gNums = numpy.zeros(tree.nNodes, numpy.int32)
    part = PartSpec(dataType, None, comps, rmats, [gammaShape] if nCat > 1 else [], nCat,
                    compNums, rNums, gNums, pInvar=pInvar, relRate=relRate)
    part.sequences = simulate(tree, part, nSites, rng)
    if ambiguity > 0:
        extra = "-?" + "".join(sorted(part.equates))
        part.sequences = sprinkle(part.sequences, rng, ambiguity, extra)
    return part


CONFIGS = {
    # name: (description) -- seeds 1000 + index
    "dna16": "DNA 16 taxa, 1,000 sites, GTR+G4, homogeneous (CPU-runnable case)",
    "dna64het": "DNA 64 taxa, 100,000 sites, GTR+G4, 4 compositions on random node sets",
    "prot48het": "Protein 48 taxa, 20,000 sites, log-normal R +G4 (0.8), 3 compositions",
    "mcmcmc32": "32 taxa, 12 partitions (8 DNA + 4 protein), 200-30,000 sites each",
    "dna32het6": "DNA 32 taxa, 50,000 sites, 6 compositions + GTR+G4",
}


def make_config(name, seed=None, scale=1.0):
    """Synthetic problem for a named workload; `scale` shrinks site counts."""
    idx = list(CONFIGS).index(name)
    rng = numpy.random.default_rng(1000 + idx if seed is None else seed)
    s = lambda n: max(16, int(round(n * scale)))
    if name == "dna16":
        tree = yule_tree(16, rng)
        parts = [make_part(tree, rng, "dna", s(1000), nComps=1, compAlpha=10.0, gammaShape=0.5)]
    elif name == "dna64het":
        tree = yule_tree(64, rng)
        parts = [make_part(tree, rng, "dna", s(100000), nComps=4, compAlpha=5.0, gammaShape=0.5)]
    elif name == "prot48het":
        tree = yule_tree(48, rng)
        parts = [make_part(tree, rng, "protein", s(20000), nComps=3, compAlpha=2.0,
                           gammaShape=0.8)]
    elif name == "mcmcmc32":
        tree = yule_tree(32, rng)
        lens = numpy.exp(rng.uniform(numpy.log(200), numpy.log(30000), size=12)).astype(int)
        parts = []
        for i, L in enumerate(lens):
            dt = "dna" if i < 8 else "protein"
            parts.append(make_part(tree, rng, dt, s(int(L)), nComps=1,
                                   compAlpha=10.0 if dt == "dna" else 2.0,
                                   gammaShape=0.5 if dt == "dna" else 0.8))
    elif name == "dna32het6":
        tree = yule_tree(32, rng)
        parts = [make_part(tree, rng, "dna", s(50000), nComps=6, compAlpha=5.0, gammaShape=0.5)]
    else:
        raise KeyError(name)
    return Problem(tree, parts, name)


# ------------------------------------------------------------------ save / load
def save_problem(problem, path, **extra):
    """Write a Problem (tree, model, alignment) plus extra arrays to an .npz."""
    t = problem.tree
    d = dict(name=problem.name, nParts=len(problem.parts), parent=t.parent,
             leftChild=t.leftChild, sibling=t.sibling, isLeaf=t.isLeaf, seqNum=t.seqNum,
             brLen=t.brLen, root=t.root)
    for p, sp in enumerate(problem.parts):
        k = "p%d_" % p
        d[k + "dataType"] = sp.dataType
        d[k + "seqs"] = numpy.frombuffer("".join(sp.sequences).encode(), numpy.uint8)
        d[k + "comps"] = sp.comps
        d[k + "rmats"] = sp.rmats
        d[k + "gammaShapes"] = sp.gammaShapes
        d[k + "nCat"] = sp.nCat
        d[k + "compNums"] = sp.compNums
        d[k + "rMatrixNums"] = sp.rMatrixNums
        d[k + "gdasrvNums"] = sp.gdasrvNums
        d[k + "pInvar"] = sp.pInvar
        d[k + "relRate"] = sp.relRate
        d[k + "rSpecs"] = numpy.asarray(sp.rSpecs, numpy.int32)
        d[k + "equates"] = numpy.array(sorted("%s:%s" % kv for kv in sp.equates.items()))
    d.update(extra)
    numpy.savez_compressed(path, **d)


def load_problem(path):
    """Read a Problem written by save_problem; returns (problem, npz dict)."""
    z = numpy.load(path, allow_pickle=False)
    tree = TreeSpec(z["parent"], z["leftChild"], z["sibling"], z["isLeaf"], z["seqNum"],
                    z["brLen"], int(z["root"]))
    parts = []
    for p in range(int(z["nParts"])):
        k = "p%d_" % p
        raw = z[k + "seqs"].tobytes().decode()
        nT = tree.nLeaves
        L = len(raw) // nT
        seqs = [raw[i * L:(i + 1) * L] for i in range(nT)]
        eqs = dict(s.split(":") for s in z[k + "equates"].tolist())
        parts.append(PartSpec(str(z[k + "dataType"]), seqs, z[k + "comps"], z[k + "rmats"],
                              z[k + "gammaShapes"], int(z[k + "nCat"]), z[k + "compNums"],
                              z[k + "rMatrixNums"], z[k + "gdasrvNums"],
                              pInvar=float(z[k + "pInvar"]), relRate=float(z[k + "relRate"]),
                              equates=eqs, rSpecs=z[k + "rSpecs"] if k + "rSpecs" in z else None))
    return Problem(tree, parts, str(z["name"])), z


def tree_from_children(kids, root, brLen=None, rng=None, meanBrLen=0.1):
    """TreeSpec from a {node: [children]} map (any labels); nodes are
    renumbered in pre-order, leaves get seqNum in pre-order."""
    order = []
    stack = [root]
    while stack:
        v = stack.pop()
        order.append(v)
        for c in reversed(kids.get(v, [])):
            stack.append(c)
    num = {v: i for i, v in enumerate(order)}
    n = len(order)
    parent = -numpy.ones(n, numpy.int32)
    left = -numpy.ones(n, numpy.int32)
    sib = -numpy.ones(n, numpy.int32)
    isLeaf = numpy.zeros(n, numpy.int32)
    seqNum = -numpy.ones(n, numpy.int32)
    t = 0
    for v in order:
        i = num[v]
        ch = [num[c] for c in kids.get(v, [])]
        if ch:
            left[i] = ch[0]
            for a, b in zip(ch[:-1], ch[1:]):
                sib[a] = b
            for c in ch:
                parent[c] = i
        else:
            isLeaf[i] = 1
            seqNum[i] = t
            t += 1
    if brLen is None:
        rng = rng or numpy.random.default_rng(0)
        brLen = numpy.maximum(rng.exponential(meanBrLen, size=n), 1e-8)
        brLen[0] = 0.0
    return TreeSpec(parent, left, sib, isLeaf, seqNum, brLen, root=0)
