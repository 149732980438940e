"""Tree rearrangements with p4's node semantics, and the eTBR proposal.

A tree here is p4's linked form (parent / leftChild / sibling per node, -1
for none) plus, per non-root node, the identity of its branch: p4 keeps a
branch object on the node at the branch's lower end, and that object -- with
its length -- travels with the node when the tree is rearranged.  The
primitives below move branches exactly as p4's do:

  nextNode(spoke, hub)      p4/tree.py:2852 (cycle round a hub's branches)
  getDegree(n)              p4/tree.py:2830
  reRoot(newRoot)           p4/tree.py:3527 (the old root takes the swivel
                            node's branch at each step of the path)
  prune(node)               pruneSubTreeWithoutParent, p4/tree.py:4143
  reconnect(node, parent)   reconnectSubTreeWithoutParent, p4/tree.py:4197
                            (the node becomes the rightmost child)

Child order matters: the random choices of eTBR are made among children and
spokes in this order, so it is kept as p4 keeps it.
"""
import math

from .p4exceptions import P4Error


class LinkedTree(object):
    """A topology in p4's linked form with branches tracked by identity.
    Branch ids are the node numbers of the starting tree; `length[b]` is the
    length of branch b."""

    def __init__(self, parent, leftChild, sibling, root, brLen, isLeaf):
        n = len(parent)
        tl = (lambda a: a.tolist() if hasattr(a, "tolist") else list(a))
        self.parent = [int(x) for x in tl(parent)]
        self.leftChild = [int(x) for x in tl(leftChild)]
        self.sibling = [int(x) for x in tl(sibling)]
        self.root = int(root)
        self.isLeaf = [int(x) for x in tl(isLeaf)]
        self.br = [v if v != self.root else -1 for v in range(n)]
        self.length = [float(x) for x in tl(brLen)]

    # ------------------------------------------------------------ queries
    def children(self, v):
        c = self.leftChild[v]
        while c >= 0:
            yield c
            c = self.sibling[c]

    def nChildren(self, v):
        return sum(1 for _ in self.children(v))

    def rightmostChild(self, v):
        c = self.leftChild[v]
        while self.sibling[c] >= 0:
            c = self.sibling[c]
        return c

    def leftSibling(self, v):
        c = self.leftChild[self.parent[v]]
        if c == v:
            return -1
        while self.sibling[c] != v:
            c = self.sibling[c]
        return c

    def getDegree(self, n):
        """Number of branches meeting at node n (p4/tree.py:2830)."""
        if self.isLeaf[n]:
            if self.parent[n] >= 0:
                return 1
            return 1 if self.leftChild[n] >= 0 else 0
        deg = 1
        if self.parent[n] >= 0:
            deg += 1
        s = self.sibling[self.leftChild[n]]
        while s >= 0:
            deg += 1
            s = self.sibling[s]
        return deg

    def nextNode(self, spoke, hub):
        """The next branch round `hub` after `spoke` (p4/tree.py:2852): the
        spoke's next sibling; after the last child the hub itself (standing
        for the branch to its parent), or the first child when the hub is
        the root; after the hub itself, its first child."""
        if self.parent[spoke] == hub or spoke == hub:
            if spoke == hub:
                return self.leftChild[spoke] if self.leftChild[spoke] >= 0 else hub
            if self.sibling[spoke] >= 0:
                return self.sibling[spoke]
            return hub if self.parent[hub] >= 0 else self.leftChild[hub]
        raise P4Error("nextNode: spoke %d is neither the hub %d nor its child" % (spoke, hub))

    # ------------------------------------------------------------ edits
    def reRoot(self, newRoot):
        """Move the root to newRoot along the path between them; at each step
        the old root hangs under the swivel node as its rightmost child and
        takes the swivel node's branch (p4/tree.py:3527-3730)."""
        if newRoot == self.root:
            return
        if self.nChildren(self.root) == 2:
            raise P4Error("reRoot: the tree has a bifurcating root")
        path = [newRoot]
        p = self.parent[newRoot]
        while p != self.root:
            path.append(p)
            p = self.parent[p]
        while path:
            old = self.root
            sw = path.pop()
            self.parent[old] = sw
            self.br[old] = self.br[sw]
            self.br[sw] = -1
            self.parent[sw] = -1
            if self.leftChild[sw] >= 0:
                self.sibling[self.rightmostChild(sw)] = old
            else:
                self.leftChild[sw] = old
            if self.leftChild[old] == sw:
                self.leftChild[old] = self.sibling[sw]
            else:
                ls = self.leftChild[old]
                while self.sibling[ls] != sw:
                    ls = self.sibling[ls]
                self.sibling[ls] = self.sibling[sw]
            self.sibling[sw] = -1
            self.root = sw

    def prune(self, r):
        """Detach node r (with everything above it and its own branch) from
        its parent (p4/tree.py:4143)."""
        if r == self.root:
            raise P4Error("prune: node %d is the root" % r)
        p = self.parent[r]
        if self.leftChild[p] == r:
            self.leftChild[p] = self.sibling[r]
        else:
            self.sibling[self.leftSibling(r)] = self.sibling[r]
        self.sibling[r] = -1
        self.parent[r] = -1

    def reconnect(self, r, newParent):
        """Attach node r as the rightmost child of newParent (p4/tree.py:4197)."""
        if self.leftChild[newParent] < 0:
            raise P4Error("reconnect: node %d has no children" % newParent)
        self.parent[r] = newParent
        self.sibling[self.rightmostChild(newParent)] = r

    def branchOf(self, a, b):
        """The branch between adjacent nodes a and b."""
        if self.parent[a] == b:
            return self.br[a]
        if self.parent[b] == a:
            return self.br[b]
        raise P4Error("nodes %d and %d are not adjacent" % (a, b))

    # ------------------------------------------------------------ output
    def brLens(self):
        """Per node, the length of its branch (0 at the root)."""
        out = [0.0] * len(self.parent)
        for v in range(len(self.parent)):
            if v != self.root:
                out[v] = self.length[self.br[v]]
        return out


def _extend(t, rng, a0, b0, pExt):
    """One end of eTBR's central branch (p4/chain.py:4227-4340 for the x end,
    :4362-4500 for the y end): from the end a0 of the branch (a0, b0), take
    one step to a random neighbour a1 (not b0), then keep stepping on with
    probability pExt while the current node is internal.  If the walk went
    past a1, regraft: reroot at the last internal node passed (r1), move one
    of a0's other subtrees onto a1, a0 onto r1, and the far node r0 onto a0.

    Returns (unconstrained, rearranged, farUnconstrained, branch a0-a1)."""
    if t.getDegree(a0) == 1:
        return False, False, False, None
    deg = t.getDegree(a0)
    k = int(rng.integers(deg - 1))
    if t.parent[b0] == a0:
        r0 = t.nextNode(b0, a0)
    elif t.parent[a0] == b0:
        r0 = t.nextNode(a0, a0)
    else:
        raise P4Error("eTBR: central branch ends are not adjacent")
    for _ in range(k):
        r0 = t.nextNode(r0, a0)
    if r0 == a0:
        r0 = t.parent[r0]
    a1 = r0
    eA1 = t.branchOf(a0, a1)
    r1 = a0
    r0Deg = t.getDegree(r0)
    r0Uncon = r0Deg > 1
    while r0Uncon:
        if pExt < rng.random():
            break
        k = int(rng.integers(r0Deg - 1))
        if t.parent[r1] == r0:
            nxt = t.nextNode(r1, r0)
        elif t.parent[r0] == r1:
            nxt = t.nextNode(r0, r0)
        else:
            raise P4Error("eTBR: walk left the tree")
        for _ in range(k):
            nxt = t.nextNode(nxt, r0)
        if nxt == r0:
            nxt = t.parent[r0]
        r1, r0 = r0, nxt
        r0Deg = t.getDegree(r0)
        r0Uncon = r0Deg > 1
    if r0 == a1:
        return True, False, r0Uncon, eA1
    t.reRoot(r1)
    if not (t.parent[a0] == a1 and t.parent[b0] == a0 and t.parent[r0] == r1):
        raise P4Error("eTBR: unexpected orientation after rerooting")
    ch = [c for c in t.children(a0) if c != b0]
    pick = ch[0] if len(ch) == 1 else ch[int(rng.integers(len(ch)))]
    t.prune(pick)
    t.reconnect(pick, a1)
    t.prune(a0)
    t.reconnect(a0, r1)
    t.prune(r0)
    t.reconnect(r0, a0)
    return True, True, r0Uncon, eA1


def propose_etbr(t, rng, etbrLambda, etbrPExt, brLenPriorLambda):
    """p4's eTBR move (Chain.proposeETBR_Blaise, p4/chain.py:4128-4709) on a
    LinkedTree, in place: a random branch (x0, y0) with a random direction,
    each end extended and regrafted (_extend), the root put back, then the
    central branch and the first branch of each unconstrained end scaled by
    exp(etbrLambda (u - 0.5)).

    Returns (logPriorRatio, logProposalRatio, topologyChanged); the prior is
    exponential(brLenPriorLambda) on branch lengths."""
    oldRoot = t.root
    n = len(t.parent)
    nonRoot = [v for v in range(n) if v != oldRoot]
    y0 = nonRoot[int(rng.integers(len(nonRoot)))]
    x0 = t.parent[y0]
    if rng.random() >= 0.5:
        x0, y0 = y0, x0
    eA = t.branchOf(x0, y0)
    x0Uncon, xRe, r0Uncon, eX = _extend(t, rng, x0, y0, etbrPExt)
    y0Uncon, yRe, s0Uncon, eY = _extend(t, rng, y0, x0, etbrPExt)
    if t.root != oldRoot:
        t.reRoot(oldRoot)
    lnProp = 0.0
    lnPrior = 0.0
    for e, used in ((eA, True), (eX, x0Uncon), (eY, y0Uncon)):
        if not used:
            continue
        lnM = etbrLambda * (rng.random() - 0.5)
        lnProp += lnM
        v0 = t.length[e]
        v1 = v0 * math.exp(lnM)
        t.length[e] = v1
        lnPrior += -brLenPriorLambda * (v1 - v0)
    # extension ratios for the constrained / unconstrained end cases
    if xRe:
        if y0Uncon:
            if not r0Uncon:
                lnProp += math.log(1.0 - etbrPExt)
        elif r0Uncon:
            lnProp += math.log(1.0 / (1.0 - etbrPExt))
    if yRe:
        if x0Uncon:
            if not s0Uncon:
                lnProp += math.log(1.0 - etbrPExt)
        elif s0Uncon:
            lnProp += math.log(1.0 / (1.0 - etbrPExt))
    return lnPrior, lnProp, bool(xRe or yRe)
