"""Node objects of the host-side tree, mirroring p4's Node / NodeBranch.

Reference: p4/node.py (Node with nodeNum, parent, leftChild, sibling, isLeaf,
seqNum, br; per-part model numbers on ``node.parts[pNum].compNum`` and
``node.br.parts[pNum].rMatrixNum / gdasrvNum``).
"""


class NodePart(object):
    def __init__(self):
        self.compNum = 0


class NodeBranchPart(object):
    def __init__(self):
        self.rMatrixNum = 0
        self.gdasrvNum = 0


class NodeBranch(object):
    def __init__(self):
        self.len = 0.1
        self.parts = []
        self.lenChanged = False


class Node(object):
    def __init__(self):
        self.nodeNum = -1
        self.name = None
        self.parent = None
        self.leftChild = None
        self.sibling = None
        self.isLeaf = 0
        self.seqNum = -1
        self.br = NodeBranch()
        self.parts = []
        self.cNode = None
        self.flag = 0

    def iterChildren(self):
        ch = self.leftChild
        while ch is not None:
            yield ch
            ch = ch.sibling

    def getNChildren(self):
        return sum(1 for _ in self.iterChildren())

    def rightmostChild(self):
        ch = self.leftChild
        if ch is None:
            return None
        while ch.sibling is not None:
            ch = ch.sibling
        return ch

    def leftSibling(self):
        if self.parent is None:
            return None
        ch = self.parent.leftChild
        if ch is self:
            return None
        while ch.sibling is not self:
            ch = ch.sibling
        return ch

    def __repr__(self):
        return "Node(%i%s)" % (self.nodeNum, (", %s" % self.name) if self.name else "")
