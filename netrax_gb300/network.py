"""Network descriptions for the netlk C ABI, and the Extended Newick reader.

``NetworkDesc`` holds exactly the arrays of ``netlk_topology`` plus branch
lengths and first-parent probabilities. ``parse_extended_newick`` reads the
reference's Extended Newick dialect (``X#H1:brlen:support:prob``) and numbers
nodes and edges the way the reference's ``Network`` does, so node ids, edge
(pmatrix) ids, reticulation indices and child order match it:

* grammar and defaults: ``src/io/RootedNetworkParser.cpp:59-381`` - missing
  probability 0.5, probabilities clamped to [1e-6, 1-1e-6], branch lengths at
  least 1e-6, a trifurcating top level gets an extra inner node, a unary root
  is dropped;
* numbering: ``src/io/NetworkIO.cpp:39-299`` - tips by their pre-order
  position in the string, inner tree nodes and reticulations in the order of a
  stack DFS from the root (root last among inner tree nodes), tip / inner edge
  id = child node id, reticulation k owns edges ``n_tips+n_inner-1+2k`` (first
  parent) and ``+1`` (second parent); children are ordered by DFS position.
"""
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

BRLEN_MIN, BRLEN_MAX = 1e-6, 100.0
PROB_MIN, PROB_MAX = 1e-6, 1.0 - 1e-6


@dataclass
class NetworkDesc:
    n_tips: int
    root: int
    edge_parent: np.ndarray        # int32 [E]
    edge_child: np.ndarray         # int32 [E]
    node_child_edges: np.ndarray   # int32 [2*N], -1 absent
    ret_node: np.ndarray           # int32 [r]
    ret_first_edge: np.ndarray     # int32 [r]
    ret_second_edge: np.ndarray    # int32 [r]
    branch_lengths: np.ndarray     # float64 [E]
    ret_first_probs: np.ndarray    # float64 [r]
    labels: List[str] = field(default_factory=list)

    @property
    def n_nodes(self):
        return self.node_child_edges.size // 2

    @property
    def n_edges(self):
        return self.edge_parent.size

    @property
    def n_reticulations(self):
        return self.ret_node.size

    def tip_index(self, label):
        return self.labels.index(label)


class _Node:
    def __init__(self, label=""):
        self.label = label
        self.kids = []
        self.parent: Optional["_Node"] = None
        self.length = 0.0
        self.ret = None           # reticulation name
        self.parents = []         # reticulation: [(parent, length, prob), ...]
        self.tip_no = -1
        self.id = -1
        self.ret_no = -1


class _Reader:
    def __init__(self, text):
        self.s = text
        self.i = 0
        self.rets = {}
        self.n_tips = 0
        self.created: List[_Node] = []

    def token(self):
        j = self.i
        while self.i < len(self.s) and self.s[self.i] not in "(),;":
            self.i += 1
        return self.s[j:self.i].strip()

    @staticmethod
    def fields(tok):
        vals = [0.0, 0.0, 0.5]
        parts = tok.split(":")[1:]
        if len(parts) > 3:
            raise ValueError("too many ':' in %r" % tok)
        for k, v in enumerate(parts):
            vals[k] = float(v) if v.strip() else 0.0
        return vals

    def make(self, tok, parent, has_kids):
        head = tok.split(":")[0]
        length, _, prob = self.fields(tok)
        if "#" in head:
            label, name = head.split("#", 1)
            if not name:
                raise ValueError("reticulation without a name")
            node = self.rets.get(name)
            if node is None:
                node = _Node(label)
                node.ret = name
                self.rets[name] = node
                self.created.append(node)
            node.parents.append((parent, length, prob))
            if len(node.parents) > 2:
                raise ValueError("reticulation %s has more than two parents" % name)
            return node
        node = _Node(head)
        node.parent = parent
        node.length = length
        self.created.append(node)
        if not has_kids:
            node.tip_no = self.n_tips
            self.n_tips += 1
        return node

    def subtree(self, parent):
        # the node token follows its children, but the node (and so the first
        # parent of a reticulation) is created before its children are read.
        # Text in front of a '(' is ignored, as the reference's reader does
        # (it takes children between the first '(' and the last ')').
        j = self.i
        while j < len(self.s) and self.s[j] not in "(),;":
            j += 1
        if j < len(self.s) and self.s[j] == "(":
            self.i = j
        if self.i < len(self.s) and self.s[self.i] == "(":
            depth, j = 0, self.i
            while True:
                if j >= len(self.s):
                    raise ValueError("unbalanced ()'s")
                c = self.s[j]
                depth += c == "("
                depth -= c == ")"
                j += 1
                if depth == 0:
                    break
            k = j
            while k < len(self.s) and self.s[k] not in "(),;":
                k += 1
            node = self.make(self.s[j:k].strip(), parent, True)
            self.i += 1
            kids = [self.subtree(node)]
            while self.i < len(self.s) and self.s[self.i] == ",":
                self.i += 1
                kids.append(self.subtree(node))
            if self.i >= len(self.s) or self.s[self.i] != ")":
                raise ValueError("unbalanced ()'s")
            self.i = k
            node.kids.extend(kids)
            for ch in kids:
                if ch.ret is None:
                    ch.parent = node
            return node
        return self.make(self.token(), parent, False)


def parse_extended_newick(text: str) -> NetworkDesc:
    text = text.strip()
    if ";" not in text:
        raise ValueError("No semicolon found")
    rd = _Reader(text[:text.index(";")])
    root = rd.subtree(None)
    for node in rd.created:
        if node.ret is not None:
            if len(node.parents) != 2:
                raise ValueError("reticulation %s needs two parents" % node.ret)
            (p1, l1, q1), (p2, l2, q2) = node.parents
            if q1 == 0 and q2 == 0:
                q1 = q2 = 0.5
            else:
                q1 = min(max(q1, PROB_MIN), PROB_MAX)
                q2 = min(max(q2, PROB_MIN), PROB_MAX)
                if abs(1.0 - (q1 + q2)) >= 1e-3:
                    raise ValueError("invalid sum of reticulation probs in input network")
            node.parents = [(p1, l1, q1), (p2, l2, q2)]
    if len(root.kids) == 3:
        extra = _Node()
        extra.kids = root.kids[1:]
        for ch in extra.kids:
            if ch.ret is None:
                ch.parent = extra
            else:
                node_parents = [(extra if p is root else p, l, q) for p, l, q in ch.parents]
                ch.parents = node_parents
        extra.parent = root
        root.kids = [root.kids[0], extra]
    while len(root.kids) == 1:
        root = root.kids[0]
    if len(root.kids) > 3:
        raise ValueError("The network is not bifurcating")
    # stack DFS
    order, seen, stack = [], set(), [root]
    while stack:
        n = stack.pop()
        if id(n) in seen:
            continue
        seen.add(id(n))
        order.append(n)
        stack.extend(ch for ch in n.kids if id(ch) not in seen)
    pos = {id(n): i for i, n in enumerate(order)}
    tips = [n for n in order if not n.kids]
    for n in tips:
        if n.ret is not None:
            raise ValueError("Found a reticulation node that has no children")
    inner = [n for n in order if n.kids and n.ret is None and n is not root] + [root]
    rets = [n for n in order if n.kids and n.ret is not None]
    nt, ni = len(tips), len(inner)
    for n in tips:
        n.id = n.tip_no
    for k, n in enumerate(inner):
        n.id = nt + k
    for k, n in enumerate(rets):
        n.id = nt + ni + k
        n.ret_no = k
    n_nodes = len(order)
    n_edges = nt + ni - 1 + 2 * len(rets)
    ep = np.full(n_edges, -1, np.int32)
    ec = np.full(n_edges, -1, np.int32)
    bl = np.zeros(n_edges)
    kid_lists = [[] for _ in range(n_nodes)]
    for n in order:
        if n is root:
            continue
        if n.ret is None:
            e = n.id
            ep[e], ec[e], bl[e] = n.parent.id, n.id, n.length
            kid_lists[n.parent.id].append((pos[id(n)], e))
        else:
            base = nt + ni - 1 + 2 * n.ret_no
            for j, (par, length, _) in enumerate(n.parents):
                ep[base + j], ec[base + j], bl[base + j] = par.id, n.id, length
                kid_lists[par.id].append((pos[id(n)], base + j))
    nce = np.full(2 * n_nodes, -1, np.int32)
    for v in range(n_nodes):
        ks = sorted(kid_lists[v], key=lambda x: x[0])
        if len(ks) > 2:
            raise ValueError("node with more than two children")
        for j, (_, e) in enumerate(ks):
            nce[2 * v + j] = e
    bl = np.clip(np.maximum(bl, BRLEN_MIN), BRLEN_MIN, BRLEN_MAX)
    labels = [""] * n_nodes
    for n in tips:
        labels[n.id] = n.label
    r = len(rets)
    return NetworkDesc(
        n_tips=nt, root=root.id, edge_parent=ep, edge_child=ec, node_child_edges=nce,
        ret_node=np.array([n.id for n in rets], np.int32),
        ret_first_edge=np.array([nt + ni - 1 + 2 * k for k in range(r)], np.int32),
        ret_second_edge=np.array([nt + ni + 2 * k for k in range(r)], np.int32),
        branch_lengths=bl,
        ret_first_probs=np.array([n.parents[0][2] for n in rets], np.float64),
        labels=labels)
