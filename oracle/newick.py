"""Oracle restatement of NetRAX's Extended Newick reader and index assignment.

Test infrastructure only (see ``oracle/__init__.py``).

Grammar (``src/io/RootedNetworkParser.cpp:59-165``): a node token is
``label[#Hname][:brlen[:support[:prob]]]``; missing fields read as 0 except the
probability, which defaults to 0.5. The first occurrence of a reticulation name
in pre-order creates the node and names its *first* parent; the second one adds
the *second* parent (``:100-165``). Tips are numbered in pre-order
(``:260-267``). A trifurcating top level gets an extra bifurcation
(``:272-289``); probabilities are clamped to [1e-6, 1-1e-6] and branch lengths
to at least ``brlen_min`` (``:318-378``).

Index assignment (``src/io/NetworkIO.cpp:39-299``): nodes are collected by a
stack DFS from the root (``:39-59``); tips keep their pre-order index as clv
index, inner tree nodes follow in DFS order with the root last, reticulations
come after them (``:114-185``). Edge (pmatrix) index of a tip or inner tree
node equals its clv index; reticulation ``i`` owns edges
``n_tips + n_inner - 1 + 2i`` (first parent) and ``+1`` (second parent)
(``:165-185``). A node's children are ordered by their position in the DFS order
(the outgoing links are created in that order, ``:187-221``).
"""

from dataclasses import dataclass, field
from typing import List, Optional

BRLEN_MIN = 1.0e-6   # raxml-ng RAXML_BRLEN_MIN, used for NetraxOptions::brlen_min
BRLEN_MAX = 100.0    # raxml-ng RAXML_BRLEN_MAX
BRPROB_MIN = 1.0e-6  # src/NetraxOptions.hpp:102
BRPROB_MAX = 1.0 - 1.0e-6


class _RNode:
    __slots__ = ("label", "is_ret", "ret_name", "parent", "children", "length",
                 "first_parent", "second_parent", "first_len", "second_len",
                 "first_prob", "second_prob", "tip_index", "clv", "ret_index")

    def __init__(self):
        self.label = ""
        self.is_ret = False
        self.ret_name = ""
        self.parent = None
        self.children = []
        self.length = 0.0
        self.first_parent = None
        self.second_parent = None
        self.first_len = 0.0
        self.second_len = 0.0
        self.first_prob = 0.0
        self.second_prob = 0.0
        self.tip_index = -1
        self.clv = -1
        self.ret_index = -1


def _fields(token: str):
    """brlen / support / prob of a token (RootedNetworkParser.cpp:59-83)."""
    res = [0.0, 0.0, 0.5]
    parts = token.split(":")
    vals = parts[1:]
    for i, v in enumerate(vals[:3]):
        res[i] = float(v) if v.strip() else 0.0
    return res


def _split_top(s: str) -> List[str]:
    out, depth, start = [], 0, 0
    for i, c in enumerate(s):
        if c == "(":
            depth += 1
        elif c == ")":
            depth -= 1
        elif c == "," and depth == 0:
            out.append(s[start:i])
            start = i + 1
    out.append(s[start:])
    return out


@dataclass
class OracleNetwork:
    """Indexed network, same numbering as the reference's ``Network``."""
    n_tips: int
    n_nodes: int
    n_edges: int
    n_ret: int
    root: int
    labels: List[str]
    node_is_ret: List[bool]
    children: List[List[int]]          # child node ids, reference order
    child_edges: List[List[int]]       # edge id to each child
    edge_parent: List[int]
    edge_child: List[int]
    edge_length: List[float]
    ret_node: List[int]
    ret_first_edge: List[int]
    ret_second_edge: List[int]
    ret_first_parent: List[int]
    ret_second_parent: List[int]
    ret_first_prob: List[float]
    tree_parent: List[int] = field(default_factory=list)  # -1 for root/rets

    def parents_of(self, node: int) -> List[int]:
        if self.node_is_ret[node]:
            k = self.ret_node.index(node)
            return [self.ret_first_parent[k], self.ret_second_parent[k]]
        p = self.tree_parent[node]
        return [] if p < 0 else [p]


def parse_newick(text: str, brlen_min: float = BRLEN_MIN) -> OracleNetwork:
    text = text.strip()
    semi = text.find(";")
    if semi < 0:
        raise ValueError("No semicolon found")
    body = text[:semi]
    nodes: List[_RNode] = []
    rets = {}
    counters = {"tips": 0, "rets": 0}

    def build(token: str, parent: Optional[_RNode]) -> _RNode:
        if "#" in token:
            h = token.find("#")
            c = token.find(":")
            name = token[h + 1:] if c < 0 else token[h + 1:c]
            if not name:
                raise ValueError("reticulation without a name")
            brl = _fields(token)
            if name in rets:
                node = rets[name]
                node.second_parent = parent
                node.second_len, node.second_prob = brl[0], brl[2]
                return node
            node = _RNode()
            node.is_ret = True
            node.label = token[:h]
            node.ret_name = name
            node.first_parent = parent
            node.first_len, node.first_prob = brl[0], brl[2]
            counters["rets"] += 1
            nodes.append(node)
            rets[name] = node
            return node
        node = _RNode()
        node.parent = parent
        c = token.find(":")
        node.label = token if c < 0 else token[:c]
        node.length = _fields(token)[0]
        nodes.append(node)
        return node

    def read(parent, s):
        lp, rp = s.find("("), s.rfind(")")
        if lp >= 0 and rp >= 0:
            node = build(s[rp + 1:], parent)
            for cs in _split_top(s[lp + 1:rp]):
                child = read(node, cs)
                node.children.append(child)
                if not child.is_ret:
                    child.parent = node
            return node
        if lp < 0 and rp < 0:
            node = build(s, parent)
            if not node.is_ret:
                node.tip_index = counters["tips"]
                counters["tips"] += 1
            return node
        raise ValueError("unbalanced ()'s")

    root = read(None, body)
    for n in nodes:
        if n.is_ret:
            if n.first_prob == 0 and n.second_prob == 0:
                n.first_prob = n.second_prob = 0.5
            else:
                n.first_prob = min(max(n.first_prob, BRPROB_MIN), BRPROB_MAX)
                n.second_prob = min(max(n.second_prob, BRPROB_MIN), BRPROB_MAX)
                if abs(1.0 - (n.first_prob + n.second_prob)) >= 1e-3:
                    raise ValueError("invalid sum of reticulation probs")
    if len(root.children) == 3:  # enforceToplevelBifurcation
        nn = _RNode()
        nn.children = [root.children[1], root.children[2]]
        for ch in nn.children:
            ch.parent = nn
        nn.parent = root
        root.children = [root.children[0], nn]
        nodes.append(nn)
    for n in nodes:
        n.length = max(n.length, brlen_min)
        if n.is_ret:
            n.first_len = max(n.first_len, brlen_min)
            n.second_len = max(n.second_len, brlen_min)
    while len(root.children) == 1:  # makeToplevel
        root = root.children[0]
    if len(root.children) > 3:
        raise ValueError("The network is not bifurcating")

    # collectNodes: stack DFS
    order, seen, stack = [], set(), [root]
    while stack:
        a = stack.pop()
        if id(a) in seen:
            continue
        seen.add(id(a))
        order.append(a)
        for ch in a.children:
            if id(ch) not in seen:
                stack.append(ch)
    tips = [n for n in order if not n.children]
    rets_l = [n for n in order if n.children and n.is_ret]
    inner = [n for n in order if n.children and not n.is_ret and n is not root]
    inner.append(root)
    for n in tips:
        if n.is_ret:
            raise ValueError("Found a reticulation node that has no children")
        n.clv = n.tip_index
    for i, n in enumerate(inner):
        n.clv = len(tips) + i
    for i, n in enumerate(rets_l):
        n.clv = len(tips) + len(inner) + i
        n.ret_index = i
    n_tips, n_nodes = len(tips), len(order)
    n_edges = n_tips + len(inner) - 1 + 2 * len(rets_l)
    by_clv = [None] * n_nodes
    for n in order:
        by_clv[n.clv] = n
    pos = {id(n): i for i, n in enumerate(order)}

    edge_parent = [-1] * n_edges
    edge_child = [-1] * n_edges
    edge_len = [0.0] * n_edges
    tree_parent = [-1] * n_nodes
    for n in order:
        if n is root:
            continue
        if n.is_ret:
            e1 = n_tips + len(inner) - 1 + 2 * n.ret_index
            edge_parent[e1], edge_child[e1], edge_len[e1] = n.first_parent.clv, n.clv, n.first_len
            edge_parent[e1 + 1], edge_child[e1 + 1], edge_len[e1 + 1] = n.second_parent.clv, n.clv, n.second_len
        else:
            e = n.clv
            edge_parent[e], edge_child[e], edge_len[e] = n.parent.clv, n.clv, n.length
            tree_parent[n.clv] = n.parent.clv
    # children ordered by DFS position of the child (outgoing links, NetworkIO.cpp:187-221)
    children = [[] for _ in range(n_nodes)]
    child_edges = [[] for _ in range(n_nodes)]
    for n in order:  # iterate children in DFS order, append to parents
        if n is root:
            continue
        if n.is_ret:
            e1 = n_tips + len(inner) - 1 + 2 * n.ret_index
            children[n.first_parent.clv].append(n.clv)
            child_edges[n.first_parent.clv].append(e1)
            children[n.second_parent.clv].append(n.clv)
            child_edges[n.second_parent.clv].append(e1 + 1)
        else:
            children[n.parent.clv].append(n.clv)
            child_edges[n.parent.clv].append(n.clv)
    del pos
    for i in range(n_nodes):
        for e in child_edges[i]:
            edge_len[e] = min(max(edge_len[e], brlen_min), BRLEN_MAX)
    labels = [by_clv[i].label for i in range(n_nodes)]
    for i in range(n_tips, n_nodes):  # dropInternalTreeNodeNames keeps tips only
        labels[i] = ""
    return OracleNetwork(
        n_tips=n_tips, n_nodes=n_nodes, n_edges=n_edges, n_ret=len(rets_l),
        root=root.clv, labels=labels,
        node_is_ret=[by_clv[i].is_ret for i in range(n_nodes)],
        children=children, child_edges=child_edges,
        edge_parent=edge_parent, edge_child=edge_child, edge_length=edge_len,
        ret_node=[n.clv for n in rets_l],
        ret_first_edge=[n_tips + len(inner) - 1 + 2 * i for i in range(len(rets_l))],
        ret_second_edge=[n_tips + len(inner) - 1 + 2 * i + 1 for i in range(len(rets_l))],
        ret_first_parent=[n.first_parent.clv for n in rets_l],
        ret_second_parent=[n.second_parent.clv for n in rets_l],
        ret_first_prob=[n.first_prob for n in rets_l],
        tree_parent=tree_parent,
    )
