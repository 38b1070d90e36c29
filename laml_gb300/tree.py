"""A small rooted-tree type for the topology search (host side).

It provides the parts of treeswift (treeswift>=1.1.39, the reference's tree
library) that laml_libs/Topology_search.py and Topology_search_parallel.py
use, with the same traversal orders -- preorder pops a stack onto which
children are pushed in order, postorder is the reverse of that walk -- so
that NNI moves, shuffles and newick strings come out in the reference's
order: read_tree_newick, Tree.newick, traverse_preorder / postorder /
leaves, resolve_polytomies, suppress_unifurcations, and the Node methods
child_nodes, get_parent, set_parent, add_child, remove_child, is_leaf,
is_root.
"""
from __future__ import annotations

from collections import deque
from typing import List, Optional


class Node:
    __slots__ = ("label", "edge_length", "children", "parent", "mark", "anchors",
                 "__weakref__")

    def __init__(self, label: Optional[str] = None, edge_length: Optional[float] = None):
        self.label = label
        self.edge_length = edge_length
        self.children: List[Node] = []
        self.parent: Optional[Node] = None
        self.mark = False
        self.anchors = None

    def is_leaf(self) -> bool:
        return not self.children

    def is_root(self) -> bool:
        return self.parent is None

    def child_nodes(self) -> List["Node"]:
        return list(self.children)

    def get_parent(self) -> Optional["Node"]:
        return self.parent

    def set_parent(self, p: Optional["Node"]):
        self.parent = p

    def add_child(self, c: "Node"):
        self.children.append(c)
        c.parent = self

    def remove_child(self, c: "Node"):
        self.children.remove(c)

    def traverse_preorder(self):
        st = [self]
        while st:
            v = st.pop()
            yield v
            st.extend(v.children)

    def traverse_postorder(self):
        s1, s2 = [self], []
        while s1:
            v = s1.pop()
            s2.append(v)
            s1.extend(v.children)
        while s2:
            yield s2.pop()

    def newick(self) -> str:
        out = []
        # iterative writer: (node, next child index)
        st = [(self, 0)]
        while st:
            v, k = st.pop()
            if v.children and k < len(v.children):
                out.append("(" if k == 0 else ",")
                st.append((v, k + 1))
                st.append((v.children[k], 0))
                continue
            if v.children:
                out.append(")")
            if v.label is not None:
                out.append(str(v.label))
            if v.edge_length is not None:
                out.append(":" + repr(float(v.edge_length)))
        return "".join(out)


class Tree:
    def __init__(self, root: Optional[Node] = None):
        self.root = root if root is not None else Node()

    def traverse_preorder(self):
        return self.root.traverse_preorder()

    def traverse_postorder(self):
        return self.root.traverse_postorder()

    def traverse_leaves(self):
        return (v for v in self.root.traverse_preorder() if v.is_leaf())

    def newick(self) -> str:
        return self.root.newick() + ";"

    def resolve_polytomies(self):
        """Binary resolution of every node with more than two children: the
        last two children join under a new zero-length node, repeatedly."""
        q = deque([self.root])
        while q:
            v = q.popleft()
            while len(v.children) > 2:
                c1 = v.children.pop()
                c2 = v.children.pop()
                nn = Node(edge_length=0.0)
                v.add_child(nn)
                nn.add_child(c1)
                nn.add_child(c2)
            q.extend(v.children)

    def suppress_unifurcations(self):
        """Remove nodes with one child, adding their edge length to the child."""
        q = deque([self.root])
        while q:
            v = q.popleft()
            if len(v.children) != 1:
                q.extend(v.children)
                continue
            c = v.children.pop()
            if v.parent is None:
                self.root = c
                c.parent = None
            else:
                p = v.parent
                i = p.children.index(v)
                p.children[i] = c
                c.parent = p
            if v.edge_length is not None:
                c.edge_length = (c.edge_length or 0.0) + v.edge_length
            if c.label is None and v.label is not None:
                c.label = v.label
            q.append(c)


def read_tree_newick(s: str) -> Tree:
    """Parse one newick string (labels, ':length', '[...]' comments)."""
    s = s.strip()
    root = Node()
    cur = root
    stack: List[Node] = []
    i, n = 0, len(s)

    def token(j):
        k = j
        while k < n and s[k] not in ",():;[":
            k += 1
        return s[j:k].strip(), k

    while i < n:
        ch = s[i]
        if ch == "(":
            c = Node()
            cur.add_child(c)
            stack.append(cur)
            cur = c
            i += 1
        elif ch == ",":
            if not stack:
                raise ValueError("newick: ',' outside parentheses")
            c = Node()
            stack[-1].add_child(c)
            cur = c
            i += 1
        elif ch == ")":
            if not stack:
                raise ValueError("newick: unbalanced ')'")
            cur = stack.pop()
            i += 1
        elif ch == ":":
            tok, i = token(i + 1)
            cur.edge_length = float(tok)
        elif ch == ";":
            break
        elif ch == "[":
            j = s.index("]", i)
            i = j + 1
        elif ch.isspace():
            i += 1
        else:
            tok, i = token(i)
            if tok:
                cur.label = tok
    if stack:
        raise ValueError("newick: unbalanced '('")
    return Tree(root)


def find_lcas(tree: Tree, queries):
    """LCA node of each (label, label) query (lca_lib.find_LCAs,
    laml_libs/lca_lib.py:13-94): depths, then both ends climbed to equal
    depth and together.  A query whose labels are missing gives None."""
    depth, by_label = {}, {}
    for v in tree.traverse_preorder():
        depth[v] = 0 if v.parent is None else depth[v.parent] + 1
        if v.label is not None:
            by_label[v.label] = v
    out = []
    for q in queries:
        nodes = [by_label.get(a) for a in q]
        if any(x is None for x in nodes):
            out.append(None)
            continue
        a = nodes[0]
        for b in nodes[1:]:
            x, y = a, b
            while depth[x] > depth[y]:
                x = x.parent
            while depth[y] > depth[x]:
                y = y.parent
            while x is not y:
                x, y = x.parent, y.parent
            a = x
        out.append(a)
    return out
