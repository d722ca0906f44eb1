"""Minimal stand-in for the third-party ``tensornetwork`` 0.4.3 package.

TEST INFRASTRUCTURE ONLY.  This package exists so that the unmodified OQuPy
reference (which imports ``tensornetwork`` at ``oqupy/process_tensor.py:30``,
``oqupy/system_dynamics.py:22`` and ``oqupy/backends/node_array.py:19-21``)
can run in a container where the real library is not installed.  It is
written from the library's public API semantics, not from its source, and
implements only the surface the TEMPO / PT-TEMPO / compute_dynamics path
touches:

* ``Node`` (``__getitem__``, ``__matmul__``, ``get_tensor``, ``tensor``,
  ``shape``, ``get_rank``, ``reorder_edges``, ``get_all_dangling``)
* ``Edge`` (``__xor__`` = connect, ``dimension``, ``disconnect``)
* ``contract``, ``contract_between``, ``copy``, ``contractors.greedy``
* ``split_node_full_svd`` (numpy's LAPACK gesdd; ``OQUPY_TNSHIM_SVD=gesvd``
  selects LAPACK gesvd) with the relative / absolute truncation rule:
  discard the longest tail of singular values whose 2-norm is
  ``<= max_truncation_err`` (times ``s[0]`` when ``relative``).  The same rule
  is stated inside the reference at ``oqupy/mps_mpo.py:452-457``.

Nothing in the product package may import this module.
"""

import os
from typing import Any, Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import backends  # noqa: F401  (import surface only)
from . import contractors  # noqa: F401


class Edge:
    """An edge between (node1, axis1) and optionally (node2, axis2)."""

    def __init__(self, node1, axis1, node2=None, axis2=None, name=None):
        self.node1 = node1
        self.axis1 = axis1
        self.node2 = node2
        self.axis2 = axis2
        self.name = name if name is not None else "__unnamed_edge__"

    @property
    def dimension(self) -> int:
        return int(self.node1.tensor.shape[self.axis1])

    def is_dangling(self) -> bool:
        return self.node2 is None

    def is_trace(self) -> bool:
        return self.node2 is self.node1

    def __xor__(self, other: "Edge") -> "Edge":
        return connect(self, other)

    def disconnect(self) -> Tuple["Edge", "Edge"]:
        if self.is_dangling():
            raise ValueError("Cannot disconnect a dangling edge.")
        e1 = Edge(self.node1, self.axis1)
        e2 = Edge(self.node2, self.axis2)
        self.node1.edges[self.axis1] = e1
        self.node2.edges[self.axis2] = e2
        return e1, e2

    def _retarget(self, old_node, old_axis, new_node, new_axis):
        if self.node1 is old_node and self.axis1 == old_axis:
            self.node1, self.axis1 = new_node, new_axis
        elif self.node2 is old_node and self.axis2 == old_axis:
            self.node2, self.axis2 = new_node, new_axis
        else:
            raise RuntimeError("edge does not attach to the given node/axis")


class Node:
    """A tensor with one ``Edge`` per axis."""

    def __init__(self, tensor, name=None, axis_names=None, backend=None):
        self.tensor = np.asarray(tensor)
        self.name = name if name is not None else "__unnamed_node__"
        self.backend = backend
        self.edges = [Edge(self, i) for i in range(self.tensor.ndim)]

    # -- access -------------------------------------------------------------
    def __getitem__(self, key):
        if isinstance(key, slice):
            return self.edges[key]
        return self.edges[key]

    def get_tensor(self):
        return self.tensor

    def set_tensor(self, tensor):
        self.tensor = np.asarray(tensor)

    @property
    def shape(self):
        return self.tensor.shape

    def get_rank(self) -> int:
        return self.tensor.ndim

    def get_all_dangling(self) -> List[Edge]:
        return [e for e in self.edges if e.is_dangling()]

    def get_all_edges(self) -> List[Edge]:
        return list(self.edges)

    def reorder_edges(self, edge_order: Sequence[Edge]) -> "Node":
        perm = []
        for e in edge_order:
            found = None
            for i, own in enumerate(self.edges):
                if own is e and i not in perm:
                    found = i
                    break
            if found is None:
                raise ValueError("edge_order contains an edge not on node")
            perm.append(found)
        if len(perm) != len(self.edges):
            raise ValueError("edge_order must list every edge of the node")
        self.tensor = np.transpose(self.tensor, perm)
        old_edges = list(self.edges)
        self.edges = [old_edges[p] for p in perm]
        for new_axis, p in enumerate(perm):
            e = old_edges[p]
            # an edge may attach to this node twice (trace edge)
            if e.node1 is self and e.axis1 == p:
                e.axis1 = new_axis
            elif e.node2 is self and e.axis2 == p:
                e.axis2 = new_axis
        return self

    def __matmul__(self, other: "Node") -> "Node":
        return contract_between(self, other)


def connect(edge1: Edge, edge2: Edge, name=None) -> Edge:
    if not edge1.is_dangling() or not edge2.is_dangling():
        raise ValueError("Both edges must be dangling to connect them.")
    if edge1.dimension != edge2.dimension:
        raise ValueError(
            f"Cannot connect edges of dimension {edge1.dimension} and "
            f"{edge2.dimension}.")
    new = Edge(edge1.node1, edge1.axis1, edge2.node1, edge2.axis1, name=name)
    edge1.node1.edges[edge1.axis1] = new
    edge2.node1.edges[edge2.axis1] = new
    return new


def contract_between(node1: Node, node2: Node, name=None, **kwargs) -> Node:
    """Contract every edge shared by ``node1`` and ``node2``.

    The result keeps the remaining edges of ``node1`` followed by those of
    ``node2`` (``np.tensordot`` order)."""
    if node1 is node2:
        raise ValueError("trace contractions are not supported by the shim")
    ax1, ax2 = [], []
    for i, e in enumerate(node1.edges):
        if e.node1 is node1 and e.node2 is node2 and e.axis1 == i:
            ax1.append(i)
            ax2.append(e.axis2)
        elif e.node2 is node1 and e.node1 is node2 and e.axis2 == i:
            ax1.append(i)
            ax2.append(e.axis1)
    if not ax1:
        # outer product
        tensor = np.tensordot(node1.tensor, node2.tensor, axes=0)
    else:
        tensor = np.tensordot(node1.tensor, node2.tensor, axes=(ax1, ax2))
    new = Node.__new__(Node)
    new.tensor = tensor
    new.name = name if name is not None else "__unnamed_node__"
    new.backend = node1.backend
    new.edges = []
    k = 0
    for i, e in enumerate(node1.edges):
        if i in ax1:
            continue
        e._retarget(node1, i, new, k)
        new.edges.append(e)
        k += 1
    for i, e in enumerate(node2.edges):
        if i in ax2:
            continue
        e._retarget(node2, i, new, k)
        new.edges.append(e)
        k += 1
    return new


def contract(edge: Edge, name=None, axis_names=None) -> Node:
    if edge.is_dangling():
        raise ValueError("Cannot contract a dangling edge.")
    return contract_between(edge.node1, edge.node2, name=name)


def copy(nodes, conjugate: bool = False) -> Tuple[Dict, Dict]:
    """Copy a list of nodes; edges to nodes outside the list dangle."""
    nodes = list(nodes)
    node_dict = {}
    for n in nodes:
        t = np.conj(n.tensor) if conjugate else n.tensor.copy()
        m = Node.__new__(Node)
        m.tensor = t
        m.name = n.name
        m.backend = n.backend
        m.edges = [None] * len(n.edges)
        node_dict[n] = m
    edge_dict = {}
    for n in nodes:
        for i, e in enumerate(n.edges):
            if e in edge_dict:
                continue
            other_in = (e.node2 is not None and e.node2 in node_dict
                        and e.node1 in node_dict)
            if other_in:
                ne = Edge(node_dict[e.node1], e.axis1,
                          node_dict[e.node2], e.axis2, name=e.name)
                node_dict[e.node1].edges[e.axis1] = ne
                node_dict[e.node2].edges[e.axis2] = ne
                edge_dict[e] = ne
            else:
                ne = Edge(node_dict[n], i, name=e.name)
                node_dict[n].edges[i] = ne
                edge_dict[e] = ne
    return node_dict, edge_dict


def replicate_nodes(nodes, conjugate: bool = False):
    node_dict, _ = copy(nodes, conjugate)
    return [node_dict[n] for n in nodes]


def _reachable(nodes):
    return list(nodes)


def split_node_full_svd(
        node: Node,
        left_edges: List[Edge],
        right_edges: List[Edge],
        max_singular_values: Optional[int] = None,
        max_truncation_err: Optional[float] = None,
        relative: Optional[bool] = False,
        left_name=None, middle_name=None, right_name=None,
        left_edge_name=None, right_edge_name=None):
    """Truncated SVD split ``node -> U @ S @ Vh``.

    Returns ``(U, S, Vh, truncated_singular_values)`` with edges
    ``U: left_edges + [u_s]``, ``S: [u_s, s_v]``, ``Vh: [s_v] + right_edges``.
    """
    left_edges = list(left_edges)
    right_edges = list(right_edges)
    order = left_edges + right_edges
    node.reorder_edges(order)
    t = node.tensor
    nl = len(left_edges)
    lshape = t.shape[:nl]
    rshape = t.shape[nl:]
    m = int(np.prod(lshape)) if lshape else 1
    n = int(np.prod(rshape)) if rshape else 1
    mat = t.reshape(m, n)
    if os.environ.get("OQUPY_TNSHIM_SVD", "gesdd") == "gesvd":
        # LAPACK's QR-iteration driver instead of divide-and-conquer: used
        # only to measure how much the reference's own result depends on
        # which (equally valid) SVD algorithm it calls
        import scipy.linalg
        u, s, vh = scipy.linalg.svd(mat, full_matrices=False, lapack_driver="gesvd")
    else:
        u, s, vh = np.linalg.svd(mat, full_matrices=False)
    if max_singular_values is None:
        max_singular_values = s.size
    if max_truncation_err is not None:
        trunc_errs = np.sqrt(np.cumsum(np.square(s[::-1])))
        if relative:
            abs_err = max_truncation_err * s[0]
        else:
            abs_err = max_truncation_err
        num_err = int(np.count_nonzero(trunc_errs > abs_err))
    else:
        num_err = max_singular_values
    keep = min(max_singular_values, num_err)
    s_rest = s[keep:]
    s = s[:keep].astype(t.dtype)
    u = u[:, :keep]
    vh = vh[:keep, :]
    U = Node.__new__(Node)
    U.tensor = u.reshape(tuple(lshape) + (keep,))
    U.name = left_name if left_name is not None else "__unnamed_node__"
    U.backend = node.backend
    U.edges = []
    for k, e in enumerate(left_edges):
        e._retarget(node, k, U, k)
        U.edges.append(e)
    U.edges.append(None)
    S = Node(np.diag(s), backend=node.backend)
    V = Node.__new__(Node)
    V.tensor = vh.reshape((keep,) + tuple(rshape))
    V.name = right_name if right_name is not None else "__unnamed_node__"
    V.backend = node.backend
    V.edges = [None]
    for k, e in enumerate(right_edges):
        e._retarget(node, nl + k, V, 1 + k)
        V.edges.append(e)
    # wire U - S - V
    e_us = Edge(U, nl, S, 0, name=left_edge_name)
    U.edges[nl] = e_us
    S.edges[0] = e_us
    e_sv = Edge(S, 1, V, 0, name=right_edge_name)
    S.edges[1] = e_sv
    V.edges[0] = e_sv
    return U, S, V, s_rest
