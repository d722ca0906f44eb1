"""Greedy network contraction for the ``tensornetwork`` stand-in.

TEST INFRASTRUCTURE ONLY (see the package docstring)."""

import numpy as np


def _shared(a, b):
    return [e for e in a.edges if (e.node1 is a and e.node2 is b)
            or (e.node1 is b and e.node2 is a)]


def greedy(nodes, output_edge_order=None, ignore_edge_order=False):
    """Contract ``nodes`` pairwise, always taking the connected pair whose
    result is smallest.  Edge order of the result is arbitrary unless
    ``output_edge_order`` is given."""
    from tensornetwork import contract_between
    nodes = list(nodes)
    while len(nodes) > 1:
        best = None
        for i in range(len(nodes)):
            for j in range(i + 1, len(nodes)):
                sh = _shared(nodes[i], nodes[j])
                if not sh:
                    continue
                size = (np.prod(nodes[i].tensor.shape, dtype=float)
                        * np.prod(nodes[j].tensor.shape, dtype=float)
                        / np.prod([e.dimension for e in sh], dtype=float) ** 2)
                if best is None or size < best[0]:
                    best = (size, i, j)
        if best is None:
            # disconnected: outer product of the first two
            best = (0, 0, 1)
        _, i, j = best
        new = contract_between(nodes[i], nodes[j])
        nodes = [n for k, n in enumerate(nodes) if k not in (i, j)] + [new]
    result = nodes[0]
    if output_edge_order is not None:
        result.reorder_edges(output_edge_order)
    return result


def optimal(nodes, output_edge_order=None, ignore_edge_order=False):
    return greedy(nodes, output_edge_order, ignore_edge_order)
