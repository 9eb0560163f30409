"""CPU ORACLE - test infrastructure, not part of the product.

topology.components (blademaster_warp/topology.py:17-57) restated for the
tests of the device piece count: the graph of the particles and the
(grid node, code) pairs of the stencil nodes each particle weighs
(weight > 0), two pairs at a node linked when their codes are compatible
(topology.py:6-14), labelled by connected components and ranked by the
lowest particle index in each piece.  Pinned to the reference's own cases
(tests/test_topology.py:5-18) and to tests/golden/topology_default_block.npz,
which was written by the reference's function.
"""

import numpy as np


def compatible(a, b):
    """topology.compatible (topology.py:6-14): no digit non-zero in both codes and different."""
    a, b = int(a), int(b)
    while a or b:
        if a % 3 and b % 3 and a % 3 != b % 3:
            return False
        a //= 3
        b //= 3
    return True


def components(nodes, weights, codes):
    """(labels, sizes): piece of each particle and particles per piece (topology.py:17-57)."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components

    nodes, weights = np.asarray(nodes), np.asarray(weights)
    codes = np.asarray(codes, np.int64)
    n = len(codes)
    used = weights > 0
    particle = np.broadcast_to(np.arange(n)[:, None], nodes.shape)[used]
    span = int(codes.max()) + 1 if n else 1
    pair = nodes[used].astype(np.int64) * span + codes[particle]
    pairs, pair_vertex = np.unique(pair, return_inverse=True)
    pair_node, pair_code = pairs // span, pairs % span
    rows, cols = [particle], [n + pair_vertex]
    kinds = np.unique(pair_code)
    for i, a in enumerate(kinds):
        for b in kinds[i + 1:]:
            if not compatible(a, b):
                continue
            at_a, at_b = np.flatnonzero(pair_code == a), np.flatnonzero(pair_code == b)
            _, ia, ib = np.intersect1d(pair_node[at_a], pair_node[at_b], return_indices=True)
            rows.append(n + at_a[ia])
            cols.append(n + at_b[ib])
    rows, cols = np.concatenate(rows), np.concatenate(cols)
    size = n + len(pairs)
    graph = coo_matrix((np.ones(len(rows), np.int8), (rows, cols)), shape=(size, size))
    _, label = connected_components(graph, directed=False)
    label = label[:n]
    lowest = np.full(label.max() + 1, n)
    np.minimum.at(lowest, label, np.arange(n))
    rank = np.empty_like(lowest)
    rank[np.argsort(lowest)] = np.arange(len(lowest))
    labels = rank[label]
    return labels, np.bincount(labels)
