"""Mechanical pieces from the reference grid and the cut codes.

Restates ``blademaster_warp/topology.py`` (compatible 6-14, components 17-57).
A cut code is an integer in base 3, one digit per cut: 0 uncut, 1 / 2 the
two sides.  Two codes are compatible unless some digit is non-zero in both
and differs.  Pieces are connected components of the graph whose vertices
are the particles and the (grid node, code) pairs: a particle links to the
pair of each stencil node it weighs, and two pairs at one node link when
their codes are compatible.  Labels are ranked by the lowest particle index
in each piece.
"""

import numpy as np


def compatible(a, b):
    """Ternary compatibility of two cut codes (topology.py:6-14)."""
    a, b = int(a), int(b)
    while a or b:
        x, y = a % 3, b % 3
        if x and y and x != y:
            return False
        a //= 3
        b //= 3
    return True


def digit_masks(codes):
    """Bit masks of the digits equal to 1 and to 2 of each code (vectorised).

    compatible(a, b) is (ones_a & twos_b) == 0 and (twos_a & ones_b) == 0.
    """
    codes = np.asarray(codes, np.int64).copy()
    ones = np.zeros(codes.shape, np.uint64)
    twos = np.zeros(codes.shape, np.uint64)
    bit = 0
    while np.any(codes):
        digit = codes % 3
        ones |= (digit == 1).astype(np.uint64) << np.uint64(bit)
        twos |= (digit == 2).astype(np.uint64) << np.uint64(bit)
        codes //= 3
        bit += 1
    return ones, twos


def components(nodes, weights, codes):
    """Piece label of every particle and the piece sizes (topology.py:17-57)."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components

    nodes = np.asarray(nodes)
    weights = np.asarray(weights)
    codes = np.asarray(codes, np.int64)
    n = len(codes)
    if n == 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    used = weights > 0
    owner = np.broadcast_to(np.arange(n)[:, None], nodes.shape)[used]
    span = int(codes.max()) + 1
    key = nodes[used].astype(np.int64) * span + codes[owner]
    keys, vertex = np.unique(key, return_inverse=True)
    key_node, key_code = keys // span, keys % span
    rows, cols = [owner], [n + vertex.reshape(-1)]
    distinct = np.unique(key_code)
    ones, twos = digit_masks(distinct)
    for i in range(len(distinct)):
        for j in range(i + 1, len(distinct)):
            if (ones[i] & twos[j]) == 0 and (twos[i] & ones[j]) == 0:
                a = np.flatnonzero(key_code == distinct[i])
                b = np.flatnonzero(key_code == distinct[j])
                _, ia, ib = np.intersect1d(key_node[a], key_node[b], return_indices=True)
                rows.append(n + a[ia])
                cols.append(n + b[ib])
    rows, cols = np.concatenate(rows), np.concatenate(cols)
    size = n + len(keys)
    graph = coo_matrix((np.ones(len(rows), np.int8), (rows, cols)), shape=(size, size))
    _, label = connected_components(graph, directed=False)
    label = label[:n]
    first = np.full(label.max() + 1, n)
    np.minimum.at(first, label, np.arange(n))
    rank = np.empty_like(first)
    rank[np.argsort(first, kind="stable")] = np.arange(len(first))
    labels = rank[label]
    return labels, np.bincount(labels)
