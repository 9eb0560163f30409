"""Mechanical pieces from the reference grid and the cut codes.

Restates ``blademaster_warp/topology.py`` (compatible 6-14, components 17-57)
with its own graph (particles joined through their fields, see components).
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
    """Piece label of every particle and the piece sizes (topology.py:17-57).

    The same pieces as the device union-find (``Solver.components``), found
    on the host: the (node, code) fields of the stencil nodes each particle
    weighs are sorted, every particle joins the lowest-indexed particle of
    each of its fields, and the lowest-indexed particles of two compatible
    fields at one node join each other.  Pieces are the connected components
    of that particle graph, numbered in the order of their lowest particle
    index.
    """
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components

    nodes = np.asarray(nodes)
    codes = np.asarray(codes, np.int64)
    n = len(codes)
    if n == 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    particle, corner = np.nonzero(np.asarray(weights) > 0)
    node = nodes[particle, corner].astype(np.int64)
    code = codes[particle]
    by_field = np.lexsort((particle, code, node))
    node, code, particle = node[by_field], code[by_field], particle[by_field]
    opens = np.ones(len(node), bool)
    opens[1:] = (node[1:] != node[:-1]) | (code[1:] != code[:-1])
    field = np.cumsum(opens) - 1
    leader, field_node, field_code = particle[opens], node[opens], code[opens]
    left, right = [particle], [leader[field]]
    # fields of one node are adjacent: pair each with the ones d places on
    first = np.flatnonzero(np.r_[True, field_node[1:] != field_node[:-1]])
    count = np.diff(np.r_[first, len(field_node)])
    end = np.repeat(first + count, count)
    ones, twos = digit_masks(field_code)
    index = np.arange(len(field_node))
    for d in range(1, int(count.max())):
        a = index[index + d < end]
        b = a + d
        joined = ((ones[a] & twos[b]) == 0) & ((twos[a] & ones[b]) == 0)
        left.append(leader[a[joined]])
        right.append(leader[b[joined]])
    left, right = np.concatenate(left), np.concatenate(right)
    graph = coo_matrix((np.ones(len(left), np.int8), (left, right)), shape=(n, n))
    _, piece = connected_components(graph, directed=False)
    _, lowest = np.unique(piece, return_index=True)  # lowest particle of each piece
    number = np.empty(len(lowest), np.int64)
    number[np.argsort(lowest)] = np.arange(len(lowest))
    labels = number[piece]
    return labels, np.bincount(labels)
