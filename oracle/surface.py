"""CPU ORACLE - test infrastructure, not part of the product.

The reference's CPU MaterialEmbedding (blademaster_warp/surface.py:846-993)
restated in float64 numpy for the tests of the device embedding: tent
supports by brute force over all points, the one-sided compatible support of
a node (surface.py:921-934), node fields with the second ring
(surface.py:936-950), node states (surface.py:952-963) and vertices through
the material grid (surface.py:965-993).  Its own cases come from the
reference's tests (tests/test_surface.py:83-126, 364-393).
"""

from itertools import product

import numpy as np

from .pieces import compatible

CORNERS = np.array([[a >> 2 & 1, a >> 1 & 1, a & 1] for a in range(8)])


def tent_supports(nodes, points, radius):
    """[(ids ascending, weights)] per node: tent weight prod(max(1 - |p - node| / r, 0)) > 1e-12."""
    nodes, points = np.asarray(nodes, float), np.asarray(points, float)
    out = []
    for node in nodes:
        w = np.maximum(1 - np.abs(points - node) / radius, 0).prod(axis=1)
        ids = np.flatnonzero(w > 1.0e-12)
        out.append((ids, w[ids]))
    return out


def one_side(code, ids, w, codes):
    """Compatible support restricted to the side of its heaviest particle (surface.py:921-934)."""
    valid = np.array([compatible(code, c) for c in codes[ids]], dtype=bool)
    ids, w = ids[valid], w[valid]
    if len(ids):
        anchor = codes[ids[np.argmax(w)]]
        keep = np.array([compatible(anchor, c) for c in codes[ids]], dtype=bool)
        ids, w = ids[keep], w[keep]
    return ids, w


class Embedding:
    def __init__(self, nodes, reference, spacing, grid_origin=None, grid_cells=None):
        self.nodes = np.asarray(nodes, float)
        self.ref = np.asarray(reference, float)
        self.h = spacing
        self.grid = None
        if grid_origin is not None:
            self.origin, self.cells = np.asarray(grid_origin, float), np.asarray(grid_cells, int)
            grid_nodes = np.array(list(product(*(range(c + 1) for c in self.cells)))) * spacing + self.origin
            self.grid = Embedding(grid_nodes, reference, spacing)
        self.support = tent_supports(self.nodes, self.ref, spacing)
        self._ring2 = None
        self.extension_nodes = 0

    @property
    def ring2(self):
        if self._ring2 is None:
            self._ring2 = tent_supports(self.nodes, self.ref, 2 * self.h)
        return self._ring2

    def field(self, x, F, codes, code):
        codes = np.asarray(codes, np.int64)
        out = np.full((len(self.nodes), 3), np.nan)
        self.extended = np.zeros(len(self.nodes), bool)
        for i, (ids, w) in enumerate(self.support):
            ids, w = one_side(code, ids, w, codes)
            if not len(ids):
                ids, w = one_side(code, *self.ring2[i], codes)
                if not len(ids):
                    continue
                self.extension_nodes += 1
                self.extended[i] = True
            e = x[ids] + np.einsum("nij,nj->ni", F[ids], self.nodes[i] - self.ref[ids])
            out[i] = (e * w[:, None]).sum(0) / w.sum()
        return out

    def node_state(self, x, F, codes, node_codes):
        codes = np.asarray(codes, np.int64)
        positions = np.full((len(self.nodes), 3), np.nan)
        deformation = np.full((len(self.nodes), 3, 3), np.nan)
        for i, (ids, w) in enumerate(self.support):
            ids, w = one_side(node_codes[i], ids, w, codes)
            if not len(ids):
                continue
            e = x[ids] + np.einsum("nij,nj->ni", F[ids], self.nodes[i] - self.ref[ids])
            positions[i] = (e * w[:, None]).sum(0) / w.sum()
            deformation[i] = (F[ids] * w[:, None, None]).sum(0) / w.sum()
        return positions, deformation

    def vertices(self, reference, vertex_codes, x, F, codes):
        """Vertices at reference positions with their codes, through the material grid."""
        reference = np.asarray(reference, float)
        fractional = (reference - self.origin) / self.h
        base = np.clip(np.floor(fractional).astype(int), 0, self.cells - 1)
        local = fractional - base
        ids = np.ravel_multi_index((base[:, None, :] + CORNERS[None]).transpose(2, 0, 1), tuple(self.cells + 1))
        weights = np.where(CORNERS[None] == 1, local[:, None, :], 1 - local[:, None, :]).prod(2)
        result = np.empty_like(reference)
        grid = self.grid
        corners_extended = grid.extension_nodes
        for code in np.unique(vertex_codes):
            field = grid.field(x, F, codes, int(code))
            at = np.flatnonzero(vertex_codes == code)
            corners_extended += int(grid.extended[ids[at]].sum())
            values, w = field[ids[at]], weights[at]
            if not np.isfinite(values[w > 1.0e-9]).all():
                raise RuntimeError("Surface region has no compatible material support")
            result[at] = np.nansum(values * w[..., None], axis=1)
        grid.extension_nodes = corners_extended
        return result
