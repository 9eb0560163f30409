"""Nodal embedding of a cut surface in the deformed material.

The reference's MaterialEmbedding (surface.py:825-993) and its CUDA variant
(surface_gpu.py:182-345): the position field of every (surface or material
grid) node for a cut code is the weighted mean of the affine extrapolations
x_p + F_p (node - ref_p) of the node's support particles (tent weights in the
reference configuration) whose codes are compatible with the code and with
the code of the heaviest such particle, so a node whose code is still
unassigned for a cut follows one side instead of bridging the gap.  Nodes
without support may use the second support ring (tent radius 2 h).  Surface
vertices interpolate their own code's field trilinearly over the material
grid cell that holds them.

Supports are built once on the host; fields and vertices are evaluated by
bm_embed_nodes / bm_embed_vertices on the device, in float64 (the default)
or float32.
"""

from dataclasses import dataclass
from functools import cached_property
from itertools import product
import ctypes

import numpy as np

from . import _native
from .geometry import OFFSETS


@dataclass
class Supports:
    """Per-node (point ids, weights) in CSR form; ids ascending within a node."""

    offsets: np.ndarray
    indices: np.ndarray
    weights: np.ndarray

    def __len__(self):
        return len(self.offsets) - 1

    def __getitem__(self, i):
        a, b = self.offsets[i], self.offsets[i + 1]
        return self.indices[a:b], self.weights[a:b]

    def __iter__(self):
        return (self[i] for i in range(len(self)))


@dataclass
class Mesh:
    """A surface mesh: reference vertex positions, triangles, the cut code of
    each vertex, and (for an embedding without a material grid) the 8 node ids
    and trilinear weights of each vertex's cell."""

    reference: np.ndarray
    triangles: np.ndarray
    codes: np.ndarray
    cells: np.ndarray = None
    weights: np.ndarray = None


_NEIGHBOURS = np.array(list(product((-1, 0, 1), repeat=3)), np.int64)


def tent_supports(nodes, points, radius, chunk=4096):
    """Per node, the points whose tent weight prod(max(1 - |p - node| / radius, 0))
    exceeds 1e-12, ascending, with their weights (surface.py:846-884).

    Points are binned in cubes of edge `radius`; a point with positive weight
    differs from the node by less than `radius` on every axis, so it lies in
    one of the 27 cubes around the node's cube.
    """
    nodes = np.asarray(nodes, float).reshape(-1, 3)
    points = np.asarray(points, float).reshape(-1, 3)
    if not len(points) or not len(nodes):
        return Supports(np.zeros(len(nodes) + 1, np.int64), np.zeros(0, np.int64), np.zeros(0))
    low = points.min(0)
    cube = np.floor((points - low) / radius).astype(np.int64)
    dims = cube.max(0) + 1
    key = (cube[:, 0] * dims[1] + cube[:, 1]) * dims[2] + cube[:, 2]
    by_key = np.argsort(key, kind="stable")
    sorted_key = key[by_key]
    counts, ids_out, w_out = [], [], []
    for start in range(0, len(nodes), chunk):
        block = nodes[start:start + chunk]
        home = np.floor((block - low) / radius).astype(np.int64)
        around = home[:, None, :] + _NEIGHBOURS[None]  # (b, 27, 3)
        inside = np.all((around >= 0) & (around < dims), axis=2)
        k = (around[..., 0] * dims[1] + around[..., 1]) * dims[2] + around[..., 2]
        first = np.searchsorted(sorted_key, k, "left")
        size = np.where(inside, np.searchsorted(sorted_key, k, "right") - first, 0).ravel()
        total = int(size.sum())
        owner = np.repeat(np.repeat(np.arange(len(block)), 27), size)
        run_start = np.repeat(first.ravel(), size)
        within = np.arange(total) - np.repeat(np.cumsum(size) - size, size)
        ids = by_key[run_start + within]
        w = np.maximum(1 - np.abs(points[ids] - block[owner]) / radius, 0).prod(axis=1)
        keep = w > 1.0e-12
        owner, ids, w = owner[keep], ids[keep], w[keep]
        order = np.lexsort((ids, owner))
        counts.append(np.bincount(owner, minlength=len(block)))
        ids_out.append(ids[order])
        w_out.append(w[order])
    counts = np.concatenate(counts)
    return Supports(np.r_[0, np.cumsum(counts)], np.concatenate(ids_out), np.concatenate(w_out))


def _codes(values, count):
    a = np.asarray(values)
    if a.shape != (count,) or not np.issubdtype(a.dtype, np.integer) or np.any(a < 0):
        raise ValueError("Cut codes must be nonnegative int64 integers")
    return np.ascontiguousarray(a, dtype=np.int64)


class MaterialEmbedding:
    """Compatible nodal position fields on the device; affine-exact and one-way.

    The reference support is fixed (not a warp of the nearest current
    particles); a node with no compatible support uses, where asked, the
    compatible affine continuation from its second support ring; missing
    support even there is an error for a surface vertex.
    """

    def __init__(self, reference_nodes, particle_reference, spacing, grid_origin=None, grid_cells=None,
                 device="cuda:0", precision="float64"):
        import torch

        if precision not in ("float64", "float32"):
            raise ValueError("Surface precision must be float64 or float32")
        self.nodes = np.asarray(reference_nodes, float)
        self.ref = np.asarray(particle_reference, float)
        self.h = spacing
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("CUDA surface embedding requires a CUDA device")
        self.precision = precision
        self.np_scalar = np.float64 if precision == "float64" else np.float32
        self._scalar = torch.float64 if precision == "float64" else torch.float32
        self.material_grid = None
        if grid_origin is not None:
            self.grid_origin = np.asarray(grid_origin, float)
            self.grid_cells = np.asarray(grid_cells, int)
            grid_nodes = np.array(list(product(*(range(c + 1) for c in self.grid_cells)))) * spacing + self.grid_origin
            self.material_grid = MaterialEmbedding(grid_nodes, particle_reference, spacing, device=device,
                                                   precision=precision)
        self.extension_nodes = 0
        self._lib = _native.lib()
        self._g_nodes = self._upload(self.nodes)
        self._g_ref = self._upload(self.ref)
        self._vertex_reference = None

    def _upload(self, a, dtype=None):
        import torch

        a = np.ascontiguousarray(a)
        if dtype is None:
            dtype = self._scalar if a.dtype.kind == "f" else torch.int32
        return torch.as_tensor(a, device=self.device).to(dtype).contiguous()

    @cached_property
    def support(self):
        return tent_supports(self.nodes, self.ref, self.h)

    @cached_property
    def extension_support(self):
        # the next reference ring: a one-sided affine continuation for display only
        return tent_supports(self.nodes, self.ref, 2 * self.h)

    @cached_property
    def _g_support(self):
        import torch

        s = self.support
        return (self._upload(s.offsets.astype(np.int32), torch.int32), self._upload(s.indices.astype(np.int32), torch.int32),
                self._upload(s.weights))

    @cached_property
    def _g_extension(self):
        import torch

        s = self.extension_support
        return (self._upload(s.offsets.astype(np.int32), torch.int32), self._upload(s.indices.astype(np.int32), torch.int32),
                self._upload(s.weights))

    def _embedding(self, extend):
        e = _native.Embedding()
        e.node_count, e.particle_count = len(self.nodes), len(self.ref)
        e.scalar_bytes = 8 if self.precision == "float64" else 4
        e.nodes, e.reference = self._g_nodes.data_ptr(), self._g_ref.data_ptr()
        e.offsets, e.indices, e.weights = (t.data_ptr() for t in self._g_support)
        if extend:
            e.extra_offsets, e.extra_indices, e.extra_weights = (t.data_ptr() for t in self._g_extension)
        return e

    def _particles(self, x, F, particle_codes):
        x = np.asarray(x, float)
        F = np.asarray(F, float)
        if x.shape != self.ref.shape or F.shape != (len(self.ref), 3, 3) or not np.isfinite(x).all() \
                or not np.isfinite(F).all():
            raise ValueError("Expected finite particle positions and deformation gradients")
        import torch

        codes = self._upload(_codes(particle_codes, len(self.ref)), torch.int64)
        return self._upload(x), self._upload(F.reshape(-1, 9)), codes

    @property
    def _stream(self):
        import torch

        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _evaluate(self, x, F, particle_codes, node_codes=None, code=0, extend=False):
        import torch

        gx, gF, gc = self._particles(x, F, particle_codes)
        node_ptr = None
        if node_codes is not None:
            g_node_codes = self._upload(_codes(node_codes, len(self.nodes)), torch.int64)
            node_ptr = g_node_codes.data_ptr()
        positions = torch.empty((len(self.nodes), 3), dtype=self._scalar, device=self.device)
        gradients = torch.empty((len(self.nodes), 3, 3), dtype=self._scalar, device=self.device)
        extensions = torch.zeros(1, dtype=torch.int32, device=self.device)
        e = self._embedding(extend)
        _native.check(self._lib.bm_embed_nodes(ctypes.byref(e), gx.data_ptr(), gF.data_ptr(), gc.data_ptr(), node_ptr,
                                               int(code), int(extend), positions.data_ptr(), gradients.data_ptr(),
                                               extensions.data_ptr(), self._stream))
        if extend:
            self.extension_nodes += int(extensions.item())
        return positions, gradients

    def field(self, x, F, particle_codes, code):
        """Position field (nodes, 3) for one code, with the second ring where needed; NaN where unsupported."""
        _codes(np.array([code]), 1)
        return self._evaluate(x, F, particle_codes, code=code, extend=True)[0].cpu().numpy().astype(np.float64)

    def node_state(self, x, F, particle_codes, node_codes):
        """(positions (nodes, 3), deformation (nodes, 3, 3)) of each node's own code, first ring only."""
        p, g = self._evaluate(x, F, particle_codes, node_codes=node_codes)
        return p.cpu().numpy().astype(np.float64), g.cpu().numpy().astype(np.float64)

    def vertices(self, mesh, x, F, particle_codes):
        """Deformed positions of the mesh vertices (surface.py:965-993, surface_gpu.py:270-345)."""
        grid = self.material_grid
        if grid is None:
            return self._vertices_on_nodes(mesh, x, F, particle_codes)
        if not len(mesh.reference):
            return np.empty((0, 3))
        import torch

        count = len(mesh.reference)
        if self._vertex_reference is None or not np.array_equal(mesh.reference, self._vertex_reference):
            fractional = (np.asarray(mesh.reference, float) - self.grid_origin) / self.h
            base = np.clip(np.floor(fractional).astype(int), 0, self.grid_cells - 1)
            local = fractional - base
            corners = np.ravel_multi_index((base[:, None, :] + OFFSETS[None]).transpose(2, 0, 1),
                                           tuple(self.grid_cells + 1))
            weights = np.where(OFFSETS[None] == 1, local[:, None, :], 1 - local[:, None, :]).prod(2)
            self._g_corners = self._upload(corners.astype(np.int32), torch.int32)
            self._g_corner_weights = self._upload(weights)
            self._vertex_reference = np.array(mesh.reference, copy=True)
        gx, gF, gc = grid._particles(x, F, particle_codes)
        vertex_codes = self._upload(_codes(mesh.codes, count), torch.int64)
        out = torch.empty((count, 3), dtype=self._scalar, device=self.device)
        counts = torch.zeros(2, dtype=torch.int32, device=self.device)
        e = grid._embedding(True)
        _native.check(self._lib.bm_embed_vertices(ctypes.byref(e), count, vertex_codes.data_ptr(),
                                                  self._g_corners.data_ptr(), self._g_corner_weights.data_ptr(),
                                                  gx.data_ptr(), gF.data_ptr(), gc.data_ptr(), out.data_ptr(),
                                                  counts.data_ptr(), self._stream))
        extended, unsupported = counts.cpu().numpy().tolist()
        grid.extension_nodes += extended
        if unsupported:
            raise RuntimeError("Surface region has no compatible material support; refine reference grid/support")
        return out.cpu().numpy().astype(np.float64)

    def _vertices_on_nodes(self, mesh, x, F, particle_codes):
        # vertices given by node ids and weights of this embedding's own nodes, one field per code
        result = np.empty((len(mesh.reference), 3))
        extended_corners = self.extension_nodes
        for code in np.unique(mesh.codes):
            plain = self._evaluate(x, F, particle_codes, code=int(code))[0].cpu().numpy()
            field = self.field(x, F, particle_codes, int(code))
            extended = np.isnan(plain[:, 0]) & np.isfinite(field[:, 0])
            ids = np.flatnonzero(mesh.codes == code)
            extended_corners += int(extended[mesh.cells[ids]].sum())
            values = field[mesh.cells[ids]]
            weights = mesh.weights[ids]
            if not np.isfinite(values[weights > 1.0e-9]).all():
                raise RuntimeError("Surface region has no compatible material support; refine reference grid/support")
            result[ids] = np.nansum(values * weights[..., None], axis=1)
        self.extension_nodes = extended_corners
        return result


class CudaMaterialEmbedding(MaterialEmbedding):
    """The reference's CUDA embedding entry point (surface_gpu.py:182-210)."""

    @classmethod
    def from_reference(cls, reference, device="cuda:0", precision="float64"):
        grid = reference.material_grid is not None
        return cls(reference.nodes, reference.ref, reference.h, reference.grid_origin if grid else None,
                   reference.grid_cells if grid else None, device=device, precision=precision)
