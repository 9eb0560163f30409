"""TopoCut topology discovery for the MLS-MPM baseline (Wang et al., CoRL 2025,
Sec. 3.1 and App. 7.6), after blademaster_warp/topocut_topology.py:1-229.

After a cut action: SDF(x) = min_p |x - x_p| - r_p on a voxel grid above the
board, with the knife trajectories of the cuts since the last new piece
forced outside the object; the zero isosurface; Laplacian smoothing;
connected components of the faces; each particle joins the closed surface
with the smallest signed distance below tau (else -1); cluster ids are
combined with the previous ones so earlier pieces stay distinct.

The signed distance field, the isosurface and the cluster assignment run on
the device (bm_topocut_*).  The isosurface comes from marching tetrahedra
(six tetrahedra per voxel cube around one diagonal) rather than marching
cubes: a closed, consistently oriented triangle mesh of the same zero set,
whose pieces are the field's pieces.  Smoothing, face components and the
id bookkeeping are host steps, as in the reference.
"""

from dataclasses import dataclass
import ctypes

import numpy as np

from . import _native


@dataclass(frozen=True)
class TopologyParams:
    # Voxel edge and particle influence radius r_p, in particle spacings (h / 2).
    voxel: float = 0.5
    influence: float = 1.0
    # The carved trajectory is at least this many voxels thick, so the gap it
    # forces survives sampling even where the blade is thinner than a voxel.
    gap_voxels: float = 2.0
    smoothing_alpha: float = 0.5
    smoothing_steps: int = 3
    # tau of Eq. 11, in particle spacings.
    tau: float = 0.5


def _adjacency(faces, n):
    from scipy.sparse import coo_matrix

    a = np.concatenate([faces[:, [0, 1, 2]].ravel(), faces[:, [1, 2, 0]].ravel()])
    b = np.concatenate([faces[:, [1, 2, 0]].ravel(), faces[:, [0, 1, 2]].ravel()])
    adjacency = coo_matrix((np.ones(len(a)), (a, b)), shape=(n, n)).tocsr()
    adjacency.data[:] = 1.0
    return adjacency


def smooth(vertices, faces, alpha, steps):
    """Eq. 10: v_i <- v_i + alpha * (mean of the neighbours - v_i), over the mesh edges."""
    if steps <= 0 or not len(faces):
        return vertices
    adjacency = _adjacency(faces, len(vertices))
    degree = np.maximum(np.asarray(adjacency.sum(1)).ravel(), 1.0)
    for _ in range(steps):
        vertices = vertices + alpha * (adjacency @ vertices / degree[:, None] - vertices)
    return vertices


def face_components(faces, n_vertices):
    """Connected component of each face (through shared vertices)."""
    from scipy.sparse.csgraph import connected_components

    _, vertex_label = connected_components(_adjacency(faces, n_vertices), directed=False)
    return vertex_label[faces[:, 0]]


def nearest_cluster(x, meshes, tau, reach, device="cuda:0"):
    """Label of each point: the mesh [(vertices, faces)] with the smallest signed
    distance below tau, negative inside by winding number, else -1
    (topocut_topology.py:67-78), on the device."""
    import torch

    x = np.ascontiguousarray(x, np.float32).reshape(-1, 3)
    offsets, verts, tris, start = 0, [], [], [0]
    for vertices, faces in meshes:
        verts.append(np.asarray(vertices, np.float32))
        tris.append(np.asarray(faces, np.int32) + offsets)
        offsets += len(vertices)
        start.append(start[-1] + len(faces))
    dev = torch.device(device)
    gv = torch.as_tensor(np.concatenate(verts) if verts else np.zeros((1, 3), np.float32), device=dev)
    gt = torch.as_tensor(np.concatenate(tris) if tris else np.zeros((1, 3), np.int32), device=dev)
    gs = torch.as_tensor(np.asarray(start, np.int32), device=dev)
    gx = torch.as_tensor(x, device=dev)
    labels = torch.zeros(len(x), dtype=torch.int32, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    _native.check(_native.lib().bm_topocut_cluster(gx.data_ptr(), len(x), gv.data_ptr(), gt.data_ptr(), gs.data_ptr(),
                                                   len(meshes), float(tau), float(reach), labels.data_ptr(), stream))
    return labels.cpu().numpy().astype(int)


class TopologyTracker:
    """Cluster ids of the particles, updated after each cut action (topocut_topology.py:117-229)."""

    def __init__(self, n, spacing, half_size, params=TopologyParams(), device="cuda:0"):
        import torch

        self.params = params
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("TopologyTracker runs on a CUDA device")
        self.particle_spacing = spacing / 2
        self.half = np.asarray(half_size, float)
        self.labels = np.zeros(n, int)
        self.meshes = []
        # Trajectories of cut actions that have not yet split off a piece; a piece
        # that needs several cuts (a wedge) is carved by all of them together.
        self.pending = []
        self.unassigned = 0
        self._lib = _native.lib()

    @property
    def _stream(self):
        import torch

        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _tensor(self, shape, dtype):
        import torch

        return torch.zeros(shape, dtype=dtype, device=self.device)

    def _surface(self, x, poses):
        """(vertices (V, 3), faces (T, 3)) of the zero isosurface of the particle SDF."""
        import torch

        prm, s = self.params, self.particle_spacing
        voxel, radius = prm.voxel * s, prm.influence * s
        lower = x.min(0) - radius - 2 * voxel
        upper = x.max(0) + radius + 2 * voxel
        dims = np.ceil((upper - lower) / voxel).astype(int) + 1
        reach = radius + 2 * voxel
        bins = np.maximum(np.ceil((dims - 1) * voxel / reach).astype(int), 1)
        half = self.half.copy()
        half[0] = max(half[0], prm.gap_voxels * voxel / 2)
        g = _native.TopoCutGrid()
        g.dims[:] = [int(d) for d in dims]
        g.bin_dims[:] = [int(b) for b in bins]
        g.lower[:] = [float(v) for v in lower]
        g.voxel, g.radius, g.reach = float(voxel), float(radius), float(reach)
        g.half[:] = [float(v) for v in half]
        pose_t = torch.as_tensor(np.asarray(poses, np.float32).reshape(-1, 7), device=self.device)
        g.pose_count = len(pose_t)
        g.poses = pose_t.data_ptr() if len(pose_t) else None
        gx = torch.as_tensor(np.ascontiguousarray(x, np.float32), device=self.device)
        n_bins = int(np.prod(bins))
        points = int(np.prod(dims))
        cubes = int(np.prod(dims - 1))
        edges = 7 * points
        field = self._tensor(points, torch.float32)
        bin_start = self._tensor(n_bins + 1, torch.int32)
        bin_fill = self._tensor(n_bins, torch.int32)
        items = self._tensor(max(len(x), 1), torch.int32)
        partials = self._tensor(max(edges, n_bins, cubes) // 1024 + 2, torch.int32)
        ticket = self._tensor(1, torch.int32)
        call = lambda name, *args: _native.check(getattr(self._lib, name)(*args))  # noqa: E731
        call("bm_topocut_sdf", ctypes.byref(g), gx.data_ptr(), len(x), field.data_ptr(), bin_start.data_ptr(),
             bin_fill.data_ptr(), items.data_ptr(), partials.data_ptr(), ticket.data_ptr(), self._stream)
        cube_tris = self._tensor(cubes, torch.int32)
        tri_start = self._tensor(cubes, torch.int32)
        edge_used = self._tensor(edges, torch.int32)
        edge_index = self._tensor(edges, torch.int32)
        totals = self._tensor(2, torch.int32)
        call("bm_topocut_count", ctypes.byref(g), field.data_ptr(), cube_tris.data_ptr(), tri_start.data_ptr(),
             edge_used.data_ptr(), edge_index.data_ptr(), partials.data_ptr(), ticket.data_ptr(), totals.data_ptr(),
             self._stream)
        n_tri, n_vert = (int(v) for v in totals.cpu().tolist())
        vertices = self._tensor((max(n_vert, 1), 3), torch.float32)
        faces = self._tensor((max(n_tri, 1), 3), torch.int32)
        if n_tri:
            call("bm_topocut_emit", ctypes.byref(g), field.data_ptr(), tri_start.data_ptr(), edge_used.data_ptr(),
                 edge_index.data_ptr(), vertices.data_ptr(), faces.data_ptr(), self._stream)
        self.field = field.reshape(tuple(int(d) for d in dims))
        self.lower, self.upper = lower, lower + (dims - 1) * voxel
        return vertices[:n_vert].cpu().numpy().astype(float), faces[:n_tri].cpu().numpy().astype(np.int64)

    def reconstruct(self, positions, knife_poses=()):
        """One topology discovery; knife_poses are (position, quaternion xyzw) of the cut's trajectory."""
        import torch

        prm, s = self.params, self.particle_spacing
        x = np.asarray(positions, np.float32)
        before = len(self.pieces())
        self.pending += list(knife_poses)
        poses = [np.r_[np.asarray(p, float), np.asarray(q, float)] for p, q in self.pending]
        vertices, faces = self._surface(x, poses)
        if not len(faces):
            self.labels[:] = -1
            self.meshes = []
            return self.labels
        vertices = smooth(vertices, faces, prm.smoothing_alpha, prm.smoothing_steps)
        face_label = face_components(faces, len(vertices))
        kept, meshes = [], []
        for c in np.unique(face_label):
            used = faces[face_label == c]
            # voids between particles extract as inward-facing closed surfaces
            a, b, d = (vertices[used[:, k]] for k in range(3))
            if np.einsum("ij,ij->i", a, np.cross(b, d)).sum() <= 0.0:
                continue
            kept.append(used)
            keep, local = np.unique(used, return_inverse=True)
            meshes.append((vertices[keep], local.reshape(-1, 3)))
        self.meshes = meshes
        start = np.r_[0, np.cumsum([len(u) for u in kept])].astype(np.int32)
        tri = np.concatenate(kept).astype(np.int32) if kept else np.zeros((1, 3), np.int32)
        # all particles and smoothed vertices lie within these bounds
        reach = float(np.linalg.norm(self.upper - self.lower)) + prm.tau * s
        gv = torch.as_tensor(np.ascontiguousarray(vertices, np.float32), device=self.device)
        gt = torch.as_tensor(tri, device=self.device)
        gs = torch.as_tensor(start, device=self.device)
        gx = torch.as_tensor(np.ascontiguousarray(x, np.float32), device=self.device)
        labels = self._tensor(len(x), torch.int32)
        _native.check(self._lib.bm_topocut_cluster(gx.data_ptr(), len(x), gv.data_ptr(), gt.data_ptr(), gs.data_ptr(),
                                                   len(kept), prm.tau * s, reach, labels.data_ptr(), self._stream))
        cluster = labels.cpu().numpy().astype(int)
        # A new id for every (previous id, cluster) pair; Eq. 11 leaves -1 unassigned.
        assigned = cluster >= 0
        previous = self.labels.copy()
        # A particle left unassigned by an earlier cut (inside its gap) takes the
        # previous id of the nearest particle of its new cluster that had one.
        orphan = assigned & (previous < 0)
        if orphan.any():
            from scipy.spatial import cKDTree

            for c in np.unique(cluster[orphan]):
                known = np.flatnonzero((cluster == c) & (previous >= 0))
                lost = np.flatnonzero(orphan & (cluster == c))
                if len(known):
                    previous[lost] = previous[known[cKDTree(x[known]).query(x[lost])[1]]]
        pair = previous * (len(meshes) + 1) + cluster
        self.labels = np.full(len(x), -1)
        self.labels[assigned] = np.unique(pair[assigned], return_inverse=True)[1]
        self.unassigned = int((~assigned).sum())
        if len(self.pieces()) > before:
            self.pending = []
        return self.labels

    def pieces(self):
        labels = self.labels[self.labels >= 0]
        return np.bincount(labels) if len(labels) else np.zeros(0, int)
