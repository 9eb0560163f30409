"""Reference-configuration particle sampling and trilinear stencils.

Restates ``blademaster_warp/geometry.py`` (levelset 13-33, check_domain 36-44,
grid_cells 47-49, points 52-74, stencil 77-90): two particles per cell and
axis at sub-cell centres (or jittered inside their sub-cells), trilinear node
weights and gradients in the reference configuration.  The values are the
reference's: the same float64 arithmetic, the same particle order
(``itertools.product`` order is C-order over the sub-cell lattice, produced
here by ``np.meshgrid(indexing="ij")`` without any arithmetic), and the same
node numbering (C-order ravel over ``cells + 1``).

Added for the GB300 layout (no reference counterpart): :func:`cell_sort`
(particles ordered by reference cell) and :func:`stencil_table` (the distinct
float32 stencil rows; a regular lattice has eight).
"""

import numpy as np

# DexLab banana demo domain, knife and bevel (geometry.py:6-10).
BANANA_DEMO_SIZE_M = (0.12, 0.06, 0.03)
DEMO_KNIFE_HALF_SIZE_M = (0.0005, 0.04, 0.02)
DEMO_KNIFE_BEVEL_HEIGHT_M = 0.005

SHAPES = ("block", "cylinder", "banana", "hcylinder")


def levelset(x, size, shape):
    """Analytic boundary, negative inside (geometry.py:13-33).

    ``hcylinder`` is a cylinder lying along x on the board (radius
    min(size[1:]) / 2, axis at height size[2] / 2); the reference's
    ``cylinder`` stands on the board along z.
    """
    x = np.asarray(x)
    size = np.asarray(size)
    if shape == "block":
        q = np.abs(x - [0, 0, size[2] / 2]) - size / 2
        return np.linalg.norm(np.maximum(q, 0), axis=-1) + np.minimum(np.max(q, axis=-1), 0)
    if shape == "cylinder":
        return np.maximum(
            np.linalg.norm(x[..., :2], axis=-1) - min(size[:2]) / 2,
            np.abs(x[..., 2] - size[2] / 2) - size[2] / 2,
        )
    if shape == "hcylinder":
        centre = np.stack([x[..., 1], x[..., 2] - size[2] / 2], axis=-1)
        return np.maximum(
            np.linalg.norm(centre, axis=-1) - min(size[1:]) / 2,
            np.abs(x[..., 0]) - size[0] / 2,
        )
    if shape == "banana":
        u = x[..., 0] / (size[0] / 2)
        cy = 0.035 * (u * u - 0.5)
        radius = 0.003 + 0.009 * np.maximum(0, 1 - u * u) ** 0.55
        return np.maximum(
            np.abs(x[..., 0]) - size[0] / 2,
            np.sqrt((x[..., 1] - cy) ** 2 + (x[..., 2] - 0.012) ** 2) - radius,
        )
    raise ValueError(shape)


def check_domain(size, shape):
    """Refuse a banana clipped by the sampling box (geometry.py:36-44)."""
    if shape == "banana":
        u = np.linspace(-1, 1, 10001)
        cy = 0.035 * (u * u - 0.5)
        r = 0.003 + 0.009 * np.maximum(0, 1 - u * u) ** 0.55
        if max(np.max(cy + r), -np.min(cy - r)) > size[1] / 2 + 1.0e-10 or 0.024 > size[2] + 1.0e-10:
            raise ValueError(
                "Banana analytic geometry is clipped by the sampling domain; use y size >= 0.059 m and z >= 0.024 m"
            )


def grid_cells(size, spacing):
    """Cells per axis covering the whole domain (geometry.py:47-49)."""
    return np.ceil(np.asarray(size) / spacing - 1.0e-9).astype(int)


def points(size, spacing, shape, seed=0):
    """Reference particles, their grid origin and cell counts (geometry.py:52-74)."""
    size = np.asarray(size)
    check_domain(size, shape)
    cells = grid_cells(size, spacing)
    origin = -np.array([size[0] / 2, size[1] / 2, 0.0])
    coords = [origin[i] + (np.arange(2 * cells[i]) + 0.5) * spacing / 2 for i in range(3)]
    lattice = np.meshgrid(*coords, indexing="ij")
    x = np.stack([c.reshape(-1) for c in lattice], axis=1)
    if seed:
        x += np.random.default_rng(seed).uniform(-spacing / 4, spacing / 4, size=x.shape)
    if shape in ("banana", "cylinder", "hcylinder"):
        x = x[levelset(x, size, shape) <= 0]
    elif shape == "block":
        x = x[np.all(x - origin <= size, axis=1)]
    else:
        raise ValueError(shape)
    if seed:
        x[:, 2] = spacing / 4 + np.abs(x[:, 2] - spacing / 4)
    return x, origin, cells


# Stencil node offsets in the reference's order: product((0, 1), repeat=3).
OFFSETS = np.array([[a >> 2 & 1, a >> 1 & 1, a & 1] for a in range(8)])


def stencil(reference, origin, spacing, cells):
    """Node ids (N, 8), weights (N, 8) and gradients (N, 8, 3) (geometry.py:77-90)."""
    fractional = (reference - origin) / spacing
    base = np.floor(fractional).astype(int)
    local = fractional - base
    factors = np.where(OFFSETS[None] == 1, local[:, None], 1 - local[:, None])
    w = factors.prod(axis=2)
    g = np.empty((*w.shape, 3))
    for a in range(3):
        other = [b for b in range(3) if b != a]
        g[:, :, a] = (2 * OFFSETS[:, a] - 1)[None] * factors[:, :, other].prod(axis=2) / spacing
    ijk = base[:, None] + OFFSETS[None]
    nodes = np.ravel_multi_index(ijk.transpose(2, 0, 1), tuple(cells + 1))
    return nodes, w, g


def reference_cells(reference, origin, spacing, cells):
    """Linear (C-order) index of each particle's reference cell, and the cell coordinates."""
    base = np.floor((reference - origin) / spacing).astype(np.int64)
    return np.ravel_multi_index(base.T, tuple(cells)), base


def cell_sort(reference, origin, spacing, cells):
    """Particle order used on the device: by reference cell, then by reference index.

    Returns (order, cell_start): ``order[i]`` is the reference index of device
    particle i and ``cell_start`` (cells + 1 entries) the CSR range of each
    cell's particles in device order.  Every float reduction over particles
    sums in this order.
    """
    linear, _ = reference_cells(reference, origin, spacing, cells)
    order = np.argsort(linear, kind="stable")
    counts = np.bincount(linear, minlength=int(np.prod(cells)))
    cell_start = np.zeros(len(counts) + 1, np.int64)
    np.cumsum(counts, out=cell_start[1:])
    return order, cell_start


def stencil_table(weights, gradients):
    """Distinct float32 stencil rows and each particle's row id.

    A regular lattice (seed 0) has exactly eight rows, one per sub-cell
    position; a jittered lattice has one per particle.  Rows are compared
    bit for bit, so table lookups return the reference's float32 values.
    """
    rows = np.concatenate(
        [weights.astype(np.float32).reshape(len(weights), 8), gradients.astype(np.float32).reshape(len(weights), 24)],
        axis=1,
    )
    bits = np.ascontiguousarray(rows).view(np.uint32)
    unique, ids = np.unique(bits, axis=0, return_inverse=True)
    table = unique.view(np.float32)
    return table[:, :8].copy(), table[:, 8:].reshape(-1, 8, 3).copy(), ids.reshape(-1).astype(np.int32)
