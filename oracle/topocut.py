"""CPU ORACLE - test infrastructure, not part of the product.

Brute-force restatements of the TopoCut pieces (blademaster_warp/
topocut_topology.py:31-78) for the tests of the device kernels: the particle
signed distance field with carved knife boxes (every particle, no binning),
and the nearest-cluster assignment (closest point over every triangle, the
winding number from the triangles' solid angles), in float64.
"""

import numpy as np


def quat_rotate_inv(q, v):
    """Rotate v by the inverse of the unit quaternion q = (x, y, z, w)."""
    u, w = -np.asarray(q[:3], float), float(q[3])
    v = np.asarray(v, float)
    t = 2.0 * np.cross(u, v)
    return v + w * t + np.cross(u, t)


def quat_rotate(q, v):
    u, w = np.asarray(q[:3], float), float(q[3])
    v = np.asarray(v, float)
    t = 2.0 * np.cross(u, v)
    return v + w * t + np.cross(u, t)


def box_sdf(v, pos, q, half):
    """topocut_topology.py:31-36 for points v (m, 3)."""
    local = quat_rotate_inv(q, np.asarray(v, float) - pos)
    d = np.abs(local) - half
    outside = np.linalg.norm(np.maximum(d, 0.0), axis=-1)
    return outside + np.minimum(np.max(d, axis=-1), 0.0)


def sdf(x, lower, dims, voxel, radius, reach, poses, half):
    """particle_sdf (topocut_topology.py:39-64) on the voxel points, float64."""
    x = np.asarray(x, float)
    axes = [lower[a] + voxel * np.arange(dims[a]) for a in range(3)]
    v = np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)
    nearest = np.full(len(v), float(reach))
    for start in range(0, len(v), 4096):
        block = v[start:start + 4096]
        d = np.linalg.norm(block[:, None, :] - x[None], axis=2)
        nearest[start:start + 4096] = np.minimum(nearest[start:start + 4096], d.min(1))
    value = np.maximum(nearest - radius, -v[:, 2])
    half = np.asarray(half, float) + [0.0, 0.0, 0.5 * voxel]
    for p in np.asarray(poses, float).reshape(-1, 7):
        centre = p[:3] - quat_rotate(p[3:], [0.0, 0.0, 0.5 * voxel])
        value = np.where(box_sdf(v, centre, p[3:], half) <= 0.0, np.maximum(value, voxel), value)
    return value.reshape(tuple(dims))


def closest_on_triangle(p, a, b, c):
    """Closest point of triangle (a, b, c) to p (region tests on the barycentric coordinates)."""
    ab, ac, ap = b - a, c - a, p - a
    d1, d2 = ab @ ap, ac @ ap
    if d1 <= 0 and d2 <= 0:
        return a
    bp = p - b
    d3, d4 = ab @ bp, ac @ bp
    if d3 >= 0 and d4 <= d3:
        return b
    vc = d1 * d4 - d3 * d2
    if vc <= 0 and d1 >= 0 and d3 <= 0:
        return a + ab * (d1 / (d1 - d3))
    cp = p - c
    d5, d6 = ab @ cp, ac @ cp
    if d6 >= 0 and d5 <= d6:
        return c
    vb = d5 * d2 - d1 * d6
    if vb <= 0 and d2 >= 0 and d6 <= 0:
        return a + ac * (d2 / (d2 - d6))
    va = d3 * d6 - d5 * d4
    if va <= 0 and d4 - d3 >= 0 and d5 - d6 >= 0:
        return b + (c - b) * ((d4 - d3) / ((d4 - d3) + (d5 - d6)))
    s = 1.0 / (va + vb + vc)
    return a + ab * (vb * s) + ac * (vc * s)


def winding_number(p, vertices, faces):
    x, y, z = (vertices[faces[:, k]] - p for k in range(3))
    lx, ly, lz = (np.linalg.norm(a, axis=1) for a in (x, y, z))
    num = np.einsum("ij,ij->i", x, np.cross(y, z))
    den = lx * ly * lz + np.einsum("ij,ij->i", x, y) * lz + np.einsum("ij,ij->i", x, z) * ly \
        + np.einsum("ij,ij->i", y, z) * lx
    return float((2.0 * np.arctan2(num, den)).sum() / (4.0 * np.pi))


def closest_distance(p, a, b, c):
    """Distance from p to each triangle (a[i], b[i], c[i]): closest_on_triangle over arrays."""
    ab, ac, ap = b - a, c - a, p - a
    d1, d2 = np.einsum("ij,ij->i", ab, ap), np.einsum("ij,ij->i", ac, ap)
    bp, cp = p - b, p - c
    d3, d4 = np.einsum("ij,ij->i", ab, bp), np.einsum("ij,ij->i", ac, bp)
    d5, d6 = np.einsum("ij,ij->i", ab, cp), np.einsum("ij,ij->i", ac, cp)
    vc, vb, va = d1 * d4 - d3 * d2, d5 * d2 - d1 * d6, d3 * d6 - d5 * d4
    with np.errstate(divide="ignore", invalid="ignore"):
        s = 1.0 / (va + vb + vc)
        q = a + ab * (vb * s)[:, None] + ac * (vc * s)[:, None]  # face region
        e3 = b + (c - b) * ((d4 - d3) / ((d4 - d3) + (d5 - d6)))[:, None]
        e2 = a + ac * (d2 / (d2 - d6))[:, None]
        e1 = a + ab * (d1 / (d1 - d3))[:, None]
    # the regions in the order closest_on_triangle tests them (first match wins)
    conds = [(d1 <= 0) & (d2 <= 0), (d3 >= 0) & (d4 <= d3), (vc <= 0) & (d1 >= 0) & (d3 <= 0),
             (d6 >= 0) & (d5 <= d6), (vb <= 0) & (d2 >= 0) & (d6 <= 0),
             (va <= 0) & (d4 - d3 >= 0) & (d5 - d6 >= 0)]
    for cond, point in reversed(list(zip(conds, [a, b, e1, c, e2, e3]))):
        q = np.where(cond[:, None], point, q)
    return np.linalg.norm(p - q, axis=1)


def nearest_cluster(x, meshes, tau, reach):
    """topocut_topology.py:67-78: meshes = [(vertices, faces)], labels -1 where no mesh is within tau."""
    out = []
    tris = [tuple(np.asarray(v, float)[np.asarray(f)[:, k]] for k in range(3)) for v, f in meshes]
    for p in np.asarray(x, float):
        best, label = tau, -1
        for m, (vertices, faces) in enumerate(meshes):
            closest = float(closest_distance(p, *tris[m]).min())
            if closest > reach:
                continue
            d = -closest if winding_number(p, np.asarray(vertices, float), np.asarray(faces)) > 0.5 else closest
            if d < best:
                best, label = d, m
        out.append(label)
    return np.array(out)


def signed_volume(vertices, faces):
    a, b, c = (np.asarray(vertices, float)[faces[:, k]] for k in range(3))
    return float(np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0)
