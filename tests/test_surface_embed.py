"""Nodal embedding of a cut surface (surface.py:825-993, surface_gpu.py:11-345).

CPU: the host tent supports against brute force (tests/test_surface.py:364-378
of the reference), the oracle's affine exactness and one-sided nodes
(tests/test_surface.py:83-106, 381-393) and its invalid empty support
(tests/test_surface_gpu.py:81-89).  GPU: bm_embed_nodes /
bm_embed_vertices against the float64 oracle within the reference's own
GPU-vs-CPU tolerance (1e-12, tests/test_surface_gpu.py:20-83), with equal
extension counts, and the affine and cut-face properties on the device.
"""

import numpy as np
import pytest

from blademaster_gb300.geometry import points
from blademaster_gb300.surface import Mesh, tent_supports
from oracle import surface as oracle

SIZE, H = (0.06, 0.03, 0.03), 0.006


def surface_nodes(step=0.003):
    """A padded node lattice over the block (stands in for a surface grid's nodes)."""
    lo = np.array([-SIZE[0] / 2, -SIZE[1] / 2, 0.0]) - step
    hi = np.array([SIZE[0] / 2, SIZE[1] / 2, SIZE[2]]) + step
    axes = [np.arange(lo[i], hi[i] + step / 2, step) for i in range(3)]
    return np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)


def mesh_points(count, seed, codes_of=None):
    rng = np.random.default_rng(seed)
    lo = np.array([-SIZE[0] / 2, -SIZE[1] / 2, 0.0]) + 0.0005
    hi = np.array([SIZE[0] / 2, SIZE[1] / 2, SIZE[2]]) - 0.0005
    reference = rng.uniform(lo, hi, (count, 3))
    codes = np.zeros(count, np.int64) if codes_of is None else codes_of(reference)
    return Mesh(reference, np.zeros((0, 3), int), codes)


# ------------------------------------------------------------------- CPU


def test_bucketed_tent_supports_match_brute_force():
    rng = np.random.default_rng(3)
    particles = rng.uniform(-0.02, 0.02, (700, 3))
    nodes = np.r_[rng.uniform(-0.03, 0.03, (300, 3)), [[0.5, 0.0, 0.0]]]
    for radius in (0.004, 0.008):
        support = tent_supports(nodes, particles, radius, chunk=64)
        assert len(support) == len(nodes)
        for (ids, w), (want_ids, want_w) in zip(support, oracle.tent_supports(nodes, particles, radius)):
            np.testing.assert_array_equal(ids, want_ids)
            np.testing.assert_allclose(w, want_w, rtol=0, atol=1.0e-15)


def test_oracle_embedding_is_affine_exact_and_separates_cut_faces():
    ref, origin, cells = points(SIZE, H, "block")
    emb = oracle.Embedding(surface_nodes(), ref, H, origin, cells)
    mesh = mesh_points(200, 1)
    A = np.array([[1, 0.1, 0], [0, 1.2, 0], [0, 0, 0.9]])
    t = np.array([0.1, 0.2, 0.3])
    F = np.tile(A, (len(ref), 1, 1))
    got = emb.vertices(mesh.reference, mesh.codes, ref @ A.T + t, F, np.zeros(len(ref), int))
    np.testing.assert_allclose(got, mesh.reference @ A.T + t, atol=1.0e-10)
    codes = np.where(ref[:, 0] < 0, 1, 2)
    x = ref.copy()
    x[:, 0] += np.where(codes == 1, -0.003, 0.003)
    mesh = mesh_points(200, 2, lambda r: np.where(r[:, 0] < 0, 1, 2))
    moved = emb.vertices(mesh.reference, mesh.codes, x, np.tile(np.eye(3), (len(ref), 1, 1)), codes)
    for code, dx in [(1, -0.003), (2, 0.003)]:
        sel = mesh.codes == code
        np.testing.assert_allclose(moved[sel, 0], mesh.reference[sel, 0] + dx, atol=1.0e-10)


def test_oracle_unassigned_node_follows_one_side():
    ref, origin, cells = points(SIZE, H, "block")
    nodes = surface_nodes()
    emb = oracle.Embedding(nodes, ref, H)
    codes = np.where(ref[:, 0] < 0, 1, 2)
    x = ref + np.where(ref[:, :1] < 0, -0.03, 0.03) * np.array([1.0, 0.0, 0.0])
    positions, _ = emb.node_state(x, np.tile(np.eye(3), (len(ref), 1, 1)), codes, np.zeros(len(nodes), np.int64))
    shift = np.abs(positions[:, 0] - nodes[:, 0])
    ok = np.isfinite(shift)
    assert ok.sum() > len(nodes) // 2
    np.testing.assert_allclose(shift[ok], 0.03, atol=1.0e-12)


def test_empty_support_stays_invalid_instead_of_freezing_or_zeroing():
    # tests/test_surface_gpu.py:81-89: code 1 opposes every particle (all carry code 2), so no node has
    # support for it: the oracle's field is NaN everywhere, and the product refuses a negative code on the
    # host before any device call
    from blademaster_gb300.surface import _codes

    ref, _, _ = points(SIZE, H, "block")
    emb = oracle.Embedding(surface_nodes(), ref, H)
    field = emb.field(ref.copy(), np.tile(np.eye(3), (len(ref), 1, 1)), np.full(len(ref), 2), 1)
    assert np.isnan(field).all()
    with pytest.raises(ValueError):
        _codes(np.array([-1]), 1)


# ------------------------------------------------------------------- GPU


def _pair(precision="float64"):
    from blademaster_gb300.surface import MaterialEmbedding

    ref, origin, cells = points(SIZE, H, "block")
    nodes = surface_nodes()
    return ref, nodes, oracle.Embedding(nodes, ref, H, origin, cells), \
        MaterialEmbedding(nodes, ref, H, origin, cells, precision=precision)


@pytest.mark.gpu
def test_gpu_node_fields_match_oracle_for_intersecting_cuts():
    ref, nodes, cpu, gpu = _pair()
    rng = np.random.default_rng(414)
    F = np.tile(np.eye(3), (len(ref), 1, 1)) + rng.normal(0, 0.03, (len(ref), 3, 3))
    for axis in (0, 1):
        codes = np.where(ref[:, 0] < 0, 1, 2) + 3 * np.where(ref[:, axis] < 0.002, 1, 2)
        node_codes = np.where(nodes[:, 0] < 0, 1, 2)
        x = ref + rng.normal(0, 0.002, ref.shape)
        for a, b in zip(cpu.node_state(x, F, codes, node_codes), gpu.node_state(x, F, codes, node_codes)):
            np.testing.assert_allclose(b, a, rtol=1.0e-12, atol=1.0e-12, equal_nan=True)
        for code in (0, 1, 2, 4, 5, 7, 8):
            cpu.extension_nodes = gpu.extension_nodes = 0
            np.testing.assert_allclose(gpu.field(x, F, codes, code), cpu.field(x, F, codes, code), rtol=1.0e-12,
                                       atol=1.0e-12, equal_nan=True)
            assert gpu.extension_nodes == cpu.extension_nodes


@pytest.mark.gpu
def test_gpu_vertices_match_oracle_after_two_crossing_cuts():
    ref, nodes, cpu, gpu = _pair()
    rng = np.random.default_rng(7)
    codes = np.where(ref[:, 0] < 0, 1, 2) + 3 * np.where(ref[:, 1] < 0.002, 1, 2)
    mesh = mesh_points(3000, 8, lambda r: np.where(r[:, 0] < 0, 1, 2) + 3 * np.where(r[:, 1] < 0.002, 1, 2))
    x = ref + rng.normal(0, 0.001, ref.shape)
    F = np.tile(np.eye(3), (len(ref), 1, 1)) + rng.normal(0, 0.03, (len(ref), 3, 3))
    cpu.grid.extension_nodes = gpu.material_grid.extension_nodes = 0
    want = cpu.vertices(mesh.reference, mesh.codes, x, F, codes)
    got = gpu.vertices(mesh, x, F, codes)
    np.testing.assert_allclose(got, want, rtol=0, atol=1.0e-12)
    assert gpu.material_grid.extension_nodes == cpu.grid.extension_nodes


@pytest.mark.gpu
def test_gpu_embedding_is_affine_exact_and_separates_faces():
    ref, nodes, cpu, gpu = _pair()
    A = np.array([[1, 0.1, 0], [0, 1.2, 0], [0, 0, 0.9]])
    t = np.array([0.1, 0.2, 0.3])
    mesh = mesh_points(500, 3)
    got = gpu.vertices(mesh, ref @ A.T + t, np.tile(A, (len(ref), 1, 1)), np.zeros(len(ref), int))
    np.testing.assert_allclose(got, mesh.reference @ A.T + t, atol=1.0e-10)
    codes = np.where(ref[:, 0] < 0, 1, 2)
    x = ref.copy()
    x[:, 0] += np.where(codes == 1, -0.004, 0.006)
    mesh = mesh_points(500, 4, lambda r: np.where(r[:, 0] < 0, 1, 2))
    moved = gpu.vertices(mesh, x, np.tile(np.eye(3), (len(ref), 1, 1)), codes)
    for code, shift in [(1, -0.004), (2, 0.006)]:
        sel = mesh.codes == code
        np.testing.assert_allclose(moved[sel, 0], mesh.reference[sel, 0] + shift, atol=1.0e-12)
    with pytest.raises(ValueError, match="finite"):
        gpu.vertices(mesh, np.full_like(x, np.nan), np.tile(np.eye(3), (len(ref), 1, 1)), codes)


@pytest.mark.gpu
def test_gpu_float32_embedding_is_close_to_float64():
    ref, nodes, cpu, gpu = _pair("float32")
    rng = np.random.default_rng(11)
    codes = np.where(ref[:, 0] < 0, 1, 2)
    x = ref + rng.normal(0, 0.001, ref.shape)
    F = np.tile(np.eye(3), (len(ref), 1, 1)) + rng.normal(0, 0.02, (len(ref), 3, 3))
    mesh = mesh_points(1000, 5, lambda r: np.where(r[:, 0] < 0, 1, 2))
    np.testing.assert_allclose(gpu.vertices(mesh, x, F, codes), cpu.vertices(mesh.reference, mesh.codes, x, F, codes),
                               atol=2.0e-7)
