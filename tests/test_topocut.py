"""TopoCut topology discovery for the MLS baseline (topocut_topology.py:1-229).

CPU: the oracle's cluster assignment on the reference's cube surface
(tests/test_topocut_topology.py:66-143 of the reference), and the host
smoothing and face components.  GPU: the
reference's own behaviours (tests/test_topocut_topology.py:17-63), the
device SDF against the brute-force oracle, the extracted surface closed and
consistently oriented with the block's volume, and the device cluster
assignment against the oracle.
"""

import numpy as np
import pytest

from blademaster_gb300.geometry import points
from oracle import topocut as oracle

SPACING = 0.006
HALF = (0.0005, 0.03, 0.03)
CUBE_VERTICES = np.array([[-1, -1, -1], [-1, -1, 1], [-1, 1, -1], [-1, 1, 1], [1, -1, -1], [1, -1, 1], [1, 1, -1],
                          [1, 1, 1]], dtype=np.float32) * 0.03 + [0, 0, 0.03]
CUBE_FACES = np.array([[0, 3, 2], [0, 1, 3], [4, 6, 7], [4, 7, 5], [0, 4, 5], [0, 5, 1], [2, 3, 7], [2, 7, 6],
                       [0, 2, 6], [0, 6, 4], [1, 5, 7], [1, 7, 3]], dtype=np.int32)
PROBES = np.array([[0, 0, 0.03], [0.025, 0, 0.03], [0.04, 0, 0.03]], dtype=np.float32)


def block(seed=1):
    return points((0.06, 0.03, 0.03), SPACING, "block", seed)[0]


def stroke(x, top=0.07, bottom=0.03, count=20):
    return [([x, 0.0, z], [0, 0, 0, 1]) for z in np.linspace(top, bottom, count)]


def test_oracle_deep_interior_assignment():
    for spacing in (0.002, 0.001, 0.0005):
        tau = 0.5 * spacing / 2
        reach = float(np.linalg.norm(CUBE_VERTICES.max(0) - CUBE_VERTICES.min(0))) + tau
        labels = oracle.nearest_cluster(PROBES, [(CUBE_VERTICES, CUBE_FACES)], tau, reach)
        np.testing.assert_array_equal(labels, [0, 0, -1])
    assert oracle.signed_volume(CUBE_VERTICES, CUBE_FACES) == pytest.approx(0.06**3)


# ------------------------------------------------------------------- GPU



def test_host_smoothing_and_face_components():
    # topocut_topology.py:81-114: Laplacian smoothing (Eq. 10) over the mesh edges, and the
    # connected components of the faces through shared vertices
    from blademaster_gb300.topocut import face_components, smooth

    v = CUBE_VERTICES.astype(float)
    smoothed = smooth(v, CUBE_FACES, 0.5, 3)
    # a point-symmetric closed mesh keeps its centroid, and every vertex moves toward it
    np.testing.assert_allclose(smoothed.mean(0), v.mean(0), atol=1e-12)
    r0 = np.linalg.norm(v - v.mean(0), axis=1)
    r = np.linalg.norm(smoothed - v.mean(0), axis=1)
    assert np.all(r < r0)
    np.testing.assert_array_equal(smooth(v, CUBE_FACES, 0.5, 0), v)
    # one step equals v + alpha (mean of the edge neighbours - v)
    one = smooth(v, CUBE_FACES, 0.5, 1)
    k = 0
    nbrs = {b for f in CUBE_FACES for a, b in zip(f, np.roll(f, 1)) if a == k} | \
           {a for f in CUBE_FACES for a, b in zip(f, np.roll(f, 1)) if b == k}
    np.testing.assert_allclose(one[k], v[k] + 0.5 * (v[sorted(nbrs)].mean(0) - v[k]), atol=1e-12)
    # two disjoint cubes: two components, each cube's faces together
    faces = np.concatenate([CUBE_FACES, CUBE_FACES + 8])
    labels = face_components(faces, 16)
    assert len(set(labels[:12])) == 1 and len(set(labels[12:])) == 1 and labels[0] != labels[12]


@pytest.mark.gpu
def test_uncut_block_is_one_piece():
    from blademaster_gb300.topocut import TopologyTracker

    x = block()
    t = TopologyTracker(len(x), SPACING, HALF)
    labels = t.reconstruct(x)
    assert len(t.meshes) == 1
    assert (labels == 0).all()


@pytest.mark.gpu
def test_carved_trajectory_splits_the_block_at_the_knife():
    from blademaster_gb300.topocut import TopologyTracker

    x = block()
    t = TopologyTracker(len(x), SPACING, HALF)
    labels = t.reconstruct(x, stroke(0.0))
    assert len(t.meshes) == 2
    assert np.array_equal(t.pieces(), np.bincount(labels[labels >= 0]))
    left, right = labels[x[:, 0] < -0.002], labels[x[:, 0] > 0.002]
    assert len(set(left)) == 1 and len(set(right)) == 1 and left[0] != right[0]


@pytest.mark.gpu
def test_earlier_pieces_keep_their_ids_after_the_gap_closes():
    from blademaster_gb300.topocut import TopologyTracker

    x = block()
    t = TopologyTracker(len(x), SPACING, HALF)
    t.reconstruct(x, stroke(-0.012))
    labels = t.reconstruct(x, stroke(0.012))
    assert len(t.pieces()) == 3
    for lo, hi in ((-1, -0.014), (-0.01, 0.01), (0.014, 1)):
        inside = labels[(x[:, 0] > lo) & (x[:, 0] < hi)]
        assert len(set(inside)) == 1


@pytest.mark.gpu
def test_a_partial_stroke_does_not_separate():
    from blademaster_gb300.topocut import TopologyTracker

    x = block()
    t = TopologyTracker(len(x), SPACING, HALF)
    t.reconstruct(x, stroke(0.0, bottom=0.045))
    assert len(t.pieces()) == 1


@pytest.mark.gpu
def test_a_piece_that_needs_two_cuts_is_carved_by_both():
    from blademaster_gb300.topocut import TopologyTracker

    x = block()
    t = TopologyTracker(len(x), SPACING, (0.0005, 0.0125, 0.03))
    first = [([0.0, -0.0125, z], [0, 0, 0, 1]) for z in np.linspace(0.07, 0.03, 20)]
    second = [([0.0, 0.0125, z], [0, 0, 0, 1]) for z in np.linspace(0.07, 0.03, 20)]
    t.reconstruct(x, first)
    assert len(t.pieces()) == 1
    t.reconstruct(x, second)
    assert len(t.pieces()) == 2
    assert not t.pending


@pytest.mark.gpu
def test_deep_interior_assignment_on_the_device():
    from blademaster_gb300.topocut import nearest_cluster

    for spacing in (0.002, 0.001, 0.0005):
        tau = 0.5 * spacing / 2
        reach = float(np.linalg.norm(CUBE_VERTICES.max(0) - CUBE_VERTICES.min(0))) + tau
        np.testing.assert_array_equal(nearest_cluster(PROBES, [(CUBE_VERTICES, CUBE_FACES)], tau, reach), [0, 0, -1])


@pytest.mark.gpu
def test_device_sdf_matches_oracle_and_surface_is_closed():
    from blademaster_gb300.topocut import TopologyTracker

    x = block()
    t = TopologyTracker(len(x), SPACING, HALF)
    poses = [np.r_[p, q] for p, q in stroke(0.0)]
    vertices, faces = t._surface(x.astype(np.float32), poses)
    prm, s = t.params, t.particle_spacing
    voxel, radius = prm.voxel * s, prm.influence * s
    half = np.array(HALF, float)
    half[0] = max(half[0], prm.gap_voxels * voxel / 2)
    want = oracle.sdf(x.astype(np.float32), t.lower, t.field.shape, voxel, radius, radius + 2 * voxel, poses, half)
    np.testing.assert_allclose(t.field.cpu().numpy(), want, atol=2.0e-6)
    # every undirected edge is shared by exactly two faces, in opposite directions
    directed = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
    keys = directed[:, 0] * len(vertices) + directed[:, 1]
    assert len(np.unique(keys)) == len(keys)
    reverse = directed[:, 1] * len(vertices) + directed[:, 0]
    assert np.isin(reverse, keys).all()
    # two closed, outward-oriented pieces whose volume is about the block's less the carved slab
    volume = oracle.signed_volume(vertices, faces)
    assert 0.8 * 0.06 * 0.03 * 0.03 < volume < 1.25 * 0.06 * 0.03 * 0.03


@pytest.mark.gpu
def test_device_cluster_matches_oracle_on_random_points():
    from blademaster_gb300.topocut import TopologyTracker, nearest_cluster

    x = block()
    t = TopologyTracker(len(x), SPACING, HALF)
    t.reconstruct(x, stroke(0.0))
    rng = np.random.default_rng(2)
    probes = rng.uniform([-0.035, -0.02, -0.005], [0.035, 0.02, 0.035], (300, 3)).astype(np.float32)
    s = t.particle_spacing
    tau, reach = t.params.tau * s, 1.0
    got = nearest_cluster(probes, t.meshes, tau, reach)
    want = oracle.nearest_cluster(probes, t.meshes, tau, reach)
    assert (got == want).mean() > 0.99
