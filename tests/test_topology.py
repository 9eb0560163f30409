"""Piece counting against the reference's blademaster_warp/topology.py outputs."""

from pathlib import Path

import numpy as np

from blademaster_gb300.topology import components, compatible, digit_masks

GOLDEN = Path(__file__).parent / "golden" / "topology_default_block.npz"


def test_uncut_bridges_and_persistent_conflicts():
    # tests/test_topology.py:5-12 of the reference
    nodes = np.zeros((3, 1), dtype=int)
    weights = np.ones((3, 1))
    assert components(nodes, weights, [1, 0, 2])[1].tolist() == [3]
    assert components(nodes, weights, [1, 1, 2])[1].tolist() == [2, 1]
    assert not compatible(1, 2)
    assert not compatible(4, 7)
    assert compatible(1, 4)


def test_zero_weight_and_spatially_disjoint_pieces():
    nodes = np.array([[0, 1], [1, 2], [3, 4]])
    weights = np.array([[1.0, 0.0], [1.0, 0.0], [1.0, 0.0]])
    assert components(nodes, weights, [0, 0, 0])[1].tolist() == [1, 1, 1]


def test_labels_match_reference_fixtures():
    f = np.load(GOLDEN)
    for key in ("uncut", "one_cut", "partial_cut", "two_cuts", "random27"):
        labels, sizes = components(f["nodes"], f["weights"], f[f"{key}_codes"])
        np.testing.assert_array_equal(labels, f[f"{key}_labels"], err_msg=key)
        np.testing.assert_array_equal(sizes, f[f"{key}_sizes"], err_msg=key)


def test_digit_masks_compatibility_matches_reference():
    f = np.load(GOLDEN)
    pairs = f["compat_pairs"]
    ones, twos = digit_masks(pairs.reshape(-1))
    ones, twos = ones.reshape(-1, 2), twos.reshape(-1, 2)
    fast = ((ones[:, 0] & twos[:, 1]) == 0) & ((twos[:, 0] & ones[:, 1]) == 0)
    np.testing.assert_array_equal(fast, f["compat_values"])
    assert [compatible(a, b) for a, b in pairs] == f["compat_values"].tolist()
