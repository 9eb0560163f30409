"""Reference sampling and stencils against fixtures made by the reference's own
blademaster_warp/geometry.py (tests/golden/make_golden.py), bit for bit."""

import glob

import numpy as np
import pytest

from blademaster_gb300.geometry import points, stencil, cell_sort, stencil_table, levelset

FIXTURES = sorted(glob.glob(str(__import__("pathlib").Path(__file__).parent / "golden" / "geometry_*.npz")))


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: p.split("geometry_")[-1][:-4])
def test_points_and_stencil_match_reference_bitwise(path):
    f = np.load(path)
    x, origin, cells = points(tuple(f["size"]), float(f["spacing"]), str(f["shape"]), int(f["seed"]))
    np.testing.assert_array_equal(x, f["x"])
    np.testing.assert_array_equal(origin, f["origin"])
    np.testing.assert_array_equal(cells, f["cells"])
    nodes, w, g = stencil(x, origin, float(f["spacing"]), cells)
    np.testing.assert_array_equal(nodes, f["nodes"])
    np.testing.assert_array_equal(w, f["weights"])
    np.testing.assert_array_equal(g, f["gradients"])


def test_partition_of_unity_and_zero_gradient_sum():
    # tests/test_mechanics.py:74-77
    x, origin, cells = points((0.06, 0.03, 0.03), 0.0075, "block", 0)
    _, w, g = stencil(x, origin, 0.0075, cells)
    np.testing.assert_allclose(w.astype(np.float32).sum(1), 1, atol=2e-7)
    np.testing.assert_allclose(g.astype(np.float32).sum(1), 0, atol=2e-5)


@pytest.mark.parametrize("seed", [0, 1])
def test_cell_sort_and_stencil_table(seed):
    x, origin, cells = points((0.06, 0.03, 0.03), 0.006, "block", seed)
    nodes, w, g = stencil(x, origin, 0.006, cells)
    order, start = cell_sort(x, origin, 0.006, cells)
    assert sorted(order.tolist()) == list(range(len(x)))
    cell = np.ravel_multi_index(np.floor((x - origin) / 0.006).astype(int).T, tuple(cells))
    assert np.all(np.diff(cell[order]) >= 0)
    assert start[-1] == len(x) and np.all(np.diff(start) <= 8)
    tw, tg, ids = stencil_table(w, g)
    np.testing.assert_array_equal(tw[ids], w.astype(np.float32))
    np.testing.assert_array_equal(tg[ids], g.astype(np.float32))
    assert len(tw) == (8 if seed == 0 else len(x))


def test_empty_and_clipped_domains():
    with pytest.raises(ValueError, match="clipped"):
        points((0.072, 0.024, 0.03), 0.006, "banana")
    # horizontal cylinder of the prescribed triple cut: r = 18 mm, L = 120 mm, on the board
    x, _, _ = points((0.12, 0.036, 0.036), 0.006, "hcylinder")
    assert len(x) > 0 and (levelset(x, (0.12, 0.036, 0.036), "hcylinder") <= 0).all()
    assert x[:, 2].min() > 0 and abs(np.ptp(x[:, 0]) - 0.117) < 1e-9


# tests/test_geometry.py of the reference: the sampling rules themselves


def test_banana_is_not_silently_clipped():
    # test_geometry.py:6-13
    with pytest.raises(ValueError, match="clipped"):
        points((0.072, 0.024, 0.03), 0.006, "banana")
    a, _, _ = points((0.072, 0.06, 0.03), 0.006, "banana")
    b, _, _ = points((0.072, 0.072, 0.03), 0.006, "banana")
    np.testing.assert_allclose(a, b)
    assert len(a) == 892
    assert (levelset(a, (0.072, 0.06, 0.03), "banana") <= 0).all()


@pytest.mark.parametrize("spacing", [0.004, 0.007])
def test_spacing_that_does_not_divide_the_size_still_covers_the_banana(spacing):
    # test_geometry.py:16-29
    from blademaster_gb300.geometry import BANANA_DEMO_SIZE_M

    size = np.array(BANANA_DEMO_SIZE_M)
    fine, _, _ = points(size, 0.003, "banana")
    x, origin, cells = points(size, spacing, "banana")
    assert np.all(cells * spacing >= size - 1.0e-12)
    assert np.all((x >= origin) & (x <= origin + cells * spacing))
    assert abs(np.ptp(x[:, 0]) - np.ptp(fine[:, 0])) < spacing / 2
    block, origin, _ = points((0.03, 0.03, 0.03), spacing, "block")
    assert np.all(block - origin <= 0.03)


@pytest.mark.parametrize("shape", ["banana", "block"])
def test_jittered_particles_start_clear_of_the_board(shape):
    # test_geometry.py:32-39
    from blademaster_gb300.geometry import BANANA_DEMO_SIZE_M

    size = BANANA_DEMO_SIZE_M if shape == "banana" else (0.06, 0.03, 0.03)
    for seed in (1, 2):
        x, _, _ = points(size, 0.006, shape, seed)
        assert x[:, 2].min() >= 0.006 / 4
