"""The seeded sweep of horizontal-cylinder cuts: reproducible from its seed and
drawn from the stated distributions (spacing from {3, 4, 4.5, 6} mm, knife
offset uniform in [0, h/2], speed log-uniform in [0.02, 0.2] m/s, E
log-uniform in [5e4, 5e5] Pa), each with a whole number of substeps per 1 ms
interval from the banana_dt rule.  Host only."""

import numpy as np
import pytest

from blademaster_gb300.geometry import points
from blademaster_gb300.sweep import INTERVAL, RADIUS, SPACINGS, impulse_bins, instances


def test_instances_are_reproducible_and_follow_their_distributions():
    a, b = instances(256, seed=0), instances(256, seed=0)
    assert [(i.config, i.offset, i.speed) for i in a] == [(i.config, i.offset, i.speed) for i in b]
    assert [i.speed for i in instances(8, seed=1)] != [i.speed for i in a[:8]]
    spacing = np.array([i.config.grid_spacing for i in a])
    assert set(spacing) == set(SPACINGS)
    offset = np.array([i.offset for i in a])
    assert np.all((offset >= 0) & (offset <= spacing / 2))
    speed = np.array([i.speed for i in a])
    assert np.all((speed >= 0.02) & (speed <= 0.2))
    assert np.log(speed).std() > 0.4  # spread over the decade, not clustered
    young = np.array([i.config.young_modulus for i in a])
    assert np.all((young >= 5.0e4) & (young <= 5.0e5))
    for i in a:
        substeps = INTERVAL / i.config.dt
        assert abs(substeps - round(substeps)) < 1e-9 and round(substeps) >= 1
        assert i.config.external_tool and i.config.cache_topology


def test_knife_states_start_above_the_cylinder_and_descend():
    inst = instances(1, seed=3, spacings=(0.006,))[0]
    first, later = inst.state(0), inst.state(10)
    edge0 = first.position[2] - 0.02
    assert abs(edge0 - (2 * RADIUS + 0.002)) < 1e-12
    assert abs((first.position[2] - later.position[2]) - 10 * INTERVAL * inst.speed) < 1e-12
    assert first.linear_velocity[2] == -inst.speed
    cfg = inst.config
    x, _, _ = points(cfg.size, cfg.grid_spacing, cfg.shape, cfg.sampling_seed)
    assert x[:, 2].max() < 2 * RADIUS + 1e-9 and len(x) > 0


# the reference's tests/test_convergence.py:6-29 on the sweep traces' impulse bins

def test_impulses_are_conserved_across_incommensurate_bins():
    times = [0.003, 0.007, 0.011, 0.02]
    forces = np.array([[2, -3, 5], [7, 2, -1], [-8, 3, 2], [4, -6, 9.0]])
    bins = impulse_bins(times, forces, [0, 0.005, 0.01, 0.015, 0.02])
    np.testing.assert_allclose(bins.sum(axis=0), (forces * np.diff([0, *times])[:, None]).sum(axis=0))
    np.testing.assert_allclose(bins[0], forces[0] * 0.003 + forces[1] * 0.002)
    np.testing.assert_allclose(bins[1], forces[1] * 0.002 + forces[2] * 0.003)


def test_resampling_constant_force_does_not_create_rate_difference():
    force = np.array([1.0, -2.0, 4.0])
    edges = np.linspace(0, 1.0, 101)
    for n in [100, 250, 1000]:
        bins = impulse_bins(np.linspace(1 / n, 1, n), np.tile(force, (n, 1)), edges)
        np.testing.assert_allclose(bins, np.tile(force * 0.01, (100, 1)), atol=1.0e-12)


def test_no_extrapolated_force_or_nonfinite_trace():
    with pytest.raises(ValueError):
        impulse_bins([0.1], [[1.0, 2.0, 3.0]], [0, 0.2])
    with pytest.raises(ValueError):
        impulse_bins([0.1], [[1.0, np.nan, 3.0]], [0, 0.1])


def test_impulse_bins_match_the_interval_overlap_integral():
    # an independent statement of the same integral: each bin sums force x overlap with every interval
    rng = np.random.default_rng(7)
    t = np.cumsum(rng.uniform(0.0005, 0.0015, 200))
    f = rng.normal(0, 1, (200, 3))
    edges = np.sort(np.concatenate([[0.0, t[-1]], rng.uniform(0, t[-1], 37)]))
    start = np.concatenate([[0.0], t[:-1]])
    overlap = np.clip(np.minimum(t[None], edges[1:, None]) - np.maximum(start[None], edges[:-1, None]), 0, None)
    np.testing.assert_allclose(impulse_bins(t, f, edges), overlap @ f, atol=1e-13)
