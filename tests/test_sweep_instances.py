"""The seeded sweep of horizontal-cylinder cuts: reproducible from its seed and
drawn from the stated distributions (spacing from {3, 4, 4.5, 6} mm, knife
offset uniform in [0, h/2], speed log-uniform in [0.02, 0.2] m/s, E
log-uniform in [5e4, 5e5] Pa), each with a whole number of substeps per 1 ms
interval from the banana_dt rule.  Host only."""

import numpy as np

from blademaster_gb300.geometry import points
from blademaster_gb300.sweep import INTERVAL, RADIUS, SPACINGS, instances


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
