"""The benchmark's scene configurations, CUDA path against the oracle.

* Gravity knife (8960 particles): at the Table I step of 2 ms the grid CFL
  number is 3.3; the oracle inverts on the fifth substep, and the CUDA path
  must detect the same failure (the same inverted-particle count, the same
  RuntimeError from ``state()``).  The stable stand-in step of 0.25 ms runs
  the whole simulated second (4000 substeps) bit for bit, with the
  reference's outputs: edge height, directional work, damage count and
  piece count (paper_freefall.py:134-157).  At this stiffness the knife
  stalls 1.3 mm into the top face and tips over; nothing is severed.  (The
  tip-over is float32 round-off breaking the scene's mirror symmetry: in the
  oracle's float64 build the knife stays upright; tests/test_fp64_scenes.py.)
* Triple cut of the Maxwell cylinder through ExternalToolPort (4480
  particles, 1390 coupling intervals of 2 ms): every interval's impulse and
  angular impulse, the final state and the four pieces, bit for bit.
* The 1.6 M-particle block with 8 knives, the configuration the throughput
  is quoted on: its first substeps from t = 0 (pair-list build, first
  registration, the side labels of every knife and the re-registration
  they cause), bit for bit, including the (node, code) field map.

The oracle's runs stop where the material has inverted: past that point its
state grows without bound and nothing compares.
"""

import numpy as np
import pytest

from blademaster_gb300 import scenes
from oracle.oracle import OracleSolver
from oracle import pieces


def oracle_det_min(o):
    return float(np.linalg.det(o.get("F").astype(np.float64)).min())


def test_gravity_knife_table_step_inverts_on_the_oracle():
    cfg, pos, vel = scenes.gravity_knife(dt=0.002)
    o = OracleSolver(cfg)
    o.set("tool_pos", pos)
    for _ in range(4):
        o.step((0.0, 0.0, 0.0), cutting=True)
    assert o.get("errors").tolist() == [0, 0, 0]
    o.step((0.0, 0.0, 0.0), cutting=True)
    errors = o.get("errors").tolist()
    assert errors[0] == 0 and errors[2] == 0 and errors[1] > 1000
    assert oracle_det_min(o) < 0


def test_gravity_knife_stable_step_stays_valid_on_the_oracle():
    cfg, pos, vel = scenes.gravity_knife()
    o = OracleSolver(cfg)
    o.set("tool_pos", pos)
    for _ in range(400):  # the first 0.1 s: the knife lands and starts cutting
        o.step((0.0, 0.0, 0.0), cutting=True)
    assert o.get("errors").tolist() == [0, 0, 0]
    assert oracle_det_min(o) > 0.5
    assert o.get("tool_pos")[0, 2] < 0.08 + 0.02  # the edge is in the block


def test_edge_height_and_tilt_follow_the_rotated_edge():
    # tests/test_cut_resistance.py:114-120: the gravity knife's edge height is the lowest point of its
    # edge; upright at 50 mm with a 30 mm half height it is 20 mm, turned flat about y it is the centre
    from scipy.spatial.transform import Rotation

    from oracle.fp64_scenes import tilt

    half = (0.0005, 0.04, 0.03)
    upright, flat = Rotation.identity().as_quat(), Rotation.from_euler("y", 90, degrees=True).as_quat()
    assert scenes.edge_height([0.0, 0.0, 0.05], upright, half) == pytest.approx(0.05 - 0.03, abs=1e-12)
    assert scenes.edge_height([0.0, 0.0, 0.0005], flat, half) == pytest.approx(0.0005, abs=1e-12)
    assert tilt(upright) == pytest.approx(0.0, abs=1e-9) and tilt(flat) == pytest.approx(90.0, abs=1e-9)


def test_triple_cut_keyframes():
    keys = scenes.triple_cut_keyframes()
    cuts = [k for k in keys if k[2] >= 0]
    assert sorted({k[2] for k in cuts}) == [0, 1, 2]
    for index, x in enumerate(scenes.TRIPLE_CUT_POSITIONS):
        own = [k for k in keys if k[2] == index]
        assert all(k[1][0] == x for k in own)
        top, bottom = own[1], own[2]
        assert np.isclose((top[1][2] - bottom[1][2]) / (bottom[0] - top[0]), 0.1)  # descends at 0.1 m/s
        assert np.isclose(bottom[1][2] - scenes.TRIPLE_CUT_KNIFE[2], 0.0003)  # to the board
    pushes = [(b[1][0] - a[1][0]) for a, b in zip(keys, keys[1:]) if a[1][2] == b[1][2] and a[2] < 0 and b[1][0] > a[1][0]]
    assert np.allclose(pushes, 0.02)
    schedule = scenes.triple_cut_schedule()
    assert len(schedule) == 1390
    assert [s[2] for s in schedule if s[1]][:1] == [0] and schedule[-1][2] == 2
    state, cutting, index = scenes.command_at(0.05 + 0.01, keys)
    assert cutting and index == 0 and np.allclose(state.linear_velocity, [0, 0, -0.1])


def test_triple_cut_config_holds_the_maxwell_viscosity():
    cfg = scenes.triple_cut_config()
    mu = cfg.young_modulus / (2 * (1 + cfg.poisson_ratio))
    assert np.isclose(cfg.maxwell_tau * cfg.maxwell_fraction * mu, 5.0)
    assert 0 < cfg.dt / cfg.maxwell_tau < 1  # resolved relaxation (1 - exp(-dt/tau) about 0.2)


# ------------------------------------------------------------------- CUDA


def _gpu_solver(cfg):
    from blademaster_gb300.solver import Solver

    return Solver(cfg)


def _assert_same(g, o, names=("x", "v", "F", "stress", "codes", "damage")):
    for name in names:
        np.testing.assert_array_equal(getattr(g, name).numpy(), o.get(name), err_msg=name)
    assert g.errors.numpy().tolist() == o.get("errors").tolist()


@pytest.mark.gpu
def test_gravity_knife_table_step_fails_like_the_oracle():
    cfg, pos, vel = scenes.gravity_knife(dt=0.002)
    g, o = _gpu_solver(cfg), OracleSolver(cfg)
    g.tool_pos.assign(pos)
    o.set("tool_pos", pos)
    g.advance(np.zeros((4, 3)), cutting=True)
    for _ in range(4):
        o.step((0.0, 0.0, 0.0), cutting=True)
    _assert_same(g, o)
    g.state()  # still valid
    # the fifth substep inverts the material on both: same count, same error
    g.advance(np.zeros((1, 3)), cutting=True)
    o.step((0.0, 0.0, 0.0), cutting=True)
    _assert_same(g, o)
    assert g.errors.numpy()[1] > 1000
    with pytest.raises(RuntimeError, match="GPU errors"):
        g.state()


@pytest.mark.gpu
def test_gravity_knife_stable_second_is_bitexact():
    cfg, pos, vel = scenes.gravity_knife()
    g, o = _gpu_solver(cfg), OracleSolver(cfg)
    g.tool_pos.assign(pos)
    o.set("tool_pos", pos)
    stride = 40  # 10 ms per call, as paper_freefall.run advances (paper_freefall.py:119-123)
    for _ in range(4000 // stride):
        g.advance(np.zeros((stride, 3)), cutting=True)
        for _ in range(stride):
            o.step((0.0, 0.0, 0.0), cutting=True)
    _assert_same(g, o)
    np.testing.assert_array_equal(g._t["tool"].cpu().numpy(), o.get("tool"))
    np.testing.assert_array_equal(g.work.numpy(), o.get("work").astype(np.float32))
    state = g.state()
    edge = scenes.edge_height(state["blade_position"][0], state["blade_orientation"][0], cfg.blade_half_size)
    released = int(np.count_nonzero(state["damage"] >= 1.0))
    _, sizes = g.components()
    _, oracle_sizes = pieces.components(o.node_numpy, o.weight_numpy, o.get("codes"))
    assert sizes.tolist() == oracle_sizes.tolist() == [8960]
    assert released == int(np.count_nonzero(o.get("damage") >= 1.0))
    # at E = 2e5 Pa the 0.2 kg knife stalls about 1.3 mm into the top face, releases 40
    # particles and tips over onto the block (turned about 90 degrees by t = 1 s)
    assert 0.075 < edge < 0.085
    assert released == 40 and float(g.work.numpy()[0]) > 0.01


@pytest.mark.gpu
def test_triple_cut_through_the_port_is_bitexact():
    from blademaster_gb300.coupling import ExternalToolPort

    cfg = scenes.triple_cut_config()
    g, o = _gpu_solver(cfg), OracleSolver(cfg)
    port = ExternalToolPort(g)
    steps = int(round(scenes.TRIPLE_CUT_INTERVAL / cfg.dt))
    schedule = scenes.triple_cut_schedule()
    for i, (state, cutting, index) in enumerate(schedule):
        reaction = port.advance(state, scenes.TRIPLE_CUT_INTERVAL, cutting=cutting, cut_index=index)
        impulse, angular, errors = o.external_interval(scenes.packed_state(state), steps, cutting, index)
        assert not errors.any()
        p = state.checked().position
        angular = angular - np.cross(p, impulse)
        np.testing.assert_array_equal(reaction.impulse_ns, impulse, err_msg=f"interval {i}")
        np.testing.assert_array_equal(reaction.angular_impulse_nms, angular, err_msg=f"interval {i}")
    _assert_same(g, o)
    np.testing.assert_array_equal(g.viscous.numpy(), o.get("viscous")[o.rank].reshape(-1, 3, 3))
    _, sizes = g.components()
    _, oracle_sizes = pieces.components(o.node_numpy, o.weight_numpy, o.get("codes"))
    assert sizes.tolist() == oracle_sizes.tolist()
    assert len(sizes) == 4  # three cuts through: four pieces


@pytest.mark.gpu
def test_block_1p6M_first_substeps_are_bitexact():
    from blademaster_gb300 import _native

    cfg, knives, velocity = scenes.block_8knives()
    g, o = _gpu_solver(cfg), OracleSolver(cfg)
    assert g.n == 1_600_000
    g.tool_pos.assign(knives)
    g.tool_vel.assign(velocity)
    o.set("tool_pos", knives)
    o.set("tool_vel", velocity)
    g.advance(np.zeros((10, 3)), cutting=True)
    for _ in range(10):
        o.step((0.0, 0.0, 0.0), cutting=True)
    _assert_same(g, o, ("x", "v", "F", "stress", "codes"))
    np.testing.assert_array_equal(g._t["tool"].cpu().numpy(), o.get("tool"))
    np.testing.assert_array_equal(np.stack([d.numpy() for d in g.tool_damage]), o.get("tool_damage"))
    # every knife labelled its own digit, and the new codes were registered
    codes = g.codes.numpy()
    digits = {int(c) for c in np.unique(codes) if c}
    assert len(digits) >= 8
    assert g._flag("REGISTRATIONS") >= 2 and g._flag("MULTI") > 0
    gk = g.keys.numpy()
    ok = o.get("keys")
    np.testing.assert_array_equal(np.sort(gk[gk >= 0]), np.sort(ok[ok >= 0]))
    np.testing.assert_array_equal(gk[g.slots.numpy()], ok[o.get("slots")][o.rank])
    assert _native.FLAG["REGISTRATIONS"] >= 0
