"""MLS-MPM cutting baseline (blademaster_warp/mlsmpm.py).

CPU: the reference's own tests (tests/test_mlsmpm.py:27-101) restated on the
oracle.  GPU: MlsSolver against the oracle, bit for bit (the P2G grid sums
are exact fixed point on both sides, so the atomics' order does not matter),
and the reference's API behaviour (divergence raises, inversions are clamped).
"""

import numpy as np
import pytest

from blademaster_gb300.coupling import ToolState
from blademaster_gb300.solver import Config
from oracle.oracle import MlsOracle

SIZE = (0.04, 0.02, 0.024)
PARKED = ([0, 0, 0.2], [0, 0, 0, 1], [0, 0, 0], [0, 0, 0])


def config(**kw):
    # tests/test_mlsmpm.py:9-20
    return Config(size=SIZE, grid_spacing=0.006, dt=0.0001, young_modulus=400000.0, poisson_ratio=0.4,
                  yield_stress=40000.0, blade_half_size=(0.0005, 0.015, 0.02), sampling_seed=1, **kw)


def soft_config():
    # tests/test_mlsmpm.py:37-48 (Fig. 4 material)
    return Config(size=(0.06, 0.06, 0.056), grid_spacing=0.01, dt=0.002, young_modulus=10000.0, poisson_ratio=0.4,
                  density=1100.0, normal_scale=1.0, board_normal_scale=1.0, blade_half_size=(0.0005, 0.05, 0.04))


def left_domain(o):
    local = (o.arrays["x"] - o.origin) / o.config.grid_spacing
    with np.errstate(invalid="ignore"):
        base = np.floor(local - 0.5)
        outside = ~np.all(np.isfinite(base) & (base >= 0) & (base + 2 < o.dims), axis=1)
    return int(outside.sum())


def cut_states():
    """The knife descending through the block (tests/test_mlsmpm.py:89-97)."""
    half, speed, interval = 0.02, 0.05, 0.002
    for i in range(int(0.024 / speed / interval)):
        edge = SIZE[2] + 0.002 - speed * i * interval
        yield ([0, 0, edge + half], [0, 0, 0, 1], [0, 0, -speed], [0, 0, 0]), interval


def test_block_rests_on_the_board_without_damage():
    o = MlsOracle(config())
    for _ in range(50):
        o.advance(*PARKED, 20)
    A = o.arrays
    assert np.abs(A["v"]).max() < 0.05
    assert A["x"][:, 2].min() > 0.9 * o.config.grid_spacing / 4
    assert not A["damage"].any()


def test_soft_block_settling_under_gravity_is_not_damage():
    literal, settled = MlsOracle(soft_config()), MlsOracle(soft_config(), damage_from_start=False)
    for _ in range(250):
        literal.advance(*PARKED, 1)
        settled.advance(*PARKED, 1)
    settled.arrays["damage_reference"][:] = np.linalg.det(settled.arrays["F"].reshape(-1, 3, 3).astype(np.float64))
    for _ in range(250):
        literal.advance(*PARKED, 1)
        settled.advance(*PARKED, 1)
    assert literal.arrays["damage"].sum() > 0.05 * literal.n
    assert not settled.arrays["damage"].any()
    assert settled.arrays["x"][:, 2].max() < 0.056


def test_inverted_particle_is_clamped_like_plasticinelab_not_fatal():
    o = MlsOracle(config())
    o.arrays["F"][0] = np.diag([1.0, 1.0, -0.5]).reshape(9)
    o.advance(*PARKED, 2)
    assert left_domain(o) == 0 and o.arrays["inversions"][0] == 1
    assert np.linalg.det(o.arrays["F"][0].reshape(3, 3)) > 0


def test_diverged_particle_is_skipped_without_out_of_bounds_access():
    o = MlsOracle(config())
    o.arrays["x"][0] = 1.0e30
    o.arrays["x"][1] = np.nan
    o.advance(*PARKED, 20)
    assert left_domain(o) == 2
    assert np.isfinite(o.arrays["x"][2:]).all()


def test_knife_damages_material_at_its_plane_and_feels_the_reaction():
    o = MlsOracle(config(), damage_from_start=False)
    for _ in range(25):
        o.advance(*PARKED, 20)
    o.arrays["damage_reference"][:] = np.linalg.det(o.arrays["F"].reshape(-1, 3, 3).astype(np.float64))
    lift = []
    for state, interval in cut_states():
        impulse, _ = o.advance(*state, 20)
        lift.append(impulse[2] / interval)
    damaged = o.arrays["damage"] > 0
    assert damaged.sum() >= 3
    assert np.abs(o.reference[damaged, 0]).mean() < 2 * o.config.grid_spacing
    assert np.mean(lift[-10:]) > 0.5


# ------------------------------------------------------------------- GPU


def same(g, o):
    A = o.arrays
    np.testing.assert_array_equal(g.x.numpy(), A["x"], err_msg="x")
    np.testing.assert_array_equal(g.v.numpy(), A["v"], err_msg="v")
    np.testing.assert_array_equal(g.C.numpy().reshape(-1, 9), A["C"], err_msg="C")
    np.testing.assert_array_equal(g.F.numpy().reshape(-1, 9), A["F"], err_msg="F")
    np.testing.assert_array_equal(g.damage.numpy(), A["damage"], err_msg="damage")
    np.testing.assert_array_equal(g.yield_stress.numpy(), A["yield_stress"], err_msg="yield_stress")
    assert g.inversions.numpy()[0] == A["inversions"][0]


@pytest.mark.gpu
def test_gpu_resting_and_cutting_match_oracle():
    from blademaster_gb300.mlsmpm import MlsSolver

    g, o = MlsSolver(config(), damage_from_start=False), MlsOracle(config(), damage_from_start=False)
    for _ in range(10):
        r = g.advance(ToolState(*PARKED), 0.002)
        imp, ang = o.advance(*PARKED, 20)
        np.testing.assert_array_equal(r.impulse_ns, imp)
    same(g, o)
    g.start_damage()
    o.arrays["damage_reference"][:] = g.damage_reference.numpy()
    for k, (state, interval) in enumerate(cut_states()):
        if k == 40:
            break
        r = g.advance(ToolState(*state), interval, graph=k % 2 == 0)
        imp, ang = o.advance(*state, 20)
        np.testing.assert_array_equal(r.impulse_ns, imp)
        np.testing.assert_array_equal(r.angular_impulse_nms, ang)
    same(g, o)


@pytest.mark.gpu
def test_gpu_plastic_softening_and_inversion_match_oracle():
    from blademaster_gb300.mlsmpm import MlsSolver, TopoCutParams

    params = TopoCutParams(softening=2.0e6, damaged_shear=0.5)
    g, o = MlsSolver(config(), params), MlsOracle(config(), params)
    F = g.F.numpy()
    F[0] = np.diag([1.0, 1.0, -0.5])
    F[1] = np.diag([1.2, 0.9, 0.95])
    g.F.assign(F)
    o.arrays["F"][:] = F.reshape(-1, 9)
    for state, interval in list(cut_states())[:30]:
        g.advance(ToolState(*state), interval)
        o.advance(*state, 20)
    same(g, o)
    assert g.diagnostics()["clamped_inversions"] >= 1


@pytest.mark.gpu
def test_gpu_diverged_particle_raises():
    from blademaster_gb300.mlsmpm import MlsSolver

    g = MlsSolver(config())
    x = g.x.numpy()
    x[0] = 1.0e30
    x[1] = np.nan
    g.x.assign(x)
    with pytest.raises(RuntimeError, match="2 particles non-finite or outside the grid"):
        g.advance(ToolState(*PARKED), 0.002)
    assert np.isfinite(g.x.numpy()[2:]).all()


@pytest.mark.gpu
def test_gpu_block_at_scale_matches_oracle():
    # The workload the MLS-MPM benchmark times: the 1.6 M-particle block (2 mm grid, dt 10 us)
    # under one knife held 1 mm into its top face.  Three substeps bit for bit, with the
    # knife's interval impulse and angular impulse.
    from blademaster_gb300 import scenes
    from blademaster_gb300.mlsmpm import MlsSolver

    cfg, knives, _ = scenes.block_8knives()
    g, o = MlsSolver(cfg), MlsOracle(cfg)
    assert g.n == o.n == 1_600_000
    state = (knives[3], [0.0, 0.0, 0.0, 1.0], [0.0, 0.0, -0.05], [0.0, 0.0, 0.0])
    r = g.advance(ToolState(*state), 3 * cfg.dt)
    imp, ang = o.advance(*state, 3)
    np.testing.assert_array_equal(r.impulse_ns, imp)
    np.testing.assert_array_equal(r.angular_impulse_nms, ang)
    assert np.abs(imp).max() > 0  # the knife is in contact
    same(g, o)
