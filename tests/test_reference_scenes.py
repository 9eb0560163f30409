"""Scene tests of the reference, restated with the reference's own assertions.

Each scene runs on the CPU oracle (the restated solver, float64 knife state)
and, marked gpu, on the CUDA solver through the reference-facing API
(Solver, ExternalToolPort, Solver._drive_tool).  The CUDA runs are compared
bit-exactly with the oracle on the same inputs:

* board penetration against the board's normal scale
  (tests/test_board_contact.py:6-29);
* a pitched blade resting on the board still cuts the bottom layer beside
  its edge, leaving two pieces (tests/test_pinched_labels.py:7-35);
* the knife servo, the free knife and the guided knife against the board,
  and the board's edge (tests/test_tool.py:6-80);
* the cut-code capacity follows the grid size
  (tests/test_stress_replays.py:61-87);
* a cut at index 25 (digit 3^25, beyond 32 bits) severs the banana into two
  pieces (tests/test_coupling.py:131-145);
* strokes found from the embedded-particle count label each cut plane with
  its own digit (tests/test_coupling.py:147-186);
* several free knives: only free knives may be several, slot order does not
  matter, mirrored knives move alike and label their own digits, a knife
  beside the block falls freely, each knife pays its own cutting work
  (tests/test_multi_tool.py:21-106);
* two or three knives, fixed or crossing and turning, over the same
  particles give each knife exactly its lone contact, in every slot order
  (tests/test_multi_tool.py:108-116, tests/test_stress_replays.py:95-107);
* three free knives falling through the block over two strokes give the same
  trajectories, damage, side codes and pieces in every slot order once the
  knives and their digits are mapped back (tests/test_multi_tool.py:119-133);
* the paper's cutting resistance stops growing with the cutting energy,
  while held particles make the force grow with it
  (tests/test_cut_resistance.py:74-111);
* the single-field baseline: cut halves move independently, one field drags
  the other half, switching back restores the separation
  (tests/test_single_field.py:7-46).
"""

from dataclasses import replace

import numpy as np
import pytest

from blademaster_gb300.coupling import ToolState
from blademaster_gb300.geometry import points, stencil
from blademaster_gb300.solver import Config, cut_capacity
from blademaster_gb300.topology import components
from oracle.oracle import OracleSolver


def packed(state):
    """The 49 floats ExternalToolPort loads for one interval (coupling.py:88-120)."""
    s = state.checked()
    return np.concatenate([s.position, s.orientation_xyzw, s.linear_velocity, s.angular_velocity,
                           s.mobility.ravel()]).astype(np.float32)


# ------------------------------------------------------------------ board

def board_config(board_normal_scale):
    return Config(size=(0.06, 0.06, 0.06), grid_spacing=0.01, dt=0.002, young_modulus=10000.0, poisson_ratio=0.4,
                  external_tool=True, board_normal_scale=board_normal_scale)


AWAY = ToolState([0.5, 0.0, 0.5], [0, 0, 0, 1], [0, 0, 0], [0, 0, 0])


def settled_oracle(board_normal_scale, intervals=500):
    c = OracleSolver(board_config(board_normal_scale))
    for _ in range(intervals):
        c.external_interval(packed(AWAY), 1, cutting=False)
    return c


@pytest.mark.parametrize("scale, bound", [(0.0, -0.003), (1.0, -0.001)])
def test_board_penetration_follows_the_normal_scale(scale, bound):
    # 12 particle layers settle about N g dt^2 / s_n into the board: 4.7 mm with
    # the default s_n = 0.1, 0.5 mm with s_n = 1 (test_board_contact.py:26-29).
    c = settled_oracle(scale)
    x = c.get("x")
    assert np.isfinite(x).all()
    bottom = x[:, 2].min() - c.radius
    assert bottom < bound if scale == 0.0 else bottom > bound


@pytest.mark.gpu
def test_board_penetration_cuda_matches_oracle():
    from blademaster_gb300.coupling import ExternalToolPort
    from blademaster_gb300.solver import Solver

    for scale in (0.0, 1.0):
        cfg = board_config(scale)
        g = Solver(cfg)
        port = ExternalToolPort(g)
        for _ in range(500):
            port.advance(AWAY, cfg.dt, cutting=False)
        c = settled_oracle(scale)
        np.testing.assert_array_equal(g.x.numpy(), c.get("x"))
        np.testing.assert_array_equal(g.v.numpy(), c.get("v"))


# --------------------------------------------------- pitched edge on board

PINCH = Config(size=(0.06, 0.03, 0.03), grid_spacing=0.006, dt=0.00025, sampling_seed=1, external_tool=True,
               board_normal_scale=1.0, blade_half_size=(0.0005, 0.025, 0.02))


def pinch_states(intervals=1000):
    """The knife pitched 10 degrees about its length axis, descending at 0.05 m/s
    to 0.2 mm above the board, then held (test_pinched_labels.py:21-30)."""
    pitch = np.deg2rad(10.0)
    q = [0.0, np.sin(pitch / 2), 0.0, np.cos(pitch / 2)]
    reach = PINCH.blade_half_size[2] * np.cos(pitch)
    lean = PINCH.blade_half_size[2] * np.sin(pitch)
    interval, speed, start, stop = 0.001, 0.05, 0.04, 0.0002
    for i in range(intervals):
        edge = max(start - speed * i * interval, stop)
        moving = edge > stop
        yield ToolState([lean, 0.0, edge + reach], q, [0.0, 0.0, -speed if moving else 0.0], [0, 0, 0])


def assert_pinched_cut(codes, x, node_numpy, weight_numpy):
    assert not ((codes == 0) & (np.abs(x[:, 0]) < 2 * PINCH.grid_spacing)).any()
    _, sizes = components(node_numpy, weight_numpy, codes)
    assert len(sizes) == 2


def test_pitched_edge_on_the_board_cuts_the_bottom_layer():
    c = OracleSolver(PINCH)
    for state in pinch_states():
        c.external_interval(packed(state), 4, cutting=True, cut_index=0)
    assert_pinched_cut(c.get("codes"), c.get("x"), c.node_numpy, c.weight_numpy)


@pytest.mark.gpu
def test_pitched_edge_cuda_matches_oracle_and_cuts():
    from blademaster_gb300.coupling import ExternalToolPort
    from blademaster_gb300.solver import Solver

    g = Solver(PINCH)
    port = ExternalToolPort(g)
    c = OracleSolver(PINCH)
    for i, state in enumerate(pinch_states()):
        port.advance(state, 0.001, cutting=True)
        if i < 200:
            c.external_interval(packed(state), 4, cutting=True, cut_index=0)
        if i == 199:
            for name in ("x", "v", "codes", "damage"):
                np.testing.assert_array_equal(getattr(g, name).numpy(), c.get(name), err_msg=name)
    assert_pinched_cut(g.codes.numpy(), g.x.numpy(), g.node_numpy, g.weight_numpy)


# ------------------------------------------------------------- knife drive

BLADE_CORNERS = np.array([[0.0, -1.0, -1.0], [0.0, 1.0, -1.0], [1.0, -1.0, -1.0], [-1.0, 1.0, -1.0]])


def lowest_vertex(cfg, pos, rot):
    """Height of the knife's lowest wedge vertex (test_tool.py:6-14)."""
    from scipy.spatial.transform import Rotation

    h, bevel = np.array(cfg.blade_half_size), cfg.blade_bevel_height
    vertices = BLADE_CORNERS * [h[0], h[1], h[2]] + [[0, 0, 0], [0, 0, 0], [0, 0, bevel], [0, 0, bevel]]
    return (Rotation.from_quat(rot).apply(vertices) + pos)[:, 2].min()


class OracleDriver:
    def __init__(self, cfg):
        self.cfg, self.s = cfg, OracleSolver(cfg)

    def place(self, pos, rot=None):
        self.s.set("tool_pos", [pos])
        if rot is not None:
            self.s.set("tool_rot", [rot])

    def drive(self, target, rot):
        self.s.drive_tool(target, rot)

    def state(self):
        return (self.s.get("tool_pos")[0], self.s.get("tool_rot")[0], self.s.get("tool_vel")[0],
                self.s.get("table_impulse")[0])


class CudaDriver:
    def __init__(self, cfg):
        from blademaster_gb300.solver import Solver

        self.cfg, self.s = cfg, Solver(cfg)

    def place(self, pos, rot=None):
        self.s.tool_pos.assign([pos])
        if rot is not None:
            self.s.tool_rot.assign([rot])

    def drive(self, target, rot):
        self.s._drive_tool(target, rot, None, None, 0)

    def state(self):
        s = self.s
        return s.tool_pos.numpy()[0], s.tool_rot.numpy()[0], s.tool_vel.numpy()[0], s.tool_table_impulse.numpy()[0]


def drive(d, target, rot, steps=3000):
    """test_tool.py:17-24: the lowest vertex every 20 tool steps."""
    lowest = []
    for i in range(steps):
        d.drive(target, rot)
        if i % 20 == 0:
            pos, q, _, _ = d.state()
            lowest.append(lowest_vertex(d.cfg, np.asarray(pos, float), np.asarray(q, float)))
    assert np.isfinite(d.state()[2]).all()
    return np.array(lowest)


TILT = 0.2
TILTED = np.array([0.0, np.sin(TILT / 2), 0.0, np.cos(TILT / 2)])


def tool_config(free):
    return replace(Config(), dt=0.00025, pose_servo=not free, free_blade=free, blade_bevel_height=0.005)


def run_tool(driver, free):
    d = driver(tool_config(free))
    d.place([0.12, 0.0, 0.05], TILTED)
    lowest = drive(d, [0.12, 0.0, -0.01], TILTED)
    assert lowest.min() > -2e-5
    assert lowest.max() - lowest.min() > 0.01
    return d


def guided(driver):
    d = driver(replace(Config(), dt=0.00025, blade_bevel_height=0.005))
    d.place([0.0, 0.0, 0.05])
    lowest = drive(d, [0.0, 0.0, -0.01], [0.0, 0.0, 0.0, 1.0])
    assert lowest.min() > -2e-5 and lowest[-1] < 1e-4
    return d


def board_edge(driver):
    cfg = replace(Config(), dt=0.00025, free_blade=True, board_half_extent=(0.05, 0.05))
    on, off = driver(cfg), driver(cfg)
    on.place([0.0, 0.0, 0.05])
    off.place([0.2, 0.0, 0.05])
    assert drive(on, [0, 0, 0], [0, 0, 0, 1], 1500).min() > -2e-5
    assert drive(off, [0, 0, 0], [0, 0, 0, 1], 1500).min() < -0.05
    return on, off


def test_six_dof_servo_rests_on_the_board():
    pos, _, _, table = run_tool(OracleDriver, free=False).state()
    assert pos[2] > 0.018
    assert table[2] > 0


def test_free_knife_falls_onto_the_board():
    run_tool(OracleDriver, free=True)


def test_guided_knife_stops_on_the_board_without_rotating():
    _, rot, _, table = guided(OracleDriver).state()
    np.testing.assert_allclose(rot, [0, 0, 0, 1], atol=1e-7)
    assert table[2] > 0


def test_board_contact_ends_at_the_board_edge():
    board_edge(OracleDriver)


@pytest.mark.gpu
def test_knife_drives_cuda_match_oracle():
    pairs = [(run_tool(CudaDriver, free), run_tool(OracleDriver, free)) for free in (False, True)]
    pairs.append((guided(CudaDriver), guided(OracleDriver)))
    pairs.extend(zip(board_edge(CudaDriver), board_edge(OracleDriver)))
    for g, c in pairs:
        for a, b in zip(g.state(), c.state()):
            np.testing.assert_array_equal(np.asarray(a), np.asarray(b).astype(np.asarray(a).dtype))


# --------------------------------------------------------------- capacity

@pytest.mark.parametrize("spacing, nodes", [(0.015, 45), (0.0075, 225), (0.00375, 1377)])
def test_capacity_follows_the_reference_geometry(spacing, nodes):
    # tests/test_stress_replays.py:72-80 and 61-69
    cfg = Config(grid_spacing=spacing)
    reference, origin, cells = points(cfg.size, cfg.grid_spacing, cfg.shape, cfg.sampling_seed)
    node_ids, _, _ = stencil(reference, origin, cfg.grid_spacing, cells)
    assert int(np.prod(cells + 1)) == nodes
    assert node_ids.min() == 0 and node_ids.max() + 1 == nodes
    digits = cut_capacity(nodes) + 1
    # every code of `digits` ternary digits keys every node within int64, one more digit would not
    assert nodes * 3**digits - 1 <= np.iinfo(np.int64).max < nodes * 3 ** (digits + 1) - 1
    if nodes == 225:
        assert digits == 34  # test_stress_replays.py:51-53
    else:
        assert digits != 34


# ------------------------------------------------------------- deep digit

def test_cut_index_beyond_32_bit_digits_still_severs():
    # tests/test_coupling.py:131-145: the banana preset with an external knife descending
    # at 20 mm/s for 1.9 s, cut index 25: all three side values at that digit, two pieces
    # of more than 30 % each.
    from blademaster_gb300.presets import banana_config

    cfg = replace(banana_config(), external_tool=True)
    c = OracleSolver(cfg)
    assert cut_capacity(c.node_count) >= 29
    half, cut = cfg.blade_half_size[2], 25
    for i in range(1900):
        edge = max(0.0, 0.036 - 0.02 * i * 0.001)
        state = ToolState([0.0, 0.0, edge + half], [0, 0, 0, 1], [0.0, 0.0, -0.02], [0, 0, 0])
        c.external_interval(packed(state), round(0.001 / cfg.dt), cutting=True, cut_index=cut)
    codes = c.get("codes")
    assert set(np.unique(codes // 3**cut)) == {0, 1, 2}
    _, sizes = components(c.node_numpy, c.weight_numpy, codes)
    assert len(sizes) == 2 and sizes.min() > 0.3 * c.n


# ----------------------------------------------------------- auto strokes

class Strokes:
    """The reference's contact-stroke rule (teleop_input.py:239-266), the caller of the embedded count: a
    stroke starts when particles are embedded beside the blade and ends once none has been for `clear_s`;
    the cut index advances as it ends."""

    def __init__(self, clear_s=0.02):
        self.clear_s, self.cut_index, self.strokes, self.inside, self.out_for = clear_s, 0, 0, False, 0.0

    def update(self, embedded, dt):
        if embedded:
            self.strokes += not self.inside
            self.inside, self.out_for = True, 0.0
        elif self.inside:
            self.out_for += dt
            if self.out_for >= self.clear_s:
                self.cut_index, self.inside = self.cut_index + 1, False
        return self.cut_index


def stroke_states(half, dt=0.001):
    """tests/test_coupling.py:154-171: the edge goes down through x = -25 mm, back out, over, down through
    x = +25 mm and out again; one ToolState per 1 ms interval, with the velocity of its leg."""
    legs = [(-0.025, 0.0, 0.9), (-0.025, 0.0, 0.1), (-0.025, 0.04, 0.6), (0.025, 0.04, 0.8),
            (0.025, 0.0, 1.0), (0.025, 0.0, 0.1), (0.025, 0.04, 0.6)]
    path = [(-0.025, 0.036)]
    for x, z, seconds in legs:
        x0, z0 = path[-1]
        path += [(x0 + (x - x0) * k * dt / seconds, z0 + (z - z0) * k * dt / seconds)
                 for k in range(1, round(seconds / dt) + 1)]
    return [ToolState([x1, 0.0, z1 + half], [0, 0, 0, 1], [(x1 - x0) / dt, 0.0, (z1 - z0) / dt], [0, 0, 0])
            for (x0, z0), (x1, z1) in zip(path, path[1:])]


def embedded_bounds(x, tool, spacing, half, margin=1e-6):
    """contact.count_embedded (contact.py:1042-1055) in float64 numpy: the particles inside the band box
    by more than `margin` (m), and those inside it or within `margin` of its faces."""
    qx, qy, qz, qw = tool[6:10] / np.linalg.norm(tool[6:10])
    R = np.array([[1 - 2 * (qy * qy + qz * qz), 2 * (qx * qy - qz * qw), 2 * (qx * qz + qy * qw)],
                  [2 * (qx * qy + qz * qw), 1 - 2 * (qx * qx + qz * qz), 2 * (qy * qz - qx * qw)],
                  [2 * (qx * qz - qy * qw), 2 * (qy * qz + qx * qw), 1 - 2 * (qx * qx + qy * qy)]])
    local = np.abs((x.astype(np.float64) - tool[0:3]) @ R)  # rows are R^T (x - pos)
    box = np.array([6.0 * spacing, half[1], half[2]])
    return int(np.all(local < box - margin, axis=1).sum()), int(np.all(local <= box + margin, axis=1).sum())


def test_auto_strokes_label_each_cut_plane_with_its_own_digit():
    # tests/test_coupling.py:147-186: the embedded-particle count drives the stroke rule; two strokes,
    # each labelled with its own digit, three pieces, and withdrawing from the first kerf writes no second
    # digit.  Every interval's count also lies within the float64 count's margin band.
    from blademaster_gb300.presets import banana_config

    cfg = replace(banana_config(), external_tool=True)
    c, strokes = OracleSolver(cfg), Strokes()
    steps, before, inside = round(0.001 / cfg.dt), None, 0
    for state in stroke_states(cfg.blade_half_size[2]):
        before = c.get("codes").copy() if strokes.strokes == 1 else before
        c.external_interval(packed(state), steps, cutting=True, cut_index=strokes.cut_index)
        n = c.embedded_particles()
        lo, hi = embedded_bounds(c.get("x"), c.get("tool")[0], cfg.grid_spacing, cfg.blade_half_size)
        assert lo <= n <= hi
        inside += n > 0
        strokes.update(n > 0, 0.001)
    assert inside > 1000 and n == 0
    assert strokes.strokes == 2 and strokes.cut_index == 2
    assert np.all((before // 3) % 3 == 0)
    codes = c.get("codes")
    assert np.any((codes // 3) % 3 != 0)
    _, sizes = components(c.node_numpy, c.weight_numpy, codes)
    assert len(sizes) == 3


# ------------------------------------------------------ several free knives

def two_knives(**kwargs):
    """tests/test_multi_tool.py:8-18"""
    return OracleSolver(Config(size=(0.06, 0.03, 0.03), grid_spacing=0.0075, dt=0.0005, free_blade=True, tool_count=2,
                               blade_half_size=(0.0005, 0.025, 0.02), **kwargs))


def test_only_free_knives_may_be_several():
    # test_multi_tool.py:21-26
    for kwargs in ({}, {"pose_servo": True}, {"external_tool": True}):
        with pytest.raises(ValueError):
            Config(tool_count=2, **kwargs)
    with pytest.raises(ValueError):
        Config(tool_count=0)


def dropped(xs, steps):
    """test_multi_tool.py:29-36: two knives dropped at 0.6 m/s into the block."""
    c = two_knives()
    z = 0.03 + 0.02 + 0.002
    c.set("tool_pos", [[x, 0.0, z] for x in xs])
    c.set("tool_vel", [[0.0, 0.0, -0.6]] * 2)
    for _ in range(steps):
        c.step(cutting=True)
    return c


def test_knife_index_does_not_matter():
    # test_multi_tool.py:39-44: swapping the knives' slots moves nothing beyond rounding
    a, b = dropped([-0.015, 0.015], 100), dropped([0.015, -0.015], 100)
    np.testing.assert_allclose(a.get("tool_pos"), b.get("tool_pos")[::-1], atol=1.0e-7)
    np.testing.assert_allclose(a.get("x"), b.get("x"), atol=1.0e-6)


def test_mirrored_knives_move_alike_and_label_their_own_digits():
    # test_multi_tool.py:47-65 (60 steps keep the edges above the board)
    steps = 60
    c = dropped([-0.015, 0.015], steps)
    p, v = c.get("tool_pos"), c.get("tool_vel")
    np.testing.assert_allclose(p[0] * [-1, 1, 1], p[1], atol=1.0e-7)
    np.testing.assert_allclose(v[0] * [-1, 1, 1], v[1], atol=1.0e-5)
    assert 0.0 < p[0, 2] - 0.02 < 0.028
    assert v[0, 2] > -0.6 - 9.81 * steps * 0.0005
    codes = c.get("codes")
    first, second = codes % 3, (codes // 3) % 3
    assert set(np.unique(first)) == {0, 1, 2} and set(np.unique(second)) == {0, 1, 2}
    assert np.all(codes < 9)
    ref = c.reference
    assert ref[first == 1, 0].max() < -0.015 < ref[first == 2, 0].min()
    assert ref[second == 1, 0].max() < 0.015 < ref[second == 2, 0].min()


def test_knife_beside_the_block_falls_freely():
    # test_multi_tool.py:68-80
    c = two_knives()
    z0 = 0.2
    c.set("tool_pos", [[-0.015, 0.0, 0.03 + 0.02 + 0.002], [0.2, 0.0, z0]])
    n = 100
    for _ in range(n):
        c.step(cutting=True)
    dt, g = 0.0005, 9.81
    pos, vel = c.get("tool_pos"), c.get("tool_vel")
    assert vel[1, 2] == pytest.approx(-g * n * dt, rel=1.0e-5)
    assert pos[1, 2] == pytest.approx(z0 - g * dt * dt * n * (n + 1) / 2, abs=1.0e-6)
    np.testing.assert_allclose(pos[1, :2], [0.2, 0.0], atol=1.0e-9)


@pytest.mark.parametrize("first", [0, 1])
def test_each_knife_pays_its_own_cutting_work(first):
    # test_multi_tool.py:83-106: one particle under knife `first`, the others far away
    c = two_knives(cutting_energy=1.0)
    x = c.reference.copy()
    x[:, 0] += 10
    x[0] = [0, 0, 0.039]
    c.set("x", x)
    positions = np.array([[3.0, 0, 0.06], [3.0, 0, 0.06]])
    positions[first, 0] = 0
    c.set("tool_pos", positions)
    c.set("tool_vel", [[0, 0, -1], [0, 0, -1]])
    c.rigid_contacts(True)
    initial = c.get("reaction")[first].copy()
    assert c.get("tool_damage")[first][0] == 1
    assert c.get("tool_damage")[1 - first][0] == 0
    positions[:, 0] = positions[::-1, 0]
    c.set("tool_pos", positions)
    c.set("acc", 0)
    c.rigid_contacts(True)
    np.testing.assert_allclose(c.get("reaction")[1 - first], initial, rtol=1e-6)
    assert c.get("tool_damage")[1 - first][0] == 1
    c.set_cut(2)
    assert not c.get("tool_damage").any()


def turn(v):
    """Unit quaternion (xyzw) of the rotation vector v."""
    v = np.asarray(v, float)
    a = np.linalg.norm(v)
    return np.r_[np.sin(a / 2) * v / a, np.cos(a / 2)] if a > 0 else np.array([0.0, 0.0, 0.0, 1.0])


def compose(a, b):
    """Hamilton product a * b of xyzw quaternions."""
    (ax, ay, az, aw), (bx, by, bz, bw) = a, b
    return np.array([aw * bx + ax * bw + ay * bz - az * by, aw * by - ax * bz + ay * bw + az * bx,
                     aw * bz + ax * by - ay * bx + az * bw, aw * bw - ax * bx - ay * by - az * bz])


SHARED = np.array([[0.0007, -0.004, 0.039], [-0.0007, 0.003, 0.039], [0.0004, 0.006, 0.0388], [0.0002, -0.006, 0.0392]])


class Knives:
    """The contact probe of scripts/stress_multi_tool.py:46-117 on the oracle: four particles that every
    knife touches (the rest of the block parked 10 m up, where only gravity acts), and one contact pass
    (blade, board and cut damage) per call with the knives' state set and the interval sums cleared."""

    def __init__(self, cfg):
        self.o = o = OracleSolver(cfg)
        x = np.column_stack([10 + 0.01 * np.arange(o.n), np.zeros(o.n), np.full(o.n, 10.0)])
        x[:4] = SHARED
        o.set("x", x.astype(np.float32))
        self.count = cfg.tool_count

    def contact(self, p, v, q, w, cutting, cut_index):
        o, A = self.o, self.o.arrays
        o.set_cut(cut_index)
        o.set("tool_pos", p), o.set("tool_vel", v), o.set("tool_rot", q), o.set("tool_omega", w)
        A["acc"][:] = 0
        A["speed"][:] = 0
        o.rigid_contacts(o.cut_bits(cutting))
        return dict(damage=A["damage"][:, o.rank][:, :4].copy(),
                    friction=A["histories"][1 : 1 + self.count][:, o.rank][:, :4].copy(),
                    reaction=o.get("reaction").copy(), torque=o.get("torque").copy(),
                    impulses=o.get("impulses").astype(float), board=o.get("board").copy(), work=o.get("work").copy())


@pytest.mark.parametrize("motion", ["fixed", "crossing"])
@pytest.mark.parametrize("seed", [0, 17, 913])
@pytest.mark.parametrize("count", [2, 3])
def test_simultaneous_knives_preserve_independent_contacts(motion, seed, count):
    # scripts/stress_multi_tool.py:289-418 as tests/test_multi_tool.py:108-116 ("fixed": the knives hold
    # their places and reverse) and tests/test_stress_replays.py:95-107 ("crossing": they cross each other
    # and turn) run it: two or three free knives cut the same four particles.  In every slot order each
    # knife's damage, friction history, reaction and torque equal that knife's contact alone; the
    # particles' impulses and the cutting work are the single knives' sums; momentum balances.
    from itertools import permutations

    rng = np.random.default_rng(seed)
    cfg = Config(free_blade=True, tool_count=count, cutting_energy=80.0)
    poses = np.tile([0.0, 0.0, 0.06], (count, 1))
    poses[:, 0] = np.linspace(-0.0003, 0.0003, count)
    velocities = rng.uniform(-0.08, 0.08, (count, 3))
    velocities[:, 2] = -np.linspace(0.25, 0.65, count)
    omegas = rng.uniform(-0.3, 0.3, (count, 3))
    rotations = np.array([turn(v) for v in rng.uniform(-0.004, 0.004, (count, 3))])
    crossing = motion == "crossing"
    if crossing:
        velocities[:, 0] = -2 * poses[:, 0] / (9 * cfg.dt)
        omegas[:, 2] += np.linspace(8.0, -8.0, count)
        rotations = np.array([turn([0, 0, a]) for a in np.linspace(-0.08, 0.08, count)])
    baseline = None
    for order in map(np.asarray, permutations(range(count))):
        inverse = np.argsort(order)
        together, alone = Knives(cfg), [Knives(replace(cfg, tool_count=1)) for _ in order]
        gravity = np.array([0.0, 0.0, -9.81 * float(np.float32(together.o.mass)) * float(np.float32(cfg.dt))])
        trace = []
        for tick in range(12):
            p, v, w, q = poses.copy(), velocities.copy(), omegas.copy(), rotations.copy()
            if crossing:
                elapsed = (tick - min(2, max(0, tick - 5))) * cfg.dt
                p[:, 0] += velocities[:, 0] * elapsed
                q = np.array([compose(turn(omega * elapsed), r) for omega, r in zip(omegas, rotations)])
            if tick in (3, 4):
                p[0, 0] += 0.2  # one knife leaves; the others keep their histories
            if tick in (6, 7):
                v[:] = w[:] = 0.0
            if tick >= 8:
                v[:, 1] *= -1
                if not crossing:
                    v[:, 0] *= -1
            cutting, cut_index = tick not in (6, 7), count if tick >= 9 else 0
            state = together.contact(p[order], v[order], q[order], w[order], cutting, cut_index)
            singles = [k.contact(p[i : i + 1], v[i : i + 1], q[i : i + 1], w[i : i + 1], cutting, cut_index)
                       for i, k in enumerate(alone)]
            for key in ("damage", "friction", "reaction", "torque"):
                state[key] = state[key][inverse]
                np.testing.assert_allclose(state[key], np.concatenate([s[key] for s in singles]), rtol=2e-5,
                                           atol=1e-9, err_msg=f"{key}, tick {tick}")
            np.testing.assert_allclose(state["impulses"], sum(s["impulses"] for s in singles) - (count - 1) * gravity,
                                       rtol=2e-5, atol=1e-9)
            np.testing.assert_allclose(state["work"], sum(s["work"] for s in singles), rtol=2e-5, atol=1e-9)
            residual = (state["impulses"].sum(0) + state["reaction"].sum(0) - together.o.n * gravity
                        - state["board"].sum(0))
            np.testing.assert_allclose(residual, 0, atol=1e-9)
            if tick == 2:
                assert np.all(state["damage"] > 0), "the knives must damage the same particles"
                assert np.all(np.linalg.norm(state["friction"], axis=(1, 2)) > 0)
                assert np.all(np.linalg.norm(state["torque"], axis=1) > 0)
                assert not np.allclose(state["friction"][0], state["friction"][1], atol=1e-9)
            if tick == 4:
                np.testing.assert_array_equal(state["friction"][0], 0)
                np.testing.assert_array_equal(state["reaction"][0], 0)
                assert np.linalg.norm(state["friction"][1:]) > 0
            if tick in (6, 7):
                np.testing.assert_array_equal(state["damage"], trace[-1]["damage"])
            trace.append(state)
        if baseline is None:
            baseline = trace
        else:
            for tick, (actual, first) in enumerate(zip(trace, baseline)):
                for key in first:
                    np.testing.assert_allclose(actual[key], first[key], rtol=2e-5, atol=1e-9,
                                               err_msg=f"order {order}, tick {tick}, {key}")
    if crossing:
        crossed = sum((poses[a, 0] - poses[b, 0]) * (p[a, 0] - p[b, 0]) < 0
                      for a in range(count) for b in range(a + 1, count))
        assert crossed == count * (count - 1) // 2
        assert np.max(2 * np.arccos(np.clip(np.abs(np.sum(q * rotations, axis=1)), 0, 1))) > 0.03


def canonical_codes(codes, order, strokes):
    """scripts/stress_multi_tool.py:135-146: codes written with knife order[slot] in slot `slot`, rewritten
    as if every knife sat in the slot of its own identity (each stroke owns len(order) digits)."""
    codes = np.asarray(codes, dtype=np.int64)
    count, out = len(order), np.zeros_like(codes)
    if np.any(codes // 3 ** (strokes * count)):
        raise AssertionError("Unexpected cut digit outside the replay history")
    for stroke in range(strokes):
        for slot, identity in enumerate(order):
            out += (codes // 3 ** (stroke * count + slot)) % 3 * 3 ** (stroke * count + identity)
    return out


def test_permutation_maps_each_strokes_ternary_digits():
    # tests/test_multi_tool.py:119-125: slot order C, A, B: [1,2,2; 1,1,2] becomes A, B, C: [2,2,1; 1,2,1]
    np.testing.assert_array_equal(canonical_codes([619, 0], [2, 0, 1], 2), [449, 0])
    with pytest.raises(AssertionError, match="Unexpected cut digit"):
        canonical_codes([3**6], [2, 0, 1], 2)


def test_three_knives_full_trajectory_and_cut_history_permutation():
    # tests/test_multi_tool.py:128-133 with scripts/stress_multi_tool.py:422-537: three free knives fall
    # into the block (two strokes of 60 substeps) in every slot order, and once again in the first order.
    # After the knives and their cut digits are mapped back to their identities, every run equals the
    # first within the reference's bounds (10 ppm of a cell in position, 5 ppm of a cell per step in
    # velocity, 1e-4 in damage, 10 uN of force), side codes and pieces exactly; momentum balances
    # each substep to 50 ppm of one substep's gravity impulse, and every knife cuts in both strokes.
    from itertools import permutations

    count, steps = 3, 120
    cfg = Config(free_blade=True, tool_count=count, cache_topology=True, grid_storage="compact", dt=0.0005)
    rng = np.random.default_rng(17)
    poses = np.tile([0.0, 0.0, 0.052], (count, 1))
    poses[:, 0] = np.linspace(-0.001, 0.001, count)
    velocities = rng.uniform(-0.015, 0.015, (count, 3))
    velocities[:, 2] = -np.linspace(0.4, 0.6, count)
    omegas = rng.uniform(-0.1, 0.1, (count, 3))
    rotations = np.array([turn(v) for v in rng.uniform(-0.005, 0.005, (count, 3))])
    h, dt = cfg.grid_spacing, cfg.dt
    speed, impulse = 5e-6 * h / dt, 1e-5 * dt
    atol = dict(position=1e-5 * h, velocity=speed, deformation=5e-6, plastic_deformation=1e-7,
                blade_position=1e-5 * h, blade_velocity=speed, blade_orientation=1e-7,
                blade_omega=speed / float(np.linalg.norm(cfg.blade_half_size)), tool_damage=1e-4,
                friction=1e-5 * h, reaction=impulse, torque=impulse * float(np.linalg.norm(cfg.blade_half_size)))
    orders = list(permutations(range(count)))
    baseline, shared = None, 0
    for order in map(np.asarray, [orders[0], *orders]):
        inverse = np.argsort(order)
        o = OracleSolver(cfg)
        o.set("tool_pos", poses[order]), o.set("tool_vel", velocities[order])
        o.set("tool_rot", rotations[order]), o.set("tool_omega", omegas[order])
        mass, total = float(o.mass), float(o.mass) * o.n + cfg.blade_mass * count
        trace, old = [], np.zeros(o.n, np.int64)
        previous_v, previous_blade = o.get("v").astype(float), o.get("tool_vel").astype(float)
        for tick in range(steps):
            o.step(cutting=True, cut_index=int(tick >= steps // 2) * count)
            v, blade_v = o.get("v").astype(float), o.get("tool_vel").astype(float)
            delta = mass * (v - previous_v).sum(0) + cfg.blade_mass * (blade_v - previous_blade).sum(0)
            # the board's impulses of this substep on the particles and (table_impulse) on the knives
            external = np.array([0.0, 0.0, -9.81 * total * dt]) + o.get("board").sum(0) + o.get("table_impulse").sum(0)
            np.testing.assert_allclose(delta, external, atol=5e-5 * 9.81 * total * dt, rtol=0, err_msg=f"tick {tick}")
            previous_v, previous_blade = v, blade_v
            sides = canonical_codes(o.get("codes"), order, 2)
            for digit in range(2 * count):  # a written digit never changes
                before, now = (old // 3**digit) % 3, (sides // 3**digit) % 3
                np.testing.assert_array_equal(now[before != 0], before[before != 0])
            old = sides
            labels, sizes = components(o.node_numpy, o.weight_numpy, sides)
            state = dict(position=o.get("x").copy(), velocity=o.get("v").copy(), deformation=o.get("F").copy(),
                         plastic_deformation=o.get("Fp").copy(), blade_position=o.get("tool_pos")[inverse].copy(),
                         blade_velocity=o.get("tool_vel")[inverse].copy(),
                         blade_orientation=o.get("tool_rot")[inverse].copy(),
                         blade_omega=o.get("tool_omega")[inverse].copy(), tool_damage=o.get("tool_damage")[inverse].copy(),
                         friction=o.arrays["histories"][1 : 1 + count][:, o.rank][inverse].copy(),
                         reaction=o.get("reaction")[inverse], torque=o.get("torque")[inverse],
                         sides=sides, component_labels=labels, component_sizes=sizes)
            shared = max(shared, int(np.count_nonzero(np.sum(state["tool_damage"] > 0, axis=0) >= 2)))
            trace.append(state)
        for stroke in range(2):
            for identity in range(count):
                assert np.any((old // 3 ** (stroke * count + identity)) % 3), "missing cut history"
        if baseline is None:
            baseline = trace
            continue
        for tick, (actual, first) in enumerate(zip(trace, baseline)):
            for key, value in first.items():
                if key in atol:
                    np.testing.assert_allclose(actual[key], value, rtol=0, atol=atol[key],
                                               err_msg=f"order {order}, tick {tick}, {key}")
                else:
                    np.testing.assert_array_equal(actual[key], value, err_msg=f"order {order}, tick {tick}, {key}")
    assert shared > 0, "no particle was cut by several knives"


# -------------------------------------------------------- cutting resistance

RESIST_SIZE = (0.04, 0.02, 0.024)


def steady_force(cutting_energy, **kwargs):
    """Mean knife force while the edge is pushed from 4 to 12 mm depth at 50 mm/s
    (test_cut_resistance.py:74-99), on the oracle."""
    cfg = Config(size=RESIST_SIZE, grid_spacing=0.006, dt=0.0001, young_modulus=400000.0, poisson_ratio=0.4,
                 yield_stress=40000.0, cutting_energy=cutting_energy, blade_half_size=(0.0005, 0.015, 0.02),
                 external_tool=True, grid_storage="compact", **kwargs)
    c = OracleSolver(cfg)
    hz, speed, interval = cfg.blade_half_size[2], 0.05, 0.002
    steps = round(interval / cfg.dt)
    edges, forces = [], []
    for i in range(int(0.016 / speed / interval)):
        edge = RESIST_SIZE[2] + 0.002 - speed * i * interval
        state = ToolState([0.0, 0.0, edge + hz], [0, 0, 0, 1], [0, 0, -speed], [0, 0, 0])
        impulse, _, _ = c.external_interval(packed(state), steps, cutting=True, cut_index=0)
        forces.append(float(impulse[2]) / interval)
        edges.append(edge)
    depth = RESIST_SIZE[2] - np.array(edges)
    return np.mean(np.array(forces)[(depth > 0.004) & (depth < 0.012)])


def test_paper_resistance_stops_growing_with_cutting_energy():
    # test_cut_resistance.py:103-106: particles slide around the edge before their damage work is paid
    low, high = steady_force(100.0), steady_force(1000.0)
    assert high == pytest.approx(low, rel=0.05)


def test_held_particles_make_the_force_grow_with_cutting_energy():
    # test_cut_resistance.py:109-111
    low, high = steady_force(100.0, cut_hold=True), steady_force(1000.0, cut_hold=True)
    assert high > 3.0 * low > 0.0


# ------------------------------------------------------------- single field

def set_single_field(c, enabled):
    """Solver.set_single_field (solver.py:382-389) on the oracle: the transfers' codes switch
    and the topology is marked dirty."""
    from blademaster_gb300 import _native

    if bool(enabled) != c.single_field:
        c.single_field = bool(enabled)
        c.arrays["flags"][_native.FLAG["TOPOLOGY_DIRTY"]] = 1


HALVES = Config(size=(0.06, 0.03, 0.03), grid_spacing=0.0075, dt=0.0005)


def pushed_halves(single_field, steps=40, arrays=False):
    """test_single_field.py:7-18: the left half (code 1) pushed at -0.2 m/s against the right (code 2).

    Returns the mean x velocity of each half and the codes, or with arrays=True the oracle itself."""
    c = OracleSolver(HALVES)
    left = c.reference[:, 0] < 0
    c.set("codes", np.where(left, 1, 2).astype(np.int64))
    v = np.zeros((c.n, 3), np.float32)
    v[left, 0] = -0.2
    c.set("v", v)
    set_single_field(c, single_field)
    for _ in range(steps):
        c.step(target_edge=(0.0, 0.0, 0.2), cutting=False)
    if arrays:
        return c
    v = c.get("v")
    return v[~left, 0].mean(), v[left, 0].mean(), c.get("codes")


def test_cut_halves_move_independently():
    # test_single_field.py:21-25
    right, left, sides = pushed_halves(False)
    assert abs(right) < 0.005
    assert left < -0.1
    assert set(np.unique(sides)) == {1, 2}


def test_single_field_drags_the_other_half():
    # test_single_field.py:28-31
    right, _, sides = pushed_halves(True)
    assert right < -0.05
    assert set(np.unique(sides)) == {1, 2}


def test_switching_back_restores_separation():
    # test_single_field.py:34-46, with the cached topology rebuilt on the switch
    c = OracleSolver(replace(HALVES, cache_topology=True))
    left = c.reference[:, 0] < 0
    c.set("codes", np.where(left, 1, 2).astype(np.int64))
    set_single_field(c, True)
    c.advance(np.tile([0.0, 0.0, 0.2], (4, 1)), cutting=False)
    assert c.single_field
    set_single_field(c, False)
    v = np.zeros((c.n, 3), np.float32)
    v[left, 0] = -0.2
    c.set("v", v)
    c.advance(np.tile([0.0, 0.0, 0.2], (40, 1)), cutting=False)
    assert abs(c.get("v")[~left, 0].mean()) < 0.005


# ------------------------------------------------------- CUDA twins of the above

@pytest.mark.gpu
def test_deep_digit_severs_on_cuda_and_matches_the_oracle_first():
    # test_coupling.py:131-145 on the CUDA solver; its first 100 intervals bit-exact with the oracle
    from blademaster_gb300.coupling import ExternalToolPort
    from blademaster_gb300.presets import banana_config
    from blademaster_gb300.solver import Solver

    cfg = replace(banana_config(), external_tool=True)
    g, c = Solver(cfg), OracleSolver(cfg)
    port = ExternalToolPort(g)
    half, cut, steps = cfg.blade_half_size[2], 25, round(0.001 / cfg.dt)
    for i in range(1900):
        edge = max(0.0, 0.036 - 0.02 * i * 0.001)
        state = ToolState([0.0, 0.0, edge + half], [0, 0, 0, 1], [0.0, 0.0, -0.02], [0, 0, 0])
        port.advance(state, 0.001, cutting=True, cut_index=cut)
        if i < 100:
            c.external_interval(packed(state), steps, cutting=True, cut_index=cut)
        if i == 99:
            for name in ("x", "v", "codes", "damage"):
                np.testing.assert_array_equal(getattr(g, name).numpy(), c.get(name), err_msg=name)
    codes = g.codes.numpy()
    assert set(np.unique(codes // 3**cut)) == {0, 1, 2}
    _, sizes = g.components()
    assert len(sizes) == 2 and sizes.min() > 0.3 * g.n


@pytest.mark.gpu
def test_auto_strokes_on_cuda_match_the_oracle():
    # test_coupling.py:147-186 on the CUDA solver: every interval's embedded count (Solver.embedded_particles,
    # solver.py:892-900) equals the oracle's, embedded_particles_previous (solver.py:902-918) lags it by one
    # call, and the strokes, digits, codes and pieces come out as on the oracle
    from blademaster_gb300.coupling import ExternalToolPort
    from blademaster_gb300.presets import banana_config
    from blademaster_gb300.solver import Solver

    cfg = replace(banana_config(), external_tool=True)
    g, c = Solver(cfg), OracleSolver(cfg)
    port, strokes, steps = ExternalToolPort(g), Strokes(), round(0.001 / cfg.dt)
    counts, previous = [], []
    for i, state in enumerate(stroke_states(cfg.blade_half_size[2])):
        port.advance(state, 0.001, cutting=True, cut_index=strokes.cut_index)
        c.external_interval(packed(state), steps, cutting=True, cut_index=strokes.cut_index)
        counts.append(g.embedded_particles())
        assert counts[-1] == c.embedded_particles(), f"interval {i}"
        previous.append(g.embedded_particles_previous())
        strokes.update(counts[-1] > 0, 0.001)
    assert previous[0] == 0 and previous[1:] == counts[:-1]
    assert strokes.strokes == 2 and strokes.cut_index == 2
    for name in ("x", "v", "codes", "damage"):
        np.testing.assert_array_equal(getattr(g, name).numpy(), c.get(name), err_msg=name)
    _, sizes = g.components()
    assert len(sizes) == 3


def cuda_two_knives(**kwargs):
    from blademaster_gb300.solver import Solver

    return Solver(Config(size=(0.06, 0.03, 0.03), grid_spacing=0.0075, dt=0.0005, free_blade=True, tool_count=2,
                         blade_half_size=(0.0005, 0.025, 0.02), **kwargs))


@pytest.mark.gpu
def test_several_knives_on_cuda_match_the_oracle():
    # test_multi_tool.py:29-80 scenes, bit-exact with the oracle
    z = 0.03 + 0.02 + 0.002
    for xs, steps in (([-0.015, 0.015], 60), ([0.015, -0.015], 100)):
        g, c = cuda_two_knives(), dropped(xs, steps)
        g.tool_pos.assign([[x, 0.0, z] for x in xs])
        g.tool_vel.assign([[0.0, 0.0, -0.6]] * 2)
        for _ in range(steps):
            g.step(cutting=True)
        for name in ("x", "v", "codes"):
            np.testing.assert_array_equal(getattr(g, name).numpy(), c.get(name), err_msg=name)
        np.testing.assert_array_equal(g.tool_pos.numpy(), c.get("tool_pos").astype(np.float32))
    g = cuda_two_knives()
    g.tool_pos.assign([[-0.015, 0.0, z], [0.2, 0.0, 0.2]])
    for _ in range(100):
        g.step(cutting=True)
    assert g.state()["blade_velocity"][1, 2] == pytest.approx(-9.81 * 100 * 0.0005, rel=1.0e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("first", [0, 1])
def test_each_knife_pays_its_own_cutting_work_on_cuda(first):
    # test_multi_tool.py:83-106 on the CUDA solver
    g = cuda_two_knives(cutting_energy=1.0)
    x = g.reference.copy()
    x[:, 0] += 10
    x[0] = [0, 0, 0.039]
    g.x.assign(x)
    positions = np.array([[3.0, 0, 0.06], [3.0, 0, 0.06]])
    positions[first, 0] = 0
    g.tool_pos.assign(positions)
    g.tool_vel.assign([[0, 0, -1], [0, 0, -1]])
    g.rigid_contacts(True)
    initial = g.reaction.numpy()[first].copy()
    assert g.tool_damage[first].numpy()[0] == 1 and g.tool_damage[1 - first].numpy()[0] == 0
    positions[:, 0] = positions[::-1, 0]
    g.tool_pos.assign(positions)
    g.reaction.zero_()
    g.torque.zero_()
    g.rigid_contacts(True)
    np.testing.assert_allclose(g.reaction.numpy()[1 - first], initial, rtol=1e-6)
    assert g.tool_damage[1 - first].numpy()[0] == 1
    g._set_cut(2)
    assert all(not d.numpy().any() for d in g.tool_damage)


@pytest.mark.gpu
def test_single_field_halves_on_cuda_match_the_oracle():
    # test_single_field.py:7-31 on the CUDA solver, bit-exact with the oracle after 40 substeps
    from blademaster_gb300.solver import Solver

    for single in (False, True):
        g = Solver(HALVES)
        left = g.reference[:, 0] < 0
        g.codes.assign(np.where(left, 1, 2).astype(np.int64))
        v = np.zeros((g.n, 3), np.float32)
        v[left, 0] = -0.2
        g.v.assign(v)
        g.set_single_field(single)
        for _ in range(40):
            g.step(target_edge=(0.0, 0.0, 0.2), cutting=False)
        o = pushed_halves(single, arrays=True)
        for name in ("x", "v", "F", "stress", "codes"):
            np.testing.assert_array_equal(getattr(g, name).numpy(), o.get(name), err_msg=f"{name} single={single}")


@pytest.mark.gpu
def test_steady_cutting_force_on_cuda_matches_the_oracle():
    # test_cut_resistance.py:74-111 scene on the CUDA solver: the same interval forces as the oracle
    from blademaster_gb300.coupling import ExternalToolPort
    from blademaster_gb300.solver import Solver

    for kwargs in ({}, {"cut_hold": True}):
        cfg = Config(size=RESIST_SIZE, grid_spacing=0.006, dt=0.0001, young_modulus=400000.0, poisson_ratio=0.4,
                     yield_stress=40000.0, cutting_energy=1000.0, blade_half_size=(0.0005, 0.015, 0.02),
                     external_tool=True, grid_storage="compact", **kwargs)
        g, c = Solver(cfg), OracleSolver(cfg)
        port = ExternalToolPort(g)
        for i in range(40):
            edge = RESIST_SIZE[2] + 0.002 - 0.05 * i * 0.002
            state = ToolState([0.0, 0.0, edge + 0.02], [0, 0, 0, 1], [0, 0, -0.05], [0, 0, 0])
            r = port.advance(state, 0.002, cutting=True, cut_index=0)
            impulse, _, _ = c.external_interval(packed(state), 20, cutting=True, cut_index=0)
            np.testing.assert_array_equal(r.impulse_ns, impulse)
