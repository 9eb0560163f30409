"""The oracle pinned to the reference's own known-answer tests.

Each test restates one of the reference's tests (cited per test) on the CPU
oracle, with the reference's inputs, expected values and tolerances.  Where
the reference compares against its external FP64 oracle (DexLab, pinned at
b955d85 and not available here), the expected values come from float64
restatements written in this file, independently of oracle/oracle.c:

* Eq. 8 field exchange as a dense matrix product over a compatibility mask;
* the blade's signed distance as the distance to a convex polygon extruded
  along y (a different construction from the reference's feature walk);
* the stick/slip friction law in float64;
* one TLMPM material step (P2G over (node, code) fields, Eq. 8, grid
  velocities, G2P with Eq. 13 advection, the MUSL re-scatter and the F
  update with the corotated stress from a float64 SVD), as dense numpy.

These tests never touch a GPU.
"""

import ctypes
from dataclasses import replace

import numpy as np
import pytest

from blademaster_gb300.coupling import ToolState
from blademaster_gb300.geometry import points, stencil
from blademaster_gb300.solver import Config
from oracle.oracle import OracleSolver, fx_to_float, lib, ptr

F32 = np.float32


def compatible(a, b):
    """Ternary cut codes: incompatible when some digit is non-zero in both and differs."""
    while a or b:
        x, y = a % 3, b % 3
        if x and y and x != y:
            return False
        a, b = a // 3, b // 3
    return True


# ------------------------------------------------------------------ stencil


def test_partition_of_unity_and_reference_gradient():
    # tests/test_mechanics.py:74-77
    cfg = Config()
    x, origin, cells = points(cfg.size, cfg.grid_spacing, cfg.shape, cfg.sampling_seed)
    _, w, g = stencil(x, origin, cfg.grid_spacing, cells)
    np.testing.assert_allclose(w.astype(F32).sum(1), 1, atol=2e-7)
    np.testing.assert_allclose(g.astype(F32).sum(1), 0, atol=2e-5)


# ----------------------------------------------------------------- exchange


def exchange_fp64(codes, masses, states):
    """Eq. 8: s_a + sum over compatible b != a of (m_a s_b - m_b s_a) / sum of all m."""
    k = len(codes)
    mask = np.array([[a != b and compatible(int(codes[a]), int(codes[b])) for b in range(k)] for a in range(k)], float)
    m = masses.astype(float)
    s = states.astype(float)
    total = m.sum()
    gain = m[:, None] * (mask @ s)
    loss = (mask @ m)[:, None] * s
    return s + (gain - loss) / total


def test_sparse_exchange_matches_equation_and_conserves_momentum():
    # tests/test_mechanics.py:80-105: one node, codes {0, 1, 2, 4, 7}
    codes = np.array([0, 1, 2, 4, 7], np.int64)
    masses = np.array([0.2, 0.5, 0.7, 0.3, 0.4], F32)
    states = np.random.default_rng(3).normal(size=(5, 3)).astype(F32)
    result = np.zeros((5, 3), F32)
    start = np.array([0, 5], np.int32)
    lib().orc_couple_fields(ptr(codes), ptr(masses), ptr(states), ptr(start), 1, ptr(result))
    np.testing.assert_allclose(result, exchange_fp64(codes, masses, states), atol=4e-7)
    np.testing.assert_allclose(result.sum(0), states.sum(0), atol=8e-7)


# -------------------------------------------------------------- blade query


def blade_polygon(half, bevel):
    """Cross-section of the knife in (x, z), counter-clockwise."""
    hx, hz = float(half[0]), float(half[2])
    if bevel == 0.0:
        return np.array([[hx, -hz], [hx, hz], [-hx, hz], [-hx, -hz]])
    return np.array([[0.0, -hz], [hx, -hz + bevel], [hx, hz], [-hx, hz], [-hx, -hz + bevel]])


def polygon_distance(q, poly):
    """Signed distance of q to a convex polygon, the nearest boundary point and the outward normal there."""
    best, near, normal = np.inf, None, None
    inside = True
    for i in range(len(poly)):
        a, b = poly[i], poly[(i + 1) % len(poly)]
        edge = b - a
        out = np.array([edge[1], -edge[0]]) / np.hypot(*edge)
        if (q - a) @ out > 0.0:
            inside = False
        t = np.clip((q - a) @ edge / (edge @ edge), 0.0, 1.0)
        c = a + t * edge
        d = np.hypot(*(q - c))
        if d < best:
            best, near, normal = d, c, out
    return (-best if inside else best), near, normal


def blade_query_fp64(local, half, bevel):
    """Closest point, normal and signed distance to the bevelled knife (polygon x [-half_y, half_y])."""
    p = np.asarray(local, float)
    hy = float(half[1])
    d2, c2, n2 = polygon_distance(p[[0, 2]], blade_polygon(half, bevel))
    dy = abs(p[1]) - hy
    sy = 1.0 if p[1] >= 0.0 else -1.0
    if d2 <= 0.0 and dy <= 0.0:
        if dy > d2:
            return np.array([p[0], sy * hy, p[2]]), np.array([0.0, sy, 0.0]), dy
        return np.array([c2[0], p[1], c2[1]]), np.array([n2[0], 0.0, n2[1]]), d2
    xz = c2 if d2 > 0.0 else p[[0, 2]]
    closest = np.array([xz[0], np.clip(p[1], -hy, hy), xz[1]])
    delta = p - closest
    distance = np.linalg.norm(delta)
    return closest, delta / distance, distance


def oracle_blade_query(x, half, bevel):
    x = np.ascontiguousarray(x, F32)
    half = np.asarray(half, F32)
    closest, normal = np.zeros_like(x), np.zeros_like(x)
    distance = np.zeros(len(x), F32)
    lib().orc_blade_query(ptr(x), len(x), ptr(half), float(bevel), ptr(closest), ptr(normal), ptr(distance))
    return closest, normal, distance


@pytest.mark.parametrize("bevel", [0.0, 0.005])
def test_blade_distance_and_normal_against_fp64(bevel):
    # tests/test_mechanics.py:108-122
    rng = np.random.default_rng(2)
    x = rng.uniform([-0.003, -0.027, -0.025], [0.003, 0.027, 0.025], (400, 3)).astype(F32)
    half = np.array([0.0005, 0.025, 0.02], F32)
    closest, normal, distance = oracle_blade_query(x, half, bevel)
    ref = [blade_query_fp64(p.astype(float), half.astype(float), float(F32(bevel))) for p in x]
    np.testing.assert_allclose(closest, [r[0] for r in ref], atol=6e-9)
    np.testing.assert_allclose(normal, [r[1] for r in ref], atol=5e-4)
    np.testing.assert_allclose(distance, [r[2] for r in ref], atol=6e-9)


def test_beveled_blade_face_normal_remains_exact_near_contact():
    # tests/test_mechanics.py:151-180
    half = np.array([0.0005, 0.04, 0.02], F32)
    x = np.array(
        [[sign * (half[0] + gap), y, z]
         for sign in (-1, 1)
         for gap in (1e-8, 1e-7, 1e-6)
         for y in (-0.03, 0.01)
         for z in (-0.01476572, -0.005, 0.00126425, 0.019)],
        F32,
    )
    closest, normal, distance = oracle_blade_query(x, half, 0.005)
    expected_points = x.copy()
    expected_points[:, 0] = np.sign(x[:, 0]) * half[0]
    expected_normals = np.zeros_like(x)
    expected_normals[:, 0] = np.sign(x[:, 0])
    np.testing.assert_array_equal(closest, expected_points)
    np.testing.assert_allclose(normal, expected_normals, atol=1e-7)
    np.testing.assert_array_equal(distance, np.abs(x[:, 0]) - half[0])


# ----------------------------------------------------------------- friction


def friction_fp64(n, relative, jn, history, me, dt, mus, mud, gk, gc):
    """Stick/slip tangential impulse with an elastic history (spring gk me / dt^2, damping ratio gc)."""
    vt = relative - (relative @ n) * n
    ht = history - (history @ n) * n
    k = gk * me / dt**2
    damping = 2.0 * gc * np.sqrt(me * k)
    trial = (-k * ht - damping * vt) * dt
    if np.linalg.norm(trial) <= mus * jn:
        return trial, ht + dt * vt
    applied = trial * (mud * jn / np.linalg.norm(trial))
    return applied, -(applied / dt + damping * vt) / k


def test_friction_stick_and_slip_history():
    # tests/test_mechanics.py:125-148
    v = np.array([[0.001, 0, 0], [1.0, 0.1, 0.3], [0, 0, 0]], F32)
    h = np.array([[0, 0, 0], [0.0002, 0.0003, 0], [0, 0, 0.2]], F32)
    n = np.tile(np.array([0.0, 0.0, 1.0], F32), (3, 1))
    jn = np.full(3, 0.003, F32)
    j, hn = np.zeros((3, 3), F32), np.zeros((3, 3), F32)
    lib().orc_friction(ptr(n), ptr(v), ptr(jn), ptr(h), 3, 0.02, 0.001, 0.3, 0.2, 0.05, 0.1, ptr(j), ptr(hn))
    expected = [friction_fp64(np.array([0.0, 0.0, 1.0]), v[i].astype(float), float(F32(0.003)), h[i].astype(float),
                              float(F32(0.02)), float(F32(0.001)), float(F32(0.3)), float(F32(0.2)),
                              float(F32(0.05)), float(F32(0.1))) for i in range(3)]
    np.testing.assert_allclose(j, [e[0] for e in expected], atol=1e-9)
    np.testing.assert_allclose(hn, [e[1] for e in expected], atol=1e-9)
    assert np.linalg.norm(j[1].astype(float)) == pytest.approx(0.2 * 0.003, rel=2e-6)


# --------------------------------------------------------------- plasticity


def corotated_fp64(F, mu, lam):
    """P = 2 mu (F - R) + lam (J - 1) J F^-T with R = U V^T from the SVD (Fp = I)."""
    U, _, Vt = np.linalg.svd(F)
    R = U @ Vt
    J = np.linalg.det(F)
    return 2.0 * mu * (F - R) + (lam * (J - 1.0) * J)[:, None, None] * np.linalg.inv(F).transpose(0, 2, 1)


def material_step_fp64(x, v, F, codes, nodes, w, g, imp, mass, volume, mu, lam, dt, flip, node_count, viscosity):
    """One material step (solver.py:334-376, 431-535) in float64: fields are the
    distinct (node, code) keys of every particle's 8 stencil nodes."""
    n = len(x)
    keys = codes[:, None] * node_count + nodes
    unique, slot = np.unique(keys, return_inverse=True)
    slot = slot.reshape(n, 8)
    S = len(unique)
    node_of, code_of = unique % node_count, unique // node_count
    same = node_of[:, None] == node_of[None, :]
    compat = np.array([[compatible(int(a), int(b)) for b in code_of] for a in code_of]) & same
    np.fill_diagonal(compat, False)
    P = corotated_fp64(F, mu, lam)
    m = np.zeros(S)
    mom = np.zeros((S, 3))
    J = np.zeros((S, 3))
    np.add.at(m, slot, mass * w)
    np.add.at(mom, slot, mass * w[..., None] * v[:, None, :])
    np.add.at(J, slot, w[..., None] * imp[:, None, :] - dt * volume * np.einsum("pij,paj->pai", P, g))
    node_mass = np.zeros(node_count)
    np.add.at(node_mass, node_of, m)
    total = node_mass[node_of]

    def couple(state):  # Eq. 8 over the compatible fields of each node
        return state + (m[:, None] * (compat @ state) - (compat @ m)[:, None] * state) / total[:, None]

    pc = couple(mom)
    if viscosity:
        old_v = pc / m[:, None]
        rate = np.einsum("pai,paj->pij", old_v[slot], g)
        inv = np.linalg.inv(F)
        L = rate @ inv
        sigma = viscosity * np.linalg.det(F)[:, None, None] * (L + L.transpose(0, 2, 1)) @ inv.transpose(0, 2, 1)
        np.add.at(J, slot, -dt * volume * np.einsum("pij,paj->pai", sigma, g))
    old_v = pc / m[:, None]
    new_v = (pc + couple(J)) / m[:, None]
    pic = np.einsum("pa,pai->pi", w, new_v[slot])
    dv = np.einsum("pa,pai->pi", w, (new_v - old_v)[slot])
    v_new = (1.0 - flip) * pic + flip * (v + dv)
    x_new = x + dt * pic
    remapped = np.zeros((S, 3))
    np.add.at(remapped, slot, mass * w[..., None] * v_new[:, None, :])
    velocity = couple(remapped) / m[:, None]
    F_new = F + dt * np.einsum("pai,paj->pij", velocity[slot], g)
    return x_new, v_new, F_new


@pytest.mark.parametrize("viscosity", [0.0, 2.0])
def test_material_step_against_fp64_and_momentum(viscosity):
    # tests/test_mechanics.py:183-225: two incompatible pieces (codes 1 | 2 across x = 0)
    # under a stretch, random velocities and contact impulses; the reference's tolerances.
    cfg = replace(Config(), dynamic_viscosity=viscosity)
    c = OracleSolver(cfg)
    rng = np.random.default_rng(4)
    vel = rng.normal(scale=0.01, size=(c.n, 3)).astype(F32)
    F = np.tile(np.diag([1.01, 0.995, 1.0]), (c.n, 1, 1)).astype(F32)
    codes = np.where(c.reference[:, 0] < 0, 1, 2).astype(np.int64)
    impulse = rng.normal(scale=1e-8, size=(c.n, 3)).astype(F32)
    c.set("v", vel)
    c.set("F", F)
    c.refresh_stress()
    c.set("codes", codes)
    c.set("impulses", impulse)
    x = c.get("x").astype(float)
    reference, origin, cells = points(cfg.size, cfg.grid_spacing, cfg.shape, cfg.sampling_seed)
    nodes, w, g = stencil(reference, origin, cfg.grid_spacing, cells)
    expect = material_step_fp64(x, vel.astype(float), F.astype(float), codes, nodes.astype(np.int64),
                                w.astype(F32).astype(float), g.astype(F32).astype(float), impulse.astype(float),
                                c.mass, c.volume, c.mu, c.lam, cfg.dt, cfg.flip_fraction, c.node_count, viscosity)
    before = c.mass * vel.astype(float).sum(0)
    c.material_step()
    np.testing.assert_allclose(c.get("x"), expect[0], atol=1e-8)
    np.testing.assert_allclose(c.get("v"), expect[1], atol=2e-6)
    np.testing.assert_allclose(c.get("F"), expect[2], atol=2e-6)
    np.testing.assert_allclose(c.mass * c.get("v").astype(float).sum(0), before + impulse.astype(float).sum(0),
                               atol=2e-9)


def test_cut_labels_persist_through_withdrawal_and_a_new_cut():
    # tests/test_mechanics.py:228-300: side labels of digit 3^0 under the knife; a withdrawn
    # knife changes nothing; a second cut with digit 3^1 keeps the first digit of every code.
    c = OracleSolver(Config())
    c.set("tool_pos", [[0.0, 0.0, 0.03]])
    c.assign_sides(0, True)
    first = c.get("codes").copy()
    assert set(np.unique(first)) == {0, 1, 2}
    c.set("tool_pos", [[0.02, 0.0, 0.1]])
    c.assign_sides(0, True)
    np.testing.assert_array_equal(c.get("codes"), first)
    c.set("tool_pos", [[0.012, 0.0, 0.03]])
    c.assign_sides(1, True)
    np.testing.assert_array_equal(c.get("codes") % 3, first)
    assert c.get("codes").max() > 2


def test_cached_topology_rebuilds_on_new_labels_and_equals_uncached():
    # tests/test_topology_cache.py:6-20; the oracle is deterministic, so the two agree exactly.
    plain, cached = OracleSolver(Config()), OracleSolver(replace(Config(), cache_topology=True))
    for c in (plain, cached):
        c.set("tool_pos", [[0.0, 0.0, 0.047]])
    for count, cut, on in [(8, 0, True), (8, 0, True), (8, 0, False), (7, 1, True), (8, 1, True)]:
        targets = np.tile([0.0, 0.0, 0.019], (count, 1))
        plain.advance(targets, cutting=on, cut_index=cut)
        cached.advance(targets, cutting=on, cut_index=cut)
        for name in ("codes", "x", "v", "F"):
            np.testing.assert_array_equal(plain.get(name), cached.get(name), err_msg=name)
    assert np.count_nonzero(cached.get("codes")) > 0


def test_unmodified_material_keeps_cached_slots():
    # tests/test_topology_cache.py:23-31
    from blademaster_gb300 import _native

    c = OracleSolver(replace(Config(), cache_topology=True))
    c.advance(np.tile([0.0, 0.0, 1.0], (2, 1)), cutting=False)
    slots, keys = c.get("slots").copy(), c.get("keys").copy()
    c.advance(np.tile([0.0, 0.0, 1.0], (2, 1)), cutting=False)
    np.testing.assert_array_equal(c.get("slots"), slots)
    np.testing.assert_array_equal(c.get("keys"), keys)
    assert c.get("flags")[_native.FLAG["TOPOLOGY_DIRTY"]] == 0


def test_codes_at_full_capacity_register_without_overflow():
    # tests/test_stress_replays.py:44-58: 225 nodes keep 34 ternary digits; the highest
    # code 3^34 - 1 at the last node gives the highest key 225 * 3^34 - 1 < 2^63.
    c = OracleSolver(Config())
    assert c.node_count == 225
    rng = np.random.default_rng(7)
    codes = rng.integers(0, 3**34, c.n, dtype=np.int64)
    nodes = c.node_numpy.astype(np.int64)
    last = int(np.argmax(nodes.max(1)))
    codes[last] = 3**34 - 1
    c.set("codes", codes)
    c.register()
    keys = c.get("keys")
    expected = np.unique(codes[:, None] * 225 + nodes)
    np.testing.assert_array_equal(np.sort(keys[keys >= 0]), expected)
    assert keys.max() == 225 * 3**34 - 1
    np.testing.assert_array_equal(keys[c.get("slots")][c.rank], codes[:, None] * 225 + nodes)
    assert not c.get("errors").any()


def test_von_mises_projection_preserves_total_and_volume():
    # tests/test_mechanics.py:303-314
    s = OracleSolver(Config())
    total = np.tile(np.diag([1.3, 1 / 1.3, 1.0]), (s.n, 1, 1)).astype(F32)
    s.set("F", total)
    s.L.orc_plastic_project(ctypes.byref(s.params), ctypes.byref(s.S), 100.0)
    fp = s.get("Fp").astype(float)
    np.testing.assert_array_equal(s.get("F"), total)
    np.testing.assert_allclose(np.linalg.det(fp), 1, atol=3e-6)
    fe = total.astype(float) @ np.linalg.inv(fp)
    logs = np.log(np.linalg.svd(fe, compute_uv=False))
    dev = logs - logs.mean(1)[:, None]
    np.testing.assert_allclose(np.linalg.norm(dev, axis=1), 100 / (2 * s.mu) * np.sqrt(2 / 3), atol=2e-6)
    assert not s.get("errors").any()


# ---------------------------------------------------------------------- G2P


def oracle_g2p(x, v, slots, weights, old, new, dt, flip):
    x, v = np.array(x, F32, order="C"), np.array(v, F32, order="C")  # copies: the oracle updates them in place
    # keep every input alive across the call (ptr holds only the address)
    slots, weights = np.ascontiguousarray(slots, np.int32), np.ascontiguousarray(weights, F32)
    old, new = np.ascontiguousarray(old, F32), np.ascontiguousarray(new, F32)
    lib().orc_g2p(ptr(x), ptr(v), ptr(slots), ptr(weights), ptr(old), ptr(new), len(x), dt, flip)
    return x, v


@pytest.mark.parametrize("flip", [0.0, 0.95, 1.0])
def test_grid_velocity_advects_positions_even_with_particle_residual(flip):
    # tests/test_particle_transport.py:9-25
    initial = np.array([[0.0, 0.0, 0.0], [0.003, 0.0, 0.0]], F32)
    velocity = np.array([[10.0, 0.0, 0.0], [-10.0, 0.0, 0.0]], F32)
    grid = np.zeros((8, 3), F32)
    x, v = oracle_g2p(initial, velocity, np.tile(np.arange(8), (2, 1)), np.full((2, 8), 1 / 8), grid, grid, 0.001, flip)
    np.testing.assert_array_equal(x, initial)
    np.testing.assert_allclose(v, flip * velocity, atol=1e-6)


@pytest.mark.parametrize("flip", [0.0, 0.95, 1.0])
def test_uniform_grid_acceleration_and_particle_momentum_are_distinct(flip):
    # tests/test_particle_transport.py:28-38
    old = np.tile([1.0, 2.0, 3.0], (8, 1))
    new = np.tile([2.0, 4.0, 6.0], (8, 1))
    x, v = oracle_g2p(np.zeros((1, 3)), [[7.0, 2.0, -1.0]], np.arange(8).reshape(1, 8), np.full((1, 8), 1 / 8),
                      old, new, 0.001, flip)
    np.testing.assert_allclose(x, [[0.002, 0.004, 0.006]], rtol=1e-6)
    np.testing.assert_allclose(v, [[2.0 + 6 * flip, 4.0, 6.0 - 4 * flip]], rtol=1e-6)


# ---------------------------------------------------------- cut resistance


@pytest.mark.parametrize("angle", [0, 35])
def test_completed_cut_resistance_stays_released_during_hold_and_reversal(angle):
    # tests/test_cut_resistance.py:45-67
    from scipy.spatial.transform import Rotation

    rotation = Rotation.from_euler("y", angle, degrees=True)
    edge = np.array([0.0, 0.0, 0.02]) + rotation.apply([0.0, 0.0, -0.02])
    c32 = lambda a: np.ascontiguousarray(a, F32)  # noqa: E731  (scipy returns Fortran-ordered arrays)
    x = c32(edge + rotation.apply([[0, 0, -0.001]] * 5 + [[0, 0, 0.001]]))
    tool_velocity = c32(rotation.apply([[0, 0, -speed] for speed in [0.01, 0, -0.01, -0.01, 0.01, 0]]))
    q = c32(rotation.as_quat())
    qd = q.astype(float)
    j_local = np.array([0.002, 0.001, -0.004])
    # wp.quat_rotate in float32, as the reference's probe computes it
    j = c32(np.tile(Rotation.from_quat(qd).apply(j_local).astype(F32), (6, 1)))
    v = np.zeros((6, 3), F32)
    damage = np.array([1, 1, 1, 0.5, 0.5, 1], F32)
    work = np.zeros(2, np.uint64)
    result = np.zeros((6, 3), F32)
    origin, angular, half = np.array([0.0, 0.0, 0.02], F32), np.zeros(3, F32), np.array([0.0005, 0.025, 0.02], F32)
    lib().orc_resist_cut(ptr(j), ptr(x), ptr(v), ptr(origin), ptr(tool_velocity), ptr(q), ptr(angular), ptr(half),
                         0.0015, 0.006, ptr(damage), 0.001, 1, ptr(work), ptr(result), 6)
    expected = rotation.apply([[0.002, 0.001, 0]] * 3 + [[0.002, 0.001, -0.004]] * 3)
    np.testing.assert_allclose(result, expected, atol=2e-9)
    np.testing.assert_allclose(damage, [1, 1, 1, 0.5, 0.54, 1], atol=1e-7)
    assert fx_to_float(work[0], work[1]) == pytest.approx(0.004 * 0.01, rel=1e-6)


# ------------------------------------------------------ rigid / coupling


def test_rigid_reaction_is_equal_opposite_with_rotated_blade():
    # tests/test_mechanics.py:423-437
    cfg = replace(Config(), free_blade=True)
    s = OracleSolver(cfg)
    theta = 0.3
    s.set("tool_rot", [[0, np.sin(theta / 2), 0, np.cos(theta / 2)]])
    s.set("tool_pos", [[0.0, 0.0, 0.02]])
    s.rigid_contacts(cut_bits=0)
    gravity = np.array([0.0, 0.0, -9.81 * float(F32(s.mass)) * float(F32(cfg.dt))]) * s.n
    material = s.get("impulses").astype(float).sum(0)
    np.testing.assert_allclose(material + s.get("reaction")[0] - s.get("board")[0] - gravity, 0, atol=3e-9)
    assert np.linalg.norm(s.get("reaction")) > 0


def test_articulated_effective_mass_in_single_contact():
    # tests/test_coupling.py:99-122
    s = OracleSolver(replace(Config(), external_tool=True))
    cfg = s.config
    s.set("tool_pos", [[0, 0, 0.15]])
    x = s.get("x").copy()
    x[0] = [cfg.blade_half_size[0] + s.radius / 2, 0.01, 0.15]
    s.set("x", x)
    mobility = np.diag([1000, 2000, 3000, 4000, 5000, 6000.0])

    def impulse(a):
        s.set("mobility", a.astype(F32))
        s.arrays["acc"][:] = 0
        s.arrays["histories"][:] = 0
        s.rigid_contacts(cut_bits=0)
        return s.get("reaction")[0, 0]

    prescribed = impulse(np.zeros((6, 6)))
    articulated = impulse(mobility)
    direction = np.array([1, 0, 0, 0, 0, -0.01])
    expected_ratio = 1 / (1 + s.mass * (direction @ mobility @ direction))
    assert prescribed < 0
    assert articulated / prescribed == pytest.approx(expected_ratio, rel=2.0e-6)


def external_setup():
    """tests/test_coupling.py:10-23: specimen lifted off the board, a moving tilted knife."""
    s = OracleSolver(replace(Config(), external_tool=True))
    x = s.get("x").copy()
    x[:, 2] += 0.1
    s.set("x", x)
    angle = 0.15
    state = ToolState([0.001, 0.0, 0.132], [0.0, np.sin(angle / 2), 0.0, np.cos(angle / 2)], [0.01, 0.0, -0.02],
                      [0.0, 0.1, 0.0]).checked()
    packed = np.concatenate([state.position, state.orientation_xyzw, state.linear_velocity, state.angular_velocity,
                             state.mobility.ravel()]).astype(F32)
    return s, state, packed


def test_tool_is_frozen_and_impulse_is_equal_opposite():
    # tests/test_coupling.py:26-42
    s, state, packed = external_setup()
    steps = 8
    duration = steps * s.config.dt
    before = s.get("v").astype(float).sum(0) * float(F32(s.mass))
    impulse, _, errors = s.external_interval(packed, steps, cutting=False)
    after = s.get("v").astype(float).sum(0) * float(F32(s.mass))
    gravity = np.array([0.0, 0.0, -9.81]) * float(F32(s.mass)) * s.n * float(F32(s.config.dt)) * steps
    np.testing.assert_allclose(after - before + impulse, gravity, atol=3.0e-9)
    for name, value in [("tool_pos", state.position), ("tool_rot", state.orientation_xyzw),
                        ("tool_vel", state.linear_velocity), ("tool_omega", state.angular_velocity)]:
        np.testing.assert_allclose(s.get(name)[0], value, atol=2.0e-8)
    assert np.linalg.norm(impulse / duration) > 0.01
    assert not errors.any()


def test_interval_accumulation_matches_single_substeps():
    # tests/test_coupling.py:45-59
    a, _, packed = external_setup()
    b, _, _ = external_setup()
    impulse, angular, _ = a.external_interval(packed, 9)
    pieces = [b.external_interval(packed, 1) for _ in range(9)]
    np.testing.assert_allclose(impulse, sum(p[0] for p in pieces), atol=2.0e-9)
    np.testing.assert_allclose(angular, sum(p[1] for p in pieces), atol=2.0e-10)
    np.testing.assert_allclose(a.get("x"), b.get("x"), atol=1.0e-7)
    np.testing.assert_array_equal(a.get("codes"), b.get("codes"))


def far_clusters(n, seed=45):
    """tests/test_hash_grid.py:15-28 restated for the particle pair search: three clusters 2-5 m outside
    the block, where hashed cells wrap (bucket wrap must not clip space).  Neighbouring particles carry
    the incompatible codes 1 and 2 or reference positions 20 mm apart, so every pair within reach is a
    contact."""
    rng = np.random.default_rng(seed)
    x = np.vstack([rng.normal(c, 0.004, (k, 3)) for c, k in
                   zip([(2, 3, 4), (-2, 0, -3), (0.1, 0, 0.2)], [n // 3, n // 3, n - 2 * (n // 3)])]).astype(np.float32)
    ref = np.column_stack([np.arange(n) * 0.02, np.zeros(n), np.zeros(n)]).astype(np.float32)
    return x, ref, np.where(np.arange(n) % 2 == 0, 1, 2).astype(np.int64)


def test_pair_search_far_outside_the_block_finds_every_pair():
    # the pair list against brute force: every pair closer than the reach (2 radius at rest) by more
    # than 1 um is found, and every found pair is within the reach plus 1 um
    o = OracleSolver(Config())
    x, ref, codes = far_clusters(o.n)
    o.set("x", x), o.set("ref", ref), o.set("codes", codes)
    o.particle_contacts()
    new = (o.step_count + 1) % 2
    keys = o.arrays["pair_keys"][new]
    found = keys[keys >= 0]
    assert len(found) == o.arrays["pair_count"][new] > 10000
    xs = o.arrays["x"].astype(np.float64)  # device order, as the keys
    d = np.linalg.norm(xs[:, None] - xs[None], axis=2)
    reach = 2.0 * float(np.float32(o.params.radius))
    inside = np.triu(d < reach - 1e-6, 1)
    lo, hi = np.nonzero(inside)
    assert set((lo * o.n + hi).tolist()) <= set(found.tolist())
    assert np.all(d[found // o.n, found % o.n] < reach + 1e-6)
    assert not o.arrays["errors"].any()


@pytest.mark.parametrize("split", [False, True])
def test_pair_recontact_reference_exclusion_and_equal_opposite_impulse(split):
    # tests/test_mechanics.py:340-420: two particles 2 mm apart closing at 2 x (0.01, 0.003, 0) m/s, their
    # reference positions where they are.  Split (codes 1 and 2) they contact with equal and opposite
    # impulses, normal plus stick/slip friction, as a float64 statement of pair_at (contact.py:583-640)
    # gives them; uncut (codes 0 and 0) the reference exclusion leaves them alone.  The rest of the block
    # is parked 20 mm apart, out of reach.
    o = OracleSolver(Config(grid_spacing=0.006, dt=0.00025))
    n = o.n
    x = np.column_stack([10 + 0.02 * np.arange(n), np.zeros(n), np.full(n, 10.0)])
    x[:2] = [[0.0, 0.0, 0.05], [0.002, 0.0, 0.05]]
    v = np.zeros((n, 3))
    v[:2] = [[0.01, 0.003, 0.0], [-0.01, -0.003, 0.0]]
    codes = np.zeros(n, np.int64)
    codes[:2] = [1, 2] if split else [0, 0]
    x, v = x.astype(F32), v.astype(F32)
    o.set("x", x), o.set("ref", x), o.set("v", v), o.set("codes", codes), o.set("impulses", np.zeros((n, 3), F32))
    o.arrays["speed"][:] = np.linalg.norm(v, axis=1).max()
    o.particle_contacts()
    out = o.get("impulses")[:2].astype(float)

    p = o.params
    r, dt, me = float(F32(p.radius)), float(F32(p.dt)), float(F32(p.mass)) / 2.0
    delta = x[0].astype(float) - x[1].astype(float)
    dist = np.linalg.norm(delta)
    normal, relative = delta / dist, v[0].astype(float) - v[1].astype(float)
    predicted = 2.0 * r - dist - dt * min(relative @ normal, 0.0)
    jn = float(F32(p.normal_scale)) * me / dt * predicted
    jt, _ = friction_fp64(normal, relative, jn, np.zeros(3), me, dt, float(F32(p.friction_static)),
                          float(F32(p.friction_dynamic)), float(F32(p.tangent_stiffness)), float(F32(p.tangent_damping)))
    expected = normal * jn + jt if split else np.zeros(3)
    np.testing.assert_allclose(out, [expected, -expected], atol=1e-10)
    np.testing.assert_allclose(out.sum(0), 0, atol=1e-12)
    assert bool(np.any(out)) == split
    assert o.arrays["pair_count"][(o.step_count + 1) % 2] == int(split)
    assert not o.arrays["errors"].any()
