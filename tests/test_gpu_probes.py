"""The CUDA probe entry points (the reference's single-function test kernels)
against the oracle on the known-answer inputs, bit for bit.

These call the device functions that the substep kernels use (blade query,
friction, Eq. 8 exchange, G2P, cutting resistance, von Mises projection)
through the C-ABI, one thread per case, and compare with the same oracle
functions that tests/test_oracle_known_answers.py pins to the reference's
expected values.
"""

import ctypes

import numpy as np
import pytest

from blademaster_gb300 import _native
from blademaster_gb300.solver import Config
from oracle.oracle import OracleSolver, lib as oracle_lib, ptr

pytestmark = pytest.mark.gpu

F32 = np.float32


def dev(a):
    import torch

    return torch.as_tensor(np.ascontiguousarray(a), device="cuda:0")


def addr(t):
    return ctypes.c_void_p(t.data_ptr())


def run(fn, *args):
    import torch

    _native.check(getattr(_native.lib(), fn)(*args, None))
    torch.cuda.synchronize()


@pytest.mark.parametrize("bevel", [0.0, 0.005])
def test_blade_query_matches_oracle(bevel):
    rng = np.random.default_rng(2)
    x = rng.uniform([-0.003, -0.027, -0.025], [0.003, 0.027, 0.025], (400, 3)).astype(F32)
    # plus the near-face points of the exact-normal test
    face = np.array([[s * (0.0005 + g), y, z] for s in (-1, 1) for g in (1e-8, 1e-7, 1e-6) for y in (-0.03, 0.01)
                     for z in (-0.01476572, -0.005, 0.00126425, 0.019)], F32)
    x = np.concatenate([x, face])
    half = np.array([0.0005, 0.025, 0.02], F32)
    gx, gc, gn, gd = dev(x), dev(np.zeros_like(x)), dev(np.zeros_like(x)), dev(np.zeros(len(x), F32))
    run("bm_blade_query", addr(gx), len(x), ptr(half), bevel, addr(gc), addr(gn), addr(gd))
    cc, cn, cd = np.zeros_like(x), np.zeros_like(x), np.zeros(len(x), F32)
    oracle_lib().orc_blade_query(ptr(x), len(x), ptr(half), bevel, ptr(cc), ptr(cn), ptr(cd))
    np.testing.assert_array_equal(gc.cpu().numpy(), cc)
    np.testing.assert_array_equal(gn.cpu().numpy(), cn)
    np.testing.assert_array_equal(gd.cpu().numpy(), cd)


def test_friction_matches_oracle():
    rng = np.random.default_rng(4)
    m = 64
    v = np.concatenate([np.array([[0.001, 0, 0], [1.0, 0.1, 0.3], [0, 0, 0]], F32), rng.normal(0, 0.5, (m, 3)).astype(F32)])
    h = np.concatenate([np.array([[0, 0, 0], [0.0002, 0.0003, 0], [0, 0, 0.2]], F32),
                        rng.normal(0, 1e-3, (m, 3)).astype(F32)])
    n = rng.normal(size=(len(v), 3))
    n[:3] = [0, 0, 1]
    n = (n / np.linalg.norm(n, axis=1)[:, None]).astype(F32)
    jn = np.full(len(v), 0.003, F32)
    args = (0.02, 0.001, 0.3, 0.2, 0.05, 0.1)
    g = [dev(a) for a in (n, v, jn, h)]
    gj, gh = dev(np.zeros_like(v)), dev(np.zeros_like(v))
    run("bm_friction", *[addr(t) for t in g], len(v), *args, addr(gj), addr(gh))
    cj, ch = np.zeros_like(v), np.zeros_like(v)
    oracle_lib().orc_friction(ptr(n), ptr(v), ptr(jn), ptr(h), len(v), *args, ptr(cj), ptr(ch))
    np.testing.assert_array_equal(gj.cpu().numpy(), cj)
    np.testing.assert_array_equal(gh.cpu().numpy(), ch)


def test_exchange_matches_oracle():
    # the {0, 1, 2, 4, 7} node plus random multi-field nodes
    rng = np.random.default_rng(3)
    codes = [np.array([0, 1, 2, 4, 7], np.int64)] + [rng.integers(0, 81, rng.integers(1, 9)) for _ in range(200)]
    start = np.cumsum([0] + [len(c) for c in codes]).astype(np.int32)
    codes = np.concatenate(codes).astype(np.int64)
    mass = rng.uniform(0.05, 1.0, len(codes)).astype(F32)
    state = rng.normal(size=(len(codes), 3)).astype(F32)
    g = [dev(a) for a in (codes, mass, state, start)]  # kept alive across the launch
    gr = dev(np.zeros_like(state))
    run("bm_couple_fields", *[addr(t) for t in g], len(start) - 1, addr(gr))
    cr = np.zeros_like(state)
    oracle_lib().orc_couple_fields(ptr(codes), ptr(mass), ptr(state), ptr(start), len(start) - 1, ptr(cr))
    np.testing.assert_array_equal(gr.cpu().numpy(), cr)


@pytest.mark.parametrize("flip", [0.0, 0.95, 1.0])
def test_g2p_matches_oracle(flip):
    rng = np.random.default_rng(5)
    n, slots_n = 300, 64
    x = rng.normal(0, 0.01, (n, 3)).astype(F32)
    v = rng.normal(0, 1.0, (n, 3)).astype(F32)
    slots = rng.integers(0, slots_n, (n, 8)).astype(np.int32)
    w = rng.dirichlet(np.ones(8), n).astype(F32)
    old, new = rng.normal(size=(slots_n, 3)).astype(F32), rng.normal(size=(slots_n, 3)).astype(F32)
    gx, gv = dev(x), dev(v)
    gs, gw, go, gn = dev(slots), dev(w), dev(old), dev(new)
    run("bm_g2p_probe", addr(gx), addr(gv), addr(gs), addr(gw), addr(go), addr(gn), n, 0.001, flip)
    cx, cv = x.copy(), v.copy()
    oracle_lib().orc_g2p(ptr(cx), ptr(cv), ptr(slots), ptr(w), ptr(old), ptr(new), n, 0.001, flip)
    np.testing.assert_array_equal(gx.cpu().numpy(), cx)
    np.testing.assert_array_equal(gv.cpu().numpy(), cv)


@pytest.mark.parametrize("angle", [0, 35])
def test_resist_cut_matches_oracle(angle):
    from scipy.spatial.transform import Rotation

    rotation = Rotation.from_euler("y", angle, degrees=True)
    c32 = lambda a: np.ascontiguousarray(a, F32)  # noqa: E731
    edge = np.array([0.0, 0.0, 0.02]) + rotation.apply([0.0, 0.0, -0.02])
    x = c32(edge + rotation.apply([[0, 0, -0.001]] * 5 + [[0, 0, 0.001]]))
    tool_velocity = c32(rotation.apply([[0, 0, -s] for s in [0.01, 0, -0.01, -0.01, 0.01, 0]]))
    q = c32(rotation.as_quat())
    j = c32(np.tile(rotation.apply([0.002, 0.001, -0.004]), (6, 1)))
    v = np.zeros((6, 3), F32)
    damage = np.array([1, 1, 1, 0.5, 0.5, 1], F32)
    origin, angular, half = np.array([0.0, 0.0, 0.02], F32), np.zeros(3, F32), np.array([0.0005, 0.025, 0.02], F32)
    for bits in (1, 3):
        g = [dev(a) for a in (j, x, v, origin, tool_velocity, q, angular)]
        gdamage, gwork, gres = dev(damage), dev(np.zeros(2, np.int64)), dev(np.zeros((6, 3), F32))
        run("bm_resist_cut_probe", *[addr(t) for t in g], ptr(half), 0.0015, 0.006, addr(gdamage), 0.001, bits,
            addr(gwork), addr(gres), 6)
        cdamage, cwork, cres = damage.copy(), np.zeros(2, np.uint64), np.zeros((6, 3), F32)
        oracle_lib().orc_resist_cut(ptr(j), ptr(x), ptr(v), ptr(origin), ptr(tool_velocity), ptr(q), ptr(angular),
                                    ptr(half), 0.0015, 0.006, ptr(cdamage), 0.001, bits, ptr(cwork), ptr(cres), 6)
        np.testing.assert_array_equal(gres.cpu().numpy(), cres)
        np.testing.assert_array_equal(gdamage.cpu().numpy(), cdamage)
        np.testing.assert_array_equal(gwork.cpu().numpy().view(np.uint64), cwork)


def test_plastic_projection_matches_oracle():
    c = OracleSolver(Config())
    rng = np.random.default_rng(6)
    total = (np.eye(3) + rng.normal(0, 0.05, (c.n, 3, 3))).astype(F32)
    total[0] = np.diag([1.3, 1 / 1.3, 1.0])
    c.set("F", total)
    c.L.orc_plastic_project(ctypes.byref(c.params), ctypes.byref(c.S), 100.0)
    # the probe takes structure-of-arrays [9][n] in the oracle's particle order
    F = dev(c.arrays["F"].T.copy())
    Fp = dev(np.tile(np.eye(3, dtype=F32).reshape(9, 1), (1, c.n)))
    errors = dev(np.zeros(3, np.int32))
    run("bm_plastic_project", addr(F), addr(Fp), c.n, float(F32(c.mu)), 100.0, addr(errors))
    np.testing.assert_array_equal(Fp.cpu().numpy().T, c.arrays["Fp"])
    np.testing.assert_array_equal(F.cpu().numpy().T, c.arrays["F"])
    assert errors.cpu().numpy().tolist() == c.get("errors").tolist()
