"""Maxwell (generalised standard linear solid) branch, material.py:478-618.

CPU: the reference's held-deformation relaxation tests (tests/test_maxwell.py
:85-118) on the oracle against the float64 closed form, including a slow
relaxation over 20000 steps, and a disabled branch (tau or fraction zero)
reproducing the elastic run exactly (:21-32).  GPU: cut substeps
with the Maxwell branch (and with plasticity on top) bit-exact against the
oracle, including the float64 viscous state.
"""

import ctypes
from dataclasses import replace

import numpy as np
import pytest

from blademaster_gb300.solver import Config
from oracle.oracle import OracleSolver


def rotation(axis, angle):
    axis = np.asarray(axis, float) / np.linalg.norm(axis)
    k = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + np.sin(angle) * k + (1 - np.cos(angle)) * k @ k


# finite stretch with shear and 1 % volume change, rotated off the axes (tests/test_maxwell.py:85-86)
HELD_F = rotation([1, 2, 3], 0.4) @ np.diag([1.08, 0.95, 0.985]) @ rotation([0, 1, 1], -0.3)


def reference_stress(F, mu, lam, mu_maxwell, factor):
    """Float64 first Piola stress with the Maxwell deviatoric Hencky strain scaled by factor."""
    u, sigma, vt = np.linalg.svd(F)
    R, J = u @ vt, np.prod(sigma)
    mu_eq, lam_eq = mu - mu_maxwell, lam + 2 / 3 * mu_maxwell
    inv_t = np.linalg.inv(F).T
    equilibrium = 2 * mu_eq * (F - R) + lam_eq * (J - 1) * J * inv_t
    e = np.log(sigma)
    kirchhoff = u @ np.diag(2 * mu_maxwell * factor * (e - e.mean())) @ u.T
    return equilibrium + kirchhoff @ inv_t


@pytest.mark.parametrize("tau_steps", [0.01, 1.0, 40.0])
def test_held_deformation_relaxes_exactly(tau_steps):
    cfg = replace(Config(), maxwell_tau=tau_steps * Config().dt, maxwell_fraction=0.6)
    o = OracleSolver(cfg)
    o.set("F", np.tile(HELD_F, (o.n, 1, 1)).astype(np.float32))
    o.refresh_stress()
    mu_maxwell = float(np.float32(0.6 * o.mu))
    decay = np.exp(-1 / tau_steps)
    done = 0
    for n in (0, 1, 5, 40, 120):
        o.L.orc_maxwell_hold(ctypes.byref(o.params), ctypes.byref(o.S), n - done)
        done = n
        expected = reference_stress(HELD_F, o.mu, o.lam, mu_maxwell, decay**n)
        np.testing.assert_allclose(o.get("stress")[0], expected, atol=2e-4 * np.abs(expected).max(), err_msg=f"step {n}")
    assert not o.get("errors").any()
    np.testing.assert_array_equal(o.get("F"), np.tile(HELD_F, (o.n, 1, 1)).astype(np.float32))
    viscous = o.arrays["viscous"].reshape(-1, 3, 3)
    np.testing.assert_allclose(np.linalg.det(np.eye(3) + viscous), 1, atol=2e-6)


def held(cfg, F):
    o = OracleSolver(cfg)
    o.set("F", np.tile(F, (o.n, 1, 1)).astype(np.float32))
    o.refresh_stress()
    return o


def test_instantaneous_and_volumetric_response_match_elastic_model():
    # tests/test_maxwell.py:123-138
    base = Config()
    cfg = replace(base, maxwell_tau=10 * base.dt, maxwell_fraction=0.7)
    small = np.eye(3) + 1e-3 * np.array([[0.5, 0.8, 0.0], [0.1, -0.3, 0.2], [0.0, 0.4, 0.6]])
    elastic = held(base, small).get("stress")[0]
    viscoelastic = held(cfg, small).get("stress")[0]
    np.testing.assert_allclose(viscoelastic, elastic, atol=3e-3 * np.abs(elastic).max())
    # a pure volume change loads only the elastic bulk response and does not relax
    o = held(cfg, 0.98 * np.eye(3))
    first = o.get("stress")[0].copy()
    o.L.orc_maxwell_hold(ctypes.byref(o.params), ctypes.byref(o.S), 50)
    scale = np.abs(first).max()
    np.testing.assert_allclose(o.get("stress")[0], first, atol=1e-5 * scale)
    np.testing.assert_allclose(first, np.diag(np.diag(first)), atol=1e-5 * scale)


@pytest.mark.gpu
@pytest.mark.parametrize("yield_stress", [0.0, 3000.0])
def test_maxwell_cut_substeps_are_bitexact(yield_stress):
    from blademaster_gb300.solver import Solver

    cfg = replace(Config(), maxwell_tau=20 * Config().dt, maxwell_fraction=0.6, yield_stress=yield_stress)
    g, c = Solver(cfg), OracleSolver(cfg)
    g.tool_pos.assign([[0.0, 0.0, 0.047]])
    c.set("tool_pos", [[0.0, 0.0, 0.047]])
    for _ in range(40):
        g.step((0.0, 0.0, 0.02), cutting=True)
        c.step((0.0, 0.0, 0.02), cutting=True)
    for name in ("x", "v", "F", "Fp", "stress", "codes", "damage"):
        np.testing.assert_array_equal(getattr(g, name).numpy(), c.get(name), err_msg=name)
    np.testing.assert_array_equal(g.viscous.numpy(), c.arrays["viscous"][c.rank].reshape(-1, 3, 3))
    assert np.abs(g.viscous.numpy()).max() > 0


def run_short(cfg, steps=100):
    """tests/test_maxwell.py:13-18: 100 guided cut substeps."""
    o = OracleSolver(cfg)
    o.set("tool_pos", [[0.0, 0.0, 0.047]])
    for _ in range(steps):
        o.step((0.0, 0.0, 0.02), cutting=True)
    return o


@pytest.mark.parametrize("tau, fraction", [(0.0, 0.5), (0.1, 0.0)])
def test_disabled_branch_runs_the_elastic_kernels(tau, fraction):
    # tests/test_maxwell.py:21-32; the oracle is deterministic, so the runs agree exactly
    reference = run_short(Config())
    o = run_short(replace(Config(), maxwell_tau=tau, maxwell_fraction=fraction))
    assert not o.params.maxwell
    for name in ("x", "v", "F", "codes", "tool_pos"):
        np.testing.assert_array_equal(o.get(name), reference.get(name), err_msg=name)


def test_slow_relaxation_is_resolved():
    # tests/test_maxwell.py:108-118: tau = 3.5e5 steps (22 s at the banana's 62.5 us), 20000 held
    # steps; the float64 viscous state keeps the error below 1 % of the relaxation so far.  Held
    # particles are independent and alike, so a 64-particle block stands in for the default one.
    tau_steps, steps = 3.5e5, 20000
    cfg = replace(Config(), size=(0.015, 0.015, 0.015), maxwell_tau=tau_steps * Config().dt, maxwell_fraction=0.6)
    o = held(cfg, HELD_F)
    start = o.get("stress")[0].copy()
    o.L.orc_maxwell_hold(ctypes.byref(o.params), ctypes.byref(o.S), steps)
    mu_maxwell = float(np.float32(0.6 * o.mu))
    expected = reference_stress(HELD_F, o.mu, o.lam, mu_maxwell, np.exp(-steps / tau_steps))
    error = np.abs(o.get("stress")[0] - expected).max()
    assert error < 0.01 * np.abs(start - expected).max()
