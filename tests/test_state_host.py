"""Solver.state(), the snapshot callers save (solver.py:1021-1051), on the host alone.

The real method runs on a stand-in that holds only the arrays it reads.  The
snapshot has the reference's keys (the Maxwell and several-knife extras only
when they apply, the viscous deformation as I + the stored offset, the time
as substeps x dt), and a run with device errors, non-finite values or
inverted material is refused with the reference's messages.  No GPU.
"""

import types

import numpy as np
import pytest

from blademaster_gb300.solver import Config, Solver

KEYS = {"position", "velocity", "deformation", "plastic_deformation", "sides", "damage", "blade_position",
        "blade_velocity", "blade_orientation", "blade_omega", "time"}


class Host:
    def __init__(self, value):
        self.value = np.asarray(value)

    def numpy(self):
        return self.value.copy()


class Snapshot:
    def __init__(self, config=Config(), maxwell=False, n=4):
        eye = np.tile(np.eye(3), (n, 1, 1))
        self.config, self.maxwell, self.step_count = config, maxwell, 7
        self.errors = Host(np.zeros(3, np.int32))
        self.x, self.v, self.F, self.Fp = Host(np.zeros((n, 3))), Host(np.zeros((n, 3))), Host(eye), Host(eye)
        self.codes, self.damage = Host(np.zeros(n, np.int64)), Host(np.zeros(n))
        K = config.tool_count
        self.tool_pos, self.tool_vel = Host(np.zeros((K, 3))), Host(np.zeros((K, 3)))
        self.tool_rot, self.tool_omega = Host(np.tile([0.0, 0, 0, 1], (K, 1))), Host(np.zeros((K, 3)))
        self.tool_damage = [Host(np.full(n, 0.1 * k)) for k in range(K)]
        self.viscous = Host(np.full((n, 3, 3), 0.01))
        self.state = types.MethodType(Solver.state, self)


def test_state_has_the_reference_keys():
    s = Snapshot()
    state = s.state()
    assert set(state) == KEYS
    assert state["time"] == 7 * s.config.dt


def test_state_adds_viscous_deformation_and_every_knifes_damage_when_they_apply():
    s = Snapshot(Config(free_blade=True, tool_count=3), maxwell=True)
    state = s.state()
    assert set(state) == KEYS | {"viscous_deformation", "tool_damage"}
    np.testing.assert_allclose(state["viscous_deformation"], np.broadcast_to(np.eye(3) + 0.01, (4, 3, 3)))
    np.testing.assert_allclose(state["tool_damage"][:, 0], [0.0, 0.1, 0.2])


def test_state_refuses_device_errors_nonfinite_values_and_inverted_material():
    s = Snapshot()
    s.errors = Host(np.array([0, 1, 0], np.int32))
    with pytest.raises(RuntimeError, match="GPU errors"):
        s.state()
    s = Snapshot()
    s.v.value[0, 0] = np.nan
    with pytest.raises(RuntimeError, match="Nonfinite"):
        s.state()
    s = Snapshot()
    s.F.value[0, 0, 0] = -1.0
    with pytest.raises(RuntimeError, match="Inverted"):
        s.state()
