"""Host side of the external-tool port (coupling.py:23-72), with the reference's
own cases (tests/test_coupling.py:62-88, 125-128): the reaction's moment shift
conserves power, and invalid tool states and configurations are refused with
the reference's exception types.  No GPU."""

from dataclasses import replace

import numpy as np
import pytest

from blademaster_gb300.coupling import Reaction, ToolState
from blademaster_gb300.solver import Config


def test_moment_shift_and_power_invariance():
    # test_coupling.py:62-71
    r = Reaction(0.02, np.array([0.1, 0.2, 0.3]), np.array([0.01, -0.02, 0.03]), np.array([1.0, 2.0, 3.0]))
    origin = np.array([-0.5, 0.3, 2.0])
    shifted = r.about(origin)
    velocity = np.array([0.2, -0.1, 0.7])
    omega = np.array([0.3, 0.5, -0.2])
    v_new = velocity + np.cross(omega, origin - r.origin_world_m)
    assert np.dot(r.force_n, velocity) + np.dot(r.torque_nm, omega) == pytest.approx(
        np.dot(shifted.force_n, v_new) + np.dot(shifted.torque_nm, omega))
    np.testing.assert_allclose(shifted.force_n, r.force_n)
    np.testing.assert_allclose(shifted.origin_world_m, origin)


def test_mobility_rejects_invalid_mass_response():
    # test_coupling.py:125-128
    for invalid in [np.eye(5), -np.eye(6), np.full((6, 6), np.nan), np.triu(np.ones((6, 6)))]:
        with pytest.raises(ValueError, match="Mobility"):
            ToolState([0, 0, 0], [0, 0, 0, 1], [0, 0, 0], [0, 0, 0], invalid).checked()


def test_tool_state_and_configuration_are_validated():
    # test_coupling.py:85-88
    with pytest.raises(ValueError):
        ToolState([0, 0, 0], [0, 0, 0, 2], [0, 0, 0], [0, 0, 0]).checked()
    with pytest.raises(ValueError):
        ToolState([0, 0, np.nan], [0, 0, 0, 1], [0, 0, 0], [0, 0, 0]).checked()
    with pytest.raises(ValueError):
        replace(Config(), external_tool=True, pose_servo=True)
    ok = ToolState([0, 0, 0.1], [0, 0, 0, 1], [0, 0, -0.02], [0, 0, 0]).checked()
    assert ok.mobility.shape == (6, 6) and not ok.mobility.any()


class NoDevice:
    """A solver stand-in for the port's host checks: reaching the cut bookkeeping means the checks let
    the call through to the device path."""

    def __init__(self, **config):
        self.config = replace(Config(), **config)

    def _set_cut(self, cut_index):
        raise AssertionError("the port went on to the device path")


def test_port_refuses_bad_durations_and_states_before_any_device_work():
    # tests/test_coupling.py:74-88 on the host: only an external-tool solver gets a port; durations that
    # are not a positive whole number of substeps (at most 4096) and invalid tool states are refused
    # before the interval touches the solver
    from blademaster_gb300.coupling import ExternalToolPort

    with pytest.raises(ValueError, match="external_tool"):
        ExternalToolPort(NoDevice())
    solver = NoDevice(external_tool=True)
    port, dt = ExternalToolPort(solver), solver.config.dt
    state = ToolState([0.001, 0.0, 0.132], [0, 0, 0, 1], [0.01, 0.0, -0.02], [0.0, 0.1, 0.0])
    for duration in [0.0, -1.0, np.nan, np.inf, 1.5 * dt, 4097 * dt]:
        with pytest.raises(ValueError):
            port.advance(state, duration)
    with pytest.raises(ValueError, match="quaternion"):
        port.advance(ToolState([0, 0, 0], [0, 0, 0, 2], [0, 0, 0], [0, 0, 0]), dt)
    with pytest.raises(AssertionError, match="device path"):
        port.advance(state, 4 * dt)  # a valid interval goes on
