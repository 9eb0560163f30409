"""The external-tool port's refusals and recorded poses on the CUDA solver.

The reference's own cases (tests/test_coupling.py:74-97, 187-204) with their
assertions: an externally owned tool refuses the solver's own stepping and
durations that are not a whole positive number of substeps; an inverted
particle makes the interval raise instead of returning a wrench; and the
recorded tool substeps follow the applied pose, in hold and predict modes,
eager and graph-replayed.
"""

from dataclasses import replace

import numpy as np
import pytest

from blademaster_gb300.coupling import ExternalToolPort, ToolState
from blademaster_gb300.solver import Config

pytestmark = pytest.mark.gpu


def setup():
    """test_coupling.py:10-23: the default block lifted off the board, a tilted, moving external knife."""
    from blademaster_gb300.solver import Solver

    s = Solver(replace(Config(), external_tool=True))
    x = s.x.numpy()
    x[:, 2] += 0.1
    s.x.assign(x)
    angle = 0.15
    state = ToolState([0.001, 0.0, 0.132], [0.0, np.sin(angle / 2), 0.0, np.cos(angle / 2)], [0.01, 0.0, -0.02],
                      [0.0, 0.1, 0.0])
    return s, ExternalToolPort(s), state


def test_external_api_rejects_wrong_ownership_and_time():
    # test_coupling.py:74-88
    s, port, state = setup()
    with pytest.raises(ValueError):
        s.step()
    with pytest.raises(ValueError):
        s.advance([[0.0, 0.0, 0.0]])
    for duration in [0.0, -1.0, np.nan, 1.5 * s.config.dt]:
        with pytest.raises(ValueError):
            port.advance(state, duration)
    assert s.step_count == 0
    with pytest.raises(ValueError):
        port.advance(ToolState([0, 0, 0], [0, 0, 0, 2], [0, 0, 0], [0, 0, 0]), s.config.dt)
    with pytest.raises(ValueError):
        replace(Config(), external_tool=True, pose_servo=True)


def test_invalid_material_interval_never_returns_a_wrench():
    # test_coupling.py:90-96
    s, port, state = setup()
    f = s.F.numpy()
    f[0, 0, 0] = -1.0
    s.F.assign(f)
    with pytest.raises(RuntimeError, match="Invalid material coupling interval"):
        port.advance(state, s.config.dt, graph=False)


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("mode", ["hold", "predict"])
def test_recorded_tool_substeps_follow_the_applied_pose(graph, mode):
    # test_coupling.py:187-204
    from blademaster_gb300.solver import Solver

    s = Solver(replace(Config(), external_tool=True, tool_substep=mode))
    port = ExternalToolPort(s, record_trajectory=True)
    state = ToolState([0, 0, 0.15], [0, 0, 0, 1], [0.01, 0, 0], [0, 0, 0.2])
    # twice the same length (a cached graph replays), then another length
    for steps in [4, 4, 2, 4]:
        port.advance(state, steps * s.config.dt, cutting=False, graph=graph)
        trace = port.trajectory
        samples = 2 if mode == "hold" else steps + 1
        assert trace.shape == (samples, 7)
        np.testing.assert_allclose(trace[0], [*state.position, *state.orientation_xyzw], atol=1e-8)
        np.testing.assert_allclose(port.trajectory_times[-1], steps * s.config.dt)
        t = port.trajectory_times if mode == "predict" else np.zeros(samples)
        np.testing.assert_allclose(trace[:, 0], 0.01 * t, atol=1e-8)
        np.testing.assert_allclose(trace[:, 5], np.sin(0.2 * t / 2), atol=1e-8)
        np.testing.assert_allclose(trace[-1, :3], s.tool_pos.numpy()[0], atol=1e-8)
