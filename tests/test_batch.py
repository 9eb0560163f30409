"""Batched sweeps (SolverBatch): one graph launch per interval for many
instances must compute exactly what each instance's own ExternalToolPort
computes, for any lane count."""

import numpy as np
import pytest

from blademaster_gb300.sweep import instances

pytestmark = pytest.mark.gpu


def test_batched_intervals_equal_per_instance_ports():
    from blademaster_gb300.batch import SolverBatch
    from blademaster_gb300.coupling import ExternalToolPort
    from blademaster_gb300.solver import Solver

    sweep = instances(5, seed=3, spacings=(0.006, 0.0045))
    batched = [Solver(i.config) for i in sweep]
    single = [Solver(i.config) for i in sweep]
    ports = [ExternalToolPort(s) for s in single]
    batch = SolverBatch(batched, lanes=2)
    for k in range(6):
        states = [i.state(k, start_gap=-0.0005) for i in sweep]
        reactions = batch.advance(states, 0.001, cutting=True, lanes=2 if k % 2 else 5)
        for j, (port, state) in enumerate(zip(ports, states)):
            r = port.advance(state, 0.001, cutting=True)
            np.testing.assert_array_equal(reactions[j].impulse_ns, r.impulse_ns, err_msg=f"instance {j}, interval {k}")
            np.testing.assert_array_equal(reactions[j].angular_impulse_nms, r.angular_impulse_nms)
    for b, s in zip(batched, single):
        for name in ("x", "v", "F", "codes", "damage"):
            np.testing.assert_array_equal(getattr(b, name).numpy(), getattr(s, name).numpy(), err_msg=name)
    assert any(np.count_nonzero(r.impulse_ns) for r in reactions)
