"""Resuming a run: the device checkpoint and the reference's state() round trip.

* ``Solver.checkpoint()`` / ``restore()`` keep every array a substep reads
  (pair lists, friction-history tables, accumulators, counters), so the
  substeps after a restore repeat the ones after the checkpoint bit for bit,
  through replayed graphs whose captured addresses stay valid.
* The reference's own resume path is ``state()`` written back through the
  arrays' ``.assign()`` (solver.py:1021-1051).  State it does not hold (pair
  lists, friction histories between particles) starts empty, so a resumed
  run equals the uninterrupted one while no particle pairs are in contact:
  a knife pressing into the block without cutting, here.
"""

import numpy as np
import pytest

from blademaster_gb300.solver import Config, Solver

pytestmark = pytest.mark.gpu

EXACT = ("x", "v", "F", "Fp", "stress", "codes", "damage")


def snapshot(s):
    out = {name: getattr(s, name).numpy() for name in EXACT}
    out["tool"] = s._t["tool"].cpu().numpy()
    out["reaction"] = s.reaction.numpy()
    out["work"] = s.work.numpy()
    out["histories"] = s.histories.numpy()
    return out


def assert_equal(a, b):
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_restore_repeats_the_substeps_after_the_checkpoint():
    cfg = Config(free_blade=True, yield_stress=2000.0)
    s = Solver(cfg)
    s.tool_pos.assign([[0.0, 0.0, 0.047]])
    s.advance(np.zeros((25, 3)), cutting=True)
    saved = s.checkpoint()
    builds = s.pair_list_builds.numpy()[0]
    s.advance(np.zeros((40, 3)), cutting=True)
    first = snapshot(s)
    assert np.count_nonzero(first["codes"]) > 0
    s.restore(saved)
    assert s.step_count == 25 and s.pair_list_builds.numpy()[0] == builds
    s.advance(np.zeros((40, 3)), cutting=True)  # the same cached graph, replayed again
    assert_equal(first, snapshot(s))


def test_state_assign_round_trip_resumes_a_contact_run():
    cfg = Config(young_modulus=20000.0)
    whole, resumed = Solver(cfg), Solver(cfg)
    for s in (whole, resumed):
        s.tool_pos.assign([[0.0, 0.0, 0.047]])
    target = (0.0, 0.0, 0.027)
    whole.advance(np.tile(target, (30, 1)), cutting=False)
    state = whole.state()
    resumed.x.assign(state["position"])
    resumed.v.assign(state["velocity"])
    resumed.F.assign(state["deformation"])
    assert np.all(state["plastic_deformation"] == np.eye(3, dtype=np.float32))  # no plasticity: Fp stays I
    resumed.codes.assign(state["sides"])
    resumed.damage.assign(state["damage"])
    resumed.tool_pos.assign(state["blade_position"])
    resumed.tool_vel.assign(state["blade_velocity"])
    resumed.tool_rot.assign(state["blade_orientation"])
    resumed.tool_omega.assign(state["blade_omega"])
    # state() gives the knife in float32, as the reference stores it; the knife
    # integrates in float64 here, so its full state is carried beside it
    np.testing.assert_array_equal(resumed._t["tool"].cpu().numpy().astype(np.float32),
                                  whole._t["tool"].cpu().numpy().astype(np.float32))
    resumed._t["tool"].copy_(whole._t["tool"])
    resumed._call("bm_sync_tool_mirror", resumed._stream)
    resumed.histories.assign(whole.histories.numpy())
    resumed.step_count = whole.step_count
    resumed.refresh_stress()
    assert np.all(resumed.pair_list_dirty.numpy() == 1)
    whole.advance(np.tile(target, (30, 1)), cutting=False)
    resumed.advance(np.tile(target, (30, 1)), cutting=False)
    a, b = snapshot(whole), snapshot(resumed)
    a.pop("work"), b.pop("work")  # the directional work sums over the whole run
    assert_equal(a, b)
    assert float(np.abs(whole.reaction.numpy()).max()) > 0  # the knife is in contact
