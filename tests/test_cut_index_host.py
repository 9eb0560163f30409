"""Cut-index bookkeeping of the Solver, on the host alone.

The reference's cases (tests/test_stress_replays.py:134-220) run the real
`Solver._set_cut`, `Solver.step` and `Solver.advance` on a stand-in that
holds only the host state they read: the configuration, the largest cut
index, the current index and the knives' damage arrays.  Kernel dispatch is
replaced by a recorder.  Invalid indices and orientations are refused before
any history changes, and numpy indices reach dispatch as Python ints.  No GPU.
"""

import types

import numpy as np
import pytest

from blademaster_gb300.solver import Config, Solver, cut_capacity
from oracle.oracle import OracleSolver

DEFAULT_NODES = OracleSolver(Config()).node_count
DEFAULT_LAST = cut_capacity(DEFAULT_NODES)


class Values:
    """A damage array's host stand-in with the device array's fill_/zero_/numpy."""

    def __init__(self, value=0.0):
        self.a = np.array([value], np.float32)

    def fill_(self, value):
        self.a[:] = value

    def zero_(self):
        self.a[:] = 0.0

    def numpy(self):
        return self.a.copy()


class HostOnly:
    def __init__(self, config=Config(), max_cut_index=DEFAULT_LAST):
        self.config = config
        self.max_cut_index = max_cut_index
        self.cut_index = 0
        self.tool_damage = [Values() for _ in range(config.tool_count)]
        self.damage = self.tool_damage[0]
        self.dispatched = []
        for name in ("_set_cut", "step", "advance"):
            setattr(self, name, types.MethodType(getattr(Solver, name), self))

    def _step_kernels(self, target, cutting, cut_index, **kwargs):
        assert type(cut_index) is int
        self.dispatched.append(3**cut_index)


def test_default_block_has_34_digits():
    # test_stress_replays.py:48-60: node_count 225 -> cut indices 0 .. 33
    assert DEFAULT_NODES == 225 and DEFAULT_LAST == 33


@pytest.mark.parametrize("value", [0.5, 1.0, float("nan"), float("inf"), True, np.bool_(True), "1", None])
def test_invalid_cut_index_type_is_rejected_before_history_mutation(value):
    # test_stress_replays.py:134-145
    probe = HostOnly(Config(free_blade=True, tool_count=3))
    for slot, damage in enumerate(probe.tool_damage):
        damage.fill_(0.125 * (slot + 1))
    with pytest.raises(ValueError, match="integer"):
        probe._set_cut(value)
    assert probe.cut_index == 0
    for slot, damage in enumerate(probe.tool_damage):
        np.testing.assert_array_equal(damage.numpy(), [0.125 * (slot + 1)])


@pytest.mark.parametrize("dtype", [np.int32, np.int64])
def test_numpy_cut_indices_normalize_to_python_int_before_power(dtype):
    # test_stress_replays.py:148-159
    probe = HostOnly()
    probe.damage.fill_(0.75)
    index = probe._set_cut(dtype(probe.max_cut_index))
    assert type(index) is int and type(probe.cut_index) is int
    assert 3**index == 3**33
    np.testing.assert_array_equal(probe.damage.numpy(), [0])
    probe.damage.fill_(0.75)
    assert probe._set_cut(dtype(index)) == index
    np.testing.assert_array_equal(probe.damage.numpy(), [0.75])


@pytest.mark.parametrize("method", ["step", "advance"])
@pytest.mark.parametrize("dtype", [np.int32, np.int64])
def test_high_numpy_indices_reach_kernel_dispatch_as_python_int(method, dtype):
    # test_stress_replays.py:162-176
    probe = HostOnly()
    if method == "step":
        probe.step(cut_index=dtype(33))
    else:
        probe.advance([[0, 0, 0.041]], cut_index=dtype(33), graph=False)
    assert probe.dispatched == [3**33]


@pytest.mark.parametrize("invalid", [-1, 34, np.int64(34), 2**80])
def test_out_of_range_cut_indices_preserve_history(invalid):
    # test_stress_replays.py:179-190
    probe = HostOnly()
    probe._set_cut(33)
    probe.damage.fill_(0.75)
    with pytest.raises(ValueError, match="monotonic"):
        probe._set_cut(invalid)
    assert probe.cut_index == 33
    np.testing.assert_array_equal(probe.damage.numpy(), [0.75])


@pytest.mark.parametrize("orientations", [[[0, 0, 1]], [[0, 0, 0, 0]], [[0, 0, float("nan"), 1]],
                                          [[0, 0, float("inf"), 1]]])
def test_malformed_advance_orientation_preserves_previous_cut_history(orientations):
    # test_stress_replays.py:193-219
    probe = HostOnly()
    probe.damage.fill_(0.75)
    with pytest.raises(ValueError, match="orientations|quaternion"):
        probe.advance([[0, 0, 0.041]], cut_index=1, graph=False, orientations=orientations)
    assert probe.cut_index == 0 and probe.dispatched == []
    np.testing.assert_array_equal(probe.damage.numpy(), [0.75])


@pytest.mark.parametrize("targets", [[], [[0, 0]], [[0, 0, float("nan")]], [[0, 0, float("inf")]], [0, 0, 0.041]])
def test_malformed_advance_targets_preserve_previous_cut_history(targets):
    # solver.py:942-973: targets must be finite (substeps, 3) edge positions, refused before the cut moves
    probe = HostOnly()
    probe.damage.fill_(0.75)
    with pytest.raises(ValueError, match="targets"):
        probe.advance(targets, cut_index=1, graph=False)
    assert probe.cut_index == 0 and probe.dispatched == []
    np.testing.assert_array_equal(probe.damage.numpy(), [0.75])


def test_externally_owned_tool_refuses_the_solvers_own_stepping():
    # tests/test_coupling.py:74-79 on the host
    probe = HostOnly(Config(external_tool=True))
    with pytest.raises(ValueError, match="ExternalToolPort"):
        probe.step()
    with pytest.raises(ValueError, match="ExternalToolPort"):
        probe.advance([[0.0, 0.0, 0.0]])
    assert probe.dispatched == [] and probe.cut_index == 0
