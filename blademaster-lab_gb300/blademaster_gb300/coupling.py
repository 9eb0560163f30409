"""External rigid-tool interface (paper III-G), restating blademaster_warp/coupling.py.

The tool state is set at the start of each coupling interval; contact
impulses are accumulated over its substeps and returned as an interval
impulse and angular impulse.  All quantities are SI in the material frame.
One interval is one CUDA-graph replay (load state, substeps, validate, store)
and one device-to-host read of the interval result.
"""

from dataclasses import dataclass
import ctypes
import time

import numpy as np

from . import _native


def vector(value, length, name):
    result = np.array(value, dtype=np.float64, copy=True)
    if result.shape != (length,) or not np.isfinite(result).all():
        raise ValueError(f"{name} must contain {length} finite values")
    return result


@dataclass(frozen=True)
class ToolState:
    """coupling.py:23-50."""

    position: object
    orientation_xyzw: object
    linear_velocity: object
    angular_velocity: object
    mobility: object = None

    def checked(self):
        position = vector(self.position, 3, "position")
        q = vector(self.orientation_xyzw, 4, "orientation_xyzw")
        if abs(np.linalg.norm(q) - 1.0) > 1.0e-5:
            raise ValueError("Tool orientation must be a unit xyzw quaternion")
        mobility = np.zeros((6, 6)) if self.mobility is None else np.asarray(self.mobility, dtype=float)
        if (
            mobility.shape != (6, 6)
            or not np.isfinite(mobility).all()
            or np.abs(mobility - mobility.T).max() > 1.0e-10
            or np.linalg.eigvalsh(mobility).min() < -1.0e-10
        ):
            raise ValueError("Mobility must be a finite symmetric positive-semidefinite 6x6 matrix")
        return ToolState(
            position,
            q / np.linalg.norm(q),
            vector(self.linear_velocity, 3, "linear_velocity"),
            vector(self.angular_velocity, 3, "angular_velocity"),
            mobility.copy(),
        )


@dataclass(frozen=True)
class Reaction:
    """coupling.py:53-72."""

    duration_s: float
    impulse_ns: np.ndarray
    angular_impulse_nms: np.ndarray
    origin_world_m: np.ndarray

    @property
    def force_n(self):
        return self.impulse_ns / self.duration_s

    @property
    def torque_nm(self):
        return self.angular_impulse_nms / self.duration_s

    def about(self, origin_world_m):
        """Shift the moment reference, preserving the same physical wrench."""
        origin = vector(origin_world_m, 3, "moment origin")
        angular = self.angular_impulse_nms + np.cross(self.origin_world_m - origin, self.impulse_ns)
        return Reaction(self.duration_s, self.impulse_ns.copy(), angular, origin)


class ExternalToolPort:
    """coupling.py:75-189."""

    def __init__(self, solver, record_trajectory=False):
        if not solver.config.external_tool:
            raise ValueError("ExternalToolPort requires Config(external_tool=True)")
        self.solver = solver
        self.record_trajectory = record_trajectory
        self.trajectory = None
        self.trajectory_times = None
        self.timing_s = dict(submission=0.0, completion_and_readback=0.0)

    def advance(self, state, duration_s, *, cutting=True, cut_index=0, graph=True):
        import torch

        submission_begin = time.perf_counter()
        state = state.checked()
        s = self.solver
        if not np.isfinite(duration_s) or duration_s <= 0:
            raise ValueError("Coupling duration must be positive and finite")
        steps = int(round(duration_s / s.config.dt))
        if steps < 1 or abs(steps * s.config.dt - duration_s) > 1.0e-12 + 1.0e-10 * abs(duration_s):
            raise ValueError("Coupling duration must be an integer number of material substeps")
        if steps > 4096:
            raise ValueError("A coupling interval holds at most 4096 substeps")
        cut_index = s._set_cut(cut_index)
        held_pose = s.config.tool_substep == "hold"
        samples = (2 if held_pose else steps + 1) if self.record_trajectory else 0
        packed = np.concatenate(
            [state.position, state.orientation_xyzw, state.linear_velocity, state.angular_velocity, state.mobility.ravel()]
        ).astype(np.float32)
        s._t["packed"].copy_(torch.as_tensor(packed, device=s.device))
        s._sync_step()
        extra = dict(external_load=1, external_finish=1, record_samples=samples, hold_pose=int(held_pose))
        if graph:
            handle = s.prepare(np.zeros((steps, 3), np.float32), cutting, cut_index, tag=("external",), use_targets=0, **extra)
            _native.check(s._lib.bm_graph_launch(handle, s._stream))
        else:
            args = s._step_args(steps, cutting, cut_index, use_targets=0, **extra)
            _native.check(s._lib.bm_substeps(s._handle, ctypes.byref(args), s._stream))
        s._advanced(steps)
        readback_begin = time.perf_counter()
        self.timing_s["submission"] += readback_begin - submission_begin
        out = s._t["result"][: 10 + 7 * samples].cpu().numpy().astype(np.float64)
        interval = s._t["interval"].cpu().numpy()
        self.timing_s["completion_and_readback"] += time.perf_counter() - readback_begin
        impulse, angular, errors = interval[:3].copy(), interval[3:6].copy(), out[6:9]
        residual = s.blade_constraint.max_violation if s.blade_constraint is not None else 0.0
        if self.record_trajectory:
            self.trajectory = out[9 : 9 + 7 * samples].reshape(samples, 7)
            self.trajectory_times = np.linspace(0.0, duration_s, samples)
        (px, py, pz), (ix, iy, iz) = state.position, impulse
        angular -= (py * iz - pz * iy, pz * ix - px * iz, px * iy - py * ix)
        if errors.any() or not np.isfinite([impulse, angular]).all():
            raise RuntimeError(f"Invalid material coupling interval: GPU errors {errors.astype(int).tolist()}")
        if not np.isfinite(residual) or residual > 1.0e-6:
            raise RuntimeError(f"Blade grid contact did not converge: inward residual {residual:.6g} m/s")
        return Reaction(float(duration_s), impulse, angular, state.position.copy())
