"""Batched sweeps: many independent cutting instances per CUDA-graph launch.

The reference runs sweep instances (different spacings, blade offsets, speeds
and materials) one after another, one ExternalToolPort.advance per instance
and coupling interval (scripts/force_convergence.py:92-129).  ``SolverBatch``
advances every instance's interval with one graph launch: each instance's
substep chain is an independent branch of the graph, captured on a number of
lanes (concurrent streams) that ``BatchTuner`` picks by measurement.  The
knife states of all instances go to the device in one copy, and all interval
results come back in one copy.  Each instance computes exactly what its own
ExternalToolPort.advance computes (the kernels and their order are the same).
"""

import ctypes
import json
import os
import time
from pathlib import Path

import numpy as np

from . import _native
from .coupling import Reaction

RESULT_WORDS = 10  # impulse 3, angular 3, errors 3, residual slot


class SolverBatch:
    """External-tool solvers advanced together (one graph launch per interval)."""

    def __init__(self, solvers, lanes=None):
        import torch

        if not solvers:
            raise ValueError("A batch needs at least one solver")
        for s in solvers:
            if not s.config.external_tool:
                raise ValueError("SolverBatch requires Config(external_tool=True) for every solver")
            if s.device != solvers[0].device:
                raise ValueError("All solvers of a batch must share one device")
        self.solvers = list(solvers)
        self.device = solvers[0].device
        self._lib = _native.lib()
        count = len(solvers)
        # gather the per-interval buffers of all instances into batch tensors
        self._packed = torch.zeros(count, 49, dtype=torch.float32, device=self.device)
        self._interval = torch.zeros(count, 6, dtype=torch.float64, device=self.device)
        self._result = torch.zeros(count, solvers[0]._t["result"].numel(), dtype=torch.float32, device=self.device)
        self._flags = torch.stack([s._t["flags"] for s in solvers]).contiguous()
        self._host_packed = torch.zeros(count, 49, dtype=torch.float32).pin_memory()
        for i, s in enumerate(self.solvers):
            s._t["packed"] = self._packed[i]
            s._t["interval"] = self._interval[i]
            s._t["result"] = self._result[i]
            s._t["flags"] = self._flags[i]
            s._drop_graphs()
            s._views()
            s._bind()
        self.lanes = lanes or min(count, 32)
        self._graphs = {}
        self.timing_s = dict(submission=0.0, completion_and_readback=0.0)
        self.failures = []  # (instance, interval) that failed the port's checks when strict=False
        self.intervals = 0

    def __del__(self):
        for g in getattr(self, "_graphs", {}).values():
            self._lib.bm_graph_destroy(g)

    @property
    def _stream(self):
        import torch

        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _order(self):
        """Largest instances first, dealt round-robin over the lanes (balances the lanes' work)."""
        return sorted(range(len(self.solvers)), key=lambda i: -self.solvers[i].n)

    def graph(self, steps, cutting, cut_index, lanes=None):
        lanes = lanes or self.lanes
        key = (tuple(steps), bool(cutting), tuple(cut_index), lanes)
        if key not in self._graphs:
            order = self._order()
            handles = (ctypes.c_void_p * len(order))()
            args = (_native.StepArgs * len(order))()
            for pos, i in enumerate(order):
                s = self.solvers[i]
                handles[pos] = s._handle.value
                held = s.config.tool_substep == "hold"
                args[pos] = s._step_args(steps[i], cutting, cut_index[i], use_targets=0, external_load=1,
                                         external_finish=1, record_samples=0, hold_pose=int(held))
            handle = ctypes.c_void_p()
            _native.check(self._lib.bm_batch_graph_create(handles, args, len(order), lanes, self._stream,
                                                          ctypes.byref(handle)))
            self._graphs[key] = handle
        return self._graphs[key]

    def advance(self, states, duration_s, *, cutting=True, cut_index=0, lanes=None, strict=True):
        """ExternalToolPort.advance (coupling.py:88-189) for every instance; returns one Reaction each.

        With strict=True an instance with device errors or a non-converged held-blade
        constraint raises RuntimeError, as the port does; with strict=False its
        Reaction is still returned and (instance, interval) is added to ``failures``.
        """
        import torch

        begin = time.perf_counter()
        if len(states) != len(self.solvers):
            raise ValueError("One tool state per instance is required")
        if not np.isfinite(duration_s) or duration_s <= 0:
            raise ValueError("Coupling duration must be positive and finite")
        cut = [cut_index] * len(self.solvers) if np.isscalar(cut_index) else list(cut_index)
        steps, checked = [], []
        for s, state, c in zip(self.solvers, states, cut):
            n = int(round(duration_s / s.config.dt))
            if n < 1 or abs(n * s.config.dt - duration_s) > 1.0e-12 + 1.0e-10 * abs(duration_s):
                raise ValueError("Coupling duration must be an integer number of material substeps")
            if n > 4096:
                raise ValueError("A coupling interval holds at most 4096 substeps")
            steps.append(n)
            state = state.checked()
            checked.append(state)
        cut = [s._set_cut(c) for s, c in zip(self.solvers, cut)]
        host = self._host_packed.numpy()
        for i, state in enumerate(checked):
            host[i, :3], host[i, 3:7] = state.position, state.orientation_xyzw
            host[i, 7:10], host[i, 10:13] = state.linear_velocity, state.angular_velocity
            host[i, 13:] = state.mobility.ravel()
        self._packed.copy_(self._host_packed, non_blocking=True)
        for s in self.solvers:
            s._sync_step()
        _native.check(self._lib.bm_graph_launch(self.graph(steps, cutting, cut, lanes), self._stream))
        for s, n in zip(self.solvers, steps):
            s._advanced(n)
        readback = time.perf_counter()
        self.timing_s["submission"] += readback - begin
        interval = self._interval.cpu().numpy()
        result = self._result[:, :RESULT_WORDS].cpu().numpy().astype(np.float64)
        residuals = self._flags[:, _native.FLAG["HOLD_RESIDUAL"]].cpu().numpy().view(np.float32)
        self.timing_s["completion_and_readback"] += time.perf_counter() - readback
        out = []
        for i, (s, state) in enumerate(zip(self.solvers, checked)):
            impulse, angular, errors = interval[i, :3].copy(), interval[i, 3:6].copy(), result[i, 6:9]
            (px, py, pz), (ix, iy, iz) = state.position, impulse
            angular -= (py * iz - pz * iy, pz * ix - px * iz, px * iy - py * ix)
            problem = None
            if errors.any() or not np.isfinite([impulse, angular]).all():
                problem = f"Invalid material coupling interval in instance {i}: GPU errors {errors.astype(int).tolist()}"
            residual = float(residuals[i]) if s.blade_constraint is not None else 0.0
            if problem is None and (not np.isfinite(residual) or residual > 1.0e-6):
                problem = f"Blade grid contact did not converge in instance {i}: inward residual {residual:.6g} m/s"
            if problem is not None:
                if strict:
                    raise RuntimeError(problem)
                self.failures.append((i, self.intervals))
            out.append(Reaction(float(duration_s), impulse, angular, state.position.copy()))
        self.intervals += 1
        return out


class BatchTuner:
    """Picks the lane count of a batch by timing real intervals.

    Candidates are timed on the batch's own coupling intervals (their results
    are real and returned); the fastest is kept for the rest of the run and
    cached in a JSON file keyed by the device and the batch's size profile.
    """

    def __init__(self, cache=None, candidates=(8, 16, 32, 64, 128)):
        self.cache = Path(cache or os.environ.get("BM_TUNE_CACHE", Path.home() / ".cache" / "blademaster_gb300_tune.json"))
        self.candidates = candidates

    @staticmethod
    def signature(batch):
        import torch

        sizes = sorted(s.n for s in batch.solvers)
        name = torch.cuda.get_device_name(batch.device)
        return f"{name}|{len(sizes)}|{sizes[0]}|{sizes[len(sizes) // 2]}|{sizes[-1]}"

    def _load(self):
        try:
            return json.loads(self.cache.read_text())
        except (OSError, ValueError):
            return {}

    def tune(self, batch, states_for, duration_s, **kw):
        """Time each candidate on one interval (states_for(i) gives interval i's states); returns the reactions."""
        import torch

        key = self.signature(batch)
        known = self._load().get(key)
        if known:
            batch.lanes = int(known)
            return []
        reactions, timings = [], {}
        for i, lanes in enumerate(c for c in self.candidates if c <= len(batch.solvers)):
            states = states_for(i)
            batch.graph([int(round(duration_s / s.config.dt)) for s in batch.solvers], kw.get("cutting", True),
                        [kw.get("cut_index", 0)] * len(batch.solvers), lanes)
            torch.cuda.synchronize(batch.device)
            begin = time.perf_counter()
            reactions.append(batch.advance(states, duration_s, lanes=lanes, **kw))
            timings[lanes] = time.perf_counter() - begin
        if timings:
            batch.lanes = min(timings, key=timings.get)
            table = self._load()
            table[key] = batch.lanes
            try:
                self.cache.parent.mkdir(parents=True, exist_ok=True)
                self.cache.write_text(json.dumps(table, indent=1))
            except OSError:
                pass
        self.timings = timings
        return reactions
