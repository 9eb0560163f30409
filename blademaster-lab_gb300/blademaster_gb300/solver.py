"""TLMPM material solver with rigid knives, all per-substep work in sm_103a CUDA.

Drop-in for ``blademaster_warp/solver.py``: the same ``Config`` (fields,
defaults and validation messages, solver.py:12-149) and the same ``Solver``
methods and device-array attributes, driving the C-ABI library
(include/blademaster_gb300.h) instead of Warp kernels.

Device layout (not visible through the API): particles are stored sorted by
reference cell in structure-of-arrays form; a node's cut fields live at slot
``f * node_count + node``; the knife state is float64 with a float32 mirror.
Attribute views (``s.x``, ``s.codes``, ...) translate to and from the
reference's shapes and particle order.
"""

from dataclasses import dataclass, asdict
import ctypes
import time

import numpy as np

from . import _native
from .arrays import DeviceArray, particle_view, plain_view, soa_view
from .geometry import points, stencil, cell_sort, stencil_table, reference_cells, OFFSETS

CUT_ON, CUT_ADVANCE, CUT_HOLD = _native.CUT_ON, _native.CUT_ADVANCE, _native.CUT_HOLD


@dataclass(frozen=True)
class Config:
    size: tuple = (0.06, 0.03, 0.03)
    grid_spacing: float = 0.0075
    dt: float = 0.0005
    density: float = 1100.0
    young_modulus: float = 6000.0
    poisson_ratio: float = 0.35
    dynamic_viscosity: float = 0.0
    maxwell_tau: float = 0.0
    maxwell_fraction: float = 0.0
    yield_stress: float = 0.0
    flip_fraction: float = 0.95
    normal_scale: float = 0.1
    friction_static: float = 0.3
    friction_dynamic: float = 0.2
    tangent_stiffness: float = 0.05
    tangent_damping: float = 0.1
    contact_reference_dt: float = 0.0
    cutting_energy: float = 0.5
    sharpness: float = 0.9
    cut_work: str = "relative"
    cut_hold: bool = False
    blade_contact_radius: float = 0.0
    blade_mass: float = 0.2
    blade_half_size: tuple = (0.0005, 0.025, 0.02)
    drive_stiffness: float = 250.0
    drive_damping: float = 14.0
    drive_force_limit: float = 10.0
    shape: str = "block"
    sampling_seed: int = 0
    blade_bevel_height: float = 0.0
    free_blade: bool = False
    pose_servo: bool = False
    external_tool: bool = False
    cache_topology: bool = False
    grid_storage: str = "hash"
    pair_search: str = "auto"
    pair_skin: float = 0.0
    tool_substep: str = "hold"
    accumulate_tool_impulses: bool = False
    rotational_stiffness: float = 0.05
    rotational_damping: float = 0.003
    board_half_extent: tuple = (0.0, 0.0)
    board_normal_scale: float = 0.0
    tool_count: int = 1

    def __post_init__(self):
        """Validation of solver.py:87-144, message for message."""
        if self.grid_storage not in ("hash", "compact"):
            raise ValueError("grid_storage must be hash or compact")
        if self.pair_search not in ("auto", "hash", "all", "list"):
            raise ValueError("pair_search must be auto, hash, all or list")
        if self.pair_skin < 0:
            raise ValueError("pair_skin must be non-negative")
        if self.blade_contact_radius < 0:
            raise ValueError("blade_contact_radius must be non-negative")
        if self.cut_work not in ("relative", "advance"):
            raise ValueError("cut_work must be relative or advance")
        if self.tool_substep not in ("hold", "predict"):
            raise ValueError("tool_substep must be hold or predict")
        if self.tool_substep == "predict" and not self.external_tool:
            raise ValueError("tool_substep=predict requires external_tool")
        numeric = [float(v) for k, v in asdict(self).items() if isinstance(v, (int, float))]
        if not np.isfinite(numeric).all():
            raise ValueError("Nonfinite configuration")
        positive = (
            "dt",
            "grid_spacing",
            "density",
            "young_modulus",
            "normal_scale",
            "tangent_stiffness",
            "blade_mass",
            "cutting_energy",
            "drive_force_limit",
        )
        if any(getattr(self, k) <= 0 for k in positive):
            raise ValueError("Invalid positive parameter")
        if not (0 < self.poisson_ratio < 0.5 and 0 < self.sharpness < 1):
            raise ValueError("Invalid material/sharpness")
        if not (0 <= self.flip_fraction <= 1 and 0 <= self.friction_dynamic <= self.friction_static):
            raise ValueError("Invalid transfer/friction")
        if min(self.dynamic_viscosity, self.yield_stress, self.tangent_damping, self.contact_reference_dt) < 0:
            raise ValueError("Negative damping/plasticity/reference step")
        if self.maxwell_tau < 0 or not 0 <= self.maxwell_fraction <= 1:
            raise ValueError("maxwell_tau must be non-negative and maxwell_fraction in [0, 1]")
        if max(self.contact_scales()) > 1:
            raise ValueError("Rescaled contact factor exceeds 1 (one-step overshoot); reduce dt")
        if not 0 <= self.board_normal_scale <= 1:
            raise ValueError("Board normal scale must be in [0, 1]")
        if min(self.board_half_extent) < 0:
            raise ValueError("Board half extent must be non-negative")
        if not 0 <= self.blade_bevel_height < 2 * self.blade_half_size[2]:
            raise ValueError("Invalid blade geometry")
        if sum((self.free_blade, self.pose_servo, self.external_tool)) > 1:
            raise ValueError("Choose free, pose-servo, or externally prescribed tool")
        if self.tool_count < 1 or (
            self.tool_count > 1 and not (self.free_blade and not self.accumulate_tool_impulses)
        ):
            raise ValueError("Several tools are supported only as free knives")
        if self.tool_count > _native.MAX_TOOLS:
            raise ValueError(f"At most {_native.MAX_TOOLS} knives")
        if self.grid_spacing <= 0 or min(np.asarray(self.size) / self.grid_spacing) < 2:
            raise ValueError("Grid spacing must be positive with at least two cells per axis")

    def contact_scales(self):
        """Effective (s_n, gamma_k) at this dt (solver.py:146-149)."""
        ratio = 1.0 if self.contact_reference_dt == 0 else (self.dt / self.contact_reference_dt) ** 2
        return self.normal_scale * ratio, self.tangent_stiffness * ratio


PAIR_LANES = 64
PAIR_LIST_LANES = _native.PAIR_LANES
MAX_BATCH = 4096
FIELD_SLOTS = 64  # a node has at most 8 cells x 8 particles = 64 distinct codes


def cut_capacity(node_count):
    """The largest cut index whose codes still key every node within int64.

    Cut index i sets ternary digit i, so indices 0 .. m give codes below 3^(m+1)
    and keys code * node_count + node below node_count * 3^(m+1), which must
    stay within 2^63 - 1 (solver.py:168-171; scripts/stress_multi_tool.py:21-43).
    """
    m = 0
    while 3 ** (m + 2) * node_count <= 2**63 - 1:
        m += 1
    return m


def _pow2_at_least(v):
    return 1 << (max(int(v), 1) - 1).bit_length()


class BladeConstraint:
    """Grid constraint of an externally held knife (blade_constraint.py:213-324).

    Runs inside every substep of an external tool in hold mode; ``solve()``
    runs it alone on the current grid velocities, as the reference's tests do.
    ``max_violation`` is the largest final inward residual (m/s) of any solve
    so far, which ExternalToolPort.advance checks against 1e-6 m/s.
    """

    def __init__(self, solver):
        self.solver = solver

    def solve(self):
        self.solver._call("bm_hold_constraint", self.solver._stream)

    @property
    def max_violation(self):
        bits = np.int32(self.solver._flag("HOLD_RESIDUAL"))
        return float(bits.view(np.float32))


class Solver:
    def __init__(self, config=Config(), device="cuda:0"):
        import torch

        self.config = config
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("CUDA device required")
        if not torch.cuda.is_available():
            raise RuntimeError("CUDA is not available: the GB300 kernels have no CPU fallback")
        self._lib = _native.lib()
        cfg = config
        self.reference, self.origin, cells = points(cfg.size, cfg.grid_spacing, cfg.shape, cfg.sampling_seed)
        self.n = n = len(self.reference)
        if n == 0:
            raise ValueError("The shape holds no particles at this spacing")
        nodes, weights, gradients = stencil(self.reference, self.origin, cfg.grid_spacing, cells)
        self.cells = cells
        self.node_dims = cells + 1
        self.node_count = int(np.prod(cells + 1))
        self.max_cut_index = cut_capacity(self.node_count)
        self.node_numpy, self.weight_numpy = nodes, weights
        self.gradient_numpy = gradients
        self.volume = (cfg.grid_spacing / 2) ** 3
        self.mass = cfg.density * self.volume
        self.radius = cfg.grid_spacing / 4
        self.blade_offset = max(cfg.blade_contact_radius or self.radius, self.radius - cfg.blade_half_size[0])
        self.mu = cfg.young_modulus / (2 * (1 + cfg.poisson_ratio))
        self.lam = cfg.young_modulus * cfg.poisson_ratio / ((1 + cfg.poisson_ratio) * (1 - 2 * cfg.poisson_ratio))
        self.maxwell = cfg.maxwell_tau > 0 and cfg.maxwell_fraction > 0
        self.mu_maxwell = cfg.maxwell_fraction * self.mu
        self.maxwell_relax = float(-np.expm1(-cfg.dt / cfg.maxwell_tau)) if self.maxwell else 0.0
        self.threshold = cfg.cutting_energy * self.volume ** (2 / 3) * (1 - cfg.sharpness) / cfg.sharpness
        self.normal_scale, self.tangent_stiffness = cfg.contact_scales()
        self.board_scale = cfg.board_normal_scale or self.normal_scale
        hx, hy, hz = cfg.blade_half_size
        self.inertia_inv = 3 / (cfg.blade_mass * np.array([hy * hy + hz * hz, hx * hx + hz * hz, hx * hx + hy * hy]))
        self.pair_list = cfg.pair_search in ("list", "auto")
        self.all_pairs = cfg.pair_search == "all"
        self.pair_skin = (cfg.pair_skin or self.radius) if self.pair_list else 0.0
        self.pair_capacity = _pow2_at_least(max(64 * n, 16))
        self.capacity = _pow2_at_least(max(16 * n, 16))
        self.compact = cfg.grid_storage == "compact"

        # device particle order: by reference cell
        order, cell_start = cell_sort(self.reference, self.origin, cfg.grid_spacing, cells)
        rank = np.empty(n, np.int64)
        rank[order] = np.arange(n)
        self.order, self.rank = order, rank
        table_w, table_g, sid = stencil_table(weights, gradients)
        _, base_cell = reference_cells(self.reference, self.origin, cfg.grid_spacing, cells)
        base_node = np.ravel_multi_index(base_cell.T, tuple(cells + 1))
        counts = np.diff(cell_start)
        occupied = np.flatnonzero(counts > 0)
        occ = np.stack(np.unravel_index(occupied, tuple(cells)), axis=1)
        corners = (occ[:, None, :] + OFFSETS[None]).reshape(-1, 3)
        active = np.unique(np.ravel_multi_index(corners.T, tuple(cells + 1)))
        self.active_nodes = active
        self.fmax = FIELD_SLOTS
        self.grid_capacity = self.fmax * self.node_count
        self.buckets = _pow2_at_least(max(2 * n, 1024))

        t = torch
        dev = self.device
        K = cfg.tool_count
        S = self.grid_capacity
        f32, f64, i32, i64 = t.float32, t.float64, t.int32, t.int64

        def zeros(*shape, dtype=f32):
            return t.zeros(shape, dtype=dtype, device=dev)

        self._order_t = t.as_tensor(order, device=dev)
        self._rank_t = t.as_tensor(rank, device=dev)
        ref_sorted = self.reference[order]
        T = {}
        T["x"] = t.as_tensor(ref_sorted.T.astype(np.float32), device=dev).contiguous()
        T["v"] = zeros(3, n)
        T["ref"] = T["x"].clone()
        eye = t.eye(3, dtype=f32, device=dev).reshape(9, 1)
        T["F"] = eye.repeat(1, n).contiguous()
        T["Fp"] = eye.repeat(1, n).contiguous()
        T["stress"] = zeros(9, n)
        T["viscous"] = zeros(9, n if self.maxwell else 1, dtype=f64)
        T["codes"] = zeros(n, dtype=i64)
        T["zero_codes"] = zeros(n, dtype=i64)
        T["damage"] = zeros(K, n)
        T["histories"] = zeros(1 + K, 3, n)
        T["impulses"] = zeros(3, n)
        T["stencil_id"] = t.as_tensor(sid[order], dtype=i32, device=dev)
        T["stencil_w"] = t.as_tensor(table_w, device=dev).contiguous()
        T["stencil_g"] = t.as_tensor(table_g, device=dev).contiguous()
        T["base_node"] = t.as_tensor(base_node[order], dtype=i32, device=dev)
        T["fidx"] = zeros(n, dtype=i64)
        T["cell_start"] = t.as_tensor(cell_start, dtype=i32, device=dev)
        T["active"] = t.as_tensor(active, dtype=i32, device=dev)
        T["nfield"] = zeros(self.node_count, dtype=i32)
        T["fcode"] = zeros(self.fmax, self.node_count, dtype=i64)
        T["fones"] = zeros(self.fmax, self.node_count, dtype=i64)
        T["ftwos"] = zeros(self.fmax, self.node_count, dtype=i64)
        T["grid_mass"] = zeros(S)
        for name in ("momentum", "grid_impulse", "old_v", "new_v", "remapped", "remap_v"):
            T[name] = zeros(3, S)
        T["cell_part"] = zeros(7, 8, self.node_count)
        T["cell_field"] = t.as_tensor(np.ascontiguousarray(self._absent_corners(cell_start).T), device=dev)
        T["multi_nodes"] = zeros(len(active), dtype=i32)
        T["mixed_cells"] = zeros(int(np.prod(cells)), dtype=i32)
        T["hist_mask"] = t.full((n,), -1, dtype=t.int16, device=dev)
        T["built_x"] = zeros(3, n)
        T["built_codes"] = zeros(n, dtype=i64)
        T["partners"] = zeros(n, PAIR_LIST_LANES, dtype=i32)
        T["partner_count"] = zeros(n, dtype=i32)
        T["candidates"] = zeros(n, dtype=i32)
        T["bucket_start"] = zeros(self.buckets + 1, dtype=i32)
        T["bucket_items"] = zeros(n, dtype=i32)
        T["bucket_fill"] = zeros(self.buckets, dtype=i32)
        T["particle_bucket"] = zeros(n, dtype=i32)
        T["particle_key"] = zeros(n, dtype=i64)
        T["bucket_key"] = zeros(n, dtype=i64)
        T["bucket_pos"] = zeros(n, 4)
        T["pair_keys"] = t.full((2, self.pair_capacity), -1, dtype=i64, device=dev)
        T["pair_history"] = zeros(2, self.pair_capacity, 3)
        T["pair_used"] = zeros(2, self.pair_capacity, dtype=i32)
        T["pair_count"] = zeros(2, dtype=i32)
        T["changed"] = zeros(n, dtype=i32)
        T["relist"] = zeros(n, dtype=i32)
        T["relist_list"] = zeros(n, dtype=i32)
        T["listed"] = zeros(n, dtype=i32)
        T["reg_node_mark"] = zeros(self.node_count, dtype=i32)
        T["reg_nodes"] = zeros(self.node_count, dtype=i32)
        T["reg_cell_mark"] = zeros(int(np.prod(cells)), dtype=i32)
        T["reg_cells"] = zeros(int(np.prod(cells)), dtype=i32)
        tool = np.zeros((K, 13))
        tool[:, 2] = np.float32(cfg.size[2] + 0.012 + hz)
        tool[:, 9] = 1.0
        T["tool"] = t.as_tensor(tool, device=dev)
        T["tool_f"] = zeros(K, _native.TOOL_F_WORDS)
        T["mobility"] = zeros(36)
        T["acc"] = zeros(_native.ACC_WORDS, dtype=i64)
        T["interval"] = zeros(6, dtype=f64)
        T["table_impulse"] = zeros(K, 3, dtype=f64)
        T["speed"] = zeros(1)
        T["errors"] = zeros(3, dtype=i32)
        T["flags"] = zeros(_native.FLAG["WORDS"], dtype=i32)
        T["targets"] = zeros(MAX_BATCH, 3)
        T["rotations"] = zeros(MAX_BATCH, 4)
        T["rotations"][:, 3] = 1.0
        T["packed"] = zeros(49)
        T["result"] = zeros(10 + 7 * (MAX_BATCH + 1))
        # held-blade constraint state (blade_constraint.py:213-240), sized only in hold mode
        hold = cfg.external_tool and cfg.tool_substep == "hold"
        nh, nc = (n, self.node_count) if hold else (1, 1)
        T["hold"] = zeros(11, nh)
        for name in ("hold_mark", "hold_pos", "hold_list"):
            T[name] = zeros(nh, dtype=i32)
        T["hold_entry"] = zeros(8 * nh, dtype=i32)
        T["hold_node_start"] = zeros(nc + 1, dtype=i32)
        T["hold_nodes"] = zeros(nc, dtype=i32)
        T["hold_node_mark"] = zeros(nc, dtype=i32)
        self._t = T
        self._use_fp = bool(cfg.yield_stress > 0)
        self._params = self._make_params()
        T["scratch"] = zeros(int(self._lib.bm_scratch_words(ctypes.byref(self._params))), dtype=i32)
        T["flags"][_native.FLAG["TOPOLOGY_DIRTY"]] = 1
        T["flags"][_native.FLAG["HOST_DIRTY"]] = 1
        T["flags"][_native.FLAG["PAIR_DIRTY"]] = 1
        self._handle = None
        self._bind()
        self._call("bm_sync_tool_mirror", self._stream)
        self._views()
        self.blade_constraint = BladeConstraint(self) if hold else None
        self.field_codes = self.codes
        self.step_count = 0
        self._device_step = 0  # the substep counter the device holds (flags start at zero)
        self.cut_index = 0
        self._batches = {}
        self.graph_build_s = 0.0
        self.refresh_stress()

    def _absent_corners(self, cell_start):
        """cell_field with 254 where node n has no (non-empty) cell at corner a.

        Particles never change reference cell, so this is set once; the cell
        pass overwrites the other entries every substep.
        """
        dims = self.node_dims
        ijk = np.stack(np.unravel_index(np.arange(self.node_count), tuple(dims)), axis=1)
        counts = np.diff(cell_start)
        field = np.full((8, self.node_count), 254, np.uint8)
        for a, offset in enumerate(OFFSETS):
            c = ijk - offset
            inside = np.all((c >= 0) & (c < self.cells), axis=1)
            linear = np.ravel_multi_index(c[inside].T, tuple(self.cells))
            occupied = np.zeros(self.node_count, bool)
            occupied[np.flatnonzero(inside)[counts[linear] > 0]] = True
            field[a][occupied] = 0
        return field

    # ------------------------------------------------------------ binding

    def _make_params(self):
        cfg = self.config
        P = _native.Params()
        P.n = self.n
        P.node_count = self.node_count
        for i in range(3):
            P.node_dims[i] = int(self.node_dims[i])
            P.cell_dims[i] = int(self.cells[i])
        P.active_nodes = len(self.active_nodes)
        P.fmax = self.fmax
        P.stencil_rows = self._t["stencil_w"].shape[0]
        P.tool_count = cfg.tool_count
        P.pair_capacity = self.pair_capacity
        P.bucket_mask = self.buckets - 1
        P.candidate_capacity = self.n
        P.tool_model = self._tool_model()
        P.external_tool = int(cfg.external_tool)
        P.predict = int(cfg.tool_substep == "predict")
        P.free_blade = int(cfg.free_blade)
        P.lock_rotation = int(not (cfg.free_blade or cfg.pose_servo))
        P.accumulate_tool_impulses = int(cfg.accumulate_tool_impulses)
        P.plastic = int(cfg.yield_stress > 0)
        P.use_fp = int(self._use_fp or cfg.yield_stress > 0 or self.maxwell)
        P.maxwell = int(self.maxwell)
        P.viscous = int(cfg.dynamic_viscosity > 0)
        P.pair_search = 0 if self.pair_list else 1
        P.cache_topology = int(cfg.cache_topology)
        P.dt = cfg.dt
        P.spacing = cfg.grid_spacing
        P.mass = self.mass
        P.volume = self.volume
        P.radius = self.radius
        P.mu = self.mu
        P.lam = self.lam
        P.mu_maxwell = self.mu_maxwell
        P.maxwell_relax = self.maxwell_relax
        P.yield_stress = cfg.yield_stress
        P.flip = cfg.flip_fraction
        P.dynamic_viscosity = cfg.dynamic_viscosity
        P.normal_scale = self.normal_scale
        P.tangent_stiffness = self.tangent_stiffness
        P.friction_static = cfg.friction_static
        P.friction_dynamic = cfg.friction_dynamic
        P.tangent_damping = cfg.tangent_damping
        P.board_scale = self.board_scale
        P.board_half[0], P.board_half[1] = cfg.board_half_extent
        for i in range(3):
            P.half[i] = cfg.blade_half_size[i]
            P.inertia_inv[i] = float(np.float32(self.inertia_inv[i]))
            P.half_d[i] = float(np.float32(cfg.blade_half_size[i]))
            P.inertia_inv_d[i] = float(np.float32(self.inertia_inv[i]))
        P.bevel = cfg.blade_bevel_height
        P.blade_offset = self.blade_offset
        P.blade_mass = cfg.blade_mass
        P.threshold = self.threshold
        P.pair_skin = self.pair_skin
        # float64 tool constants start from the float32 values the reference stores
        f = lambda v: float(np.float32(v))  # noqa: E731
        P.dt_d = f(cfg.dt)
        P.blade_mass_d = f(cfg.blade_mass)
        P.bevel_d = f(cfg.blade_bevel_height)
        P.drive_stiffness = f(cfg.drive_stiffness)
        P.drive_damping = f(cfg.drive_damping)
        P.drive_force_limit = f(cfg.drive_force_limit)
        P.rot_stiffness = f(cfg.rotational_stiffness)
        P.rot_damping = f(cfg.rotational_damping)
        P.friction_dynamic_d = f(cfg.friction_dynamic)
        P.board_half_d[0], P.board_half_d[1] = f(cfg.board_half_extent[0]), f(cfg.board_half_extent[1])
        return P

    def _bind(self):
        B = _native.Buffers()
        for name, _ in _native.Buffers._fields_:
            setattr(B, name, self._t[name].data_ptr())
        self._buffers = B
        handle = ctypes.c_void_p()
        _native.check(self._lib.bm_solver_create(ctypes.byref(self._params), ctypes.byref(B), ctypes.byref(handle)))
        if self._handle is not None:
            self._lib.bm_solver_destroy(self._handle)
        self._handle = handle

    def _rebind(self):
        """New parameters: rebind the solver and drop captured graphs."""
        self._params = self._make_params()
        self._drop_graphs()
        self._bind()

    def _drop_graphs(self):
        for entry in getattr(self, "_batches", {}).values():
            self._lib.bm_graph_destroy(entry)
        self._batches = {}

    def __del__(self):
        try:
            self._drop_graphs()
            if self._handle is not None:
                self._lib.bm_solver_destroy(self._handle)
        except Exception:
            pass

    @property
    def _stream(self):
        import torch

        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _call(self, fn, *args):
        _native.check(getattr(self._lib, fn)(self._handle, *args))

    def _sync_step(self):
        """Make the device's substep counter (friction-history parity) equal step_count.

        Every substep launch advances the device counter and step_count
        together, so this writes only when something else moved one of them.
        """
        if self._device_step != self.step_count:
            self._flag("STEP", self.step_count)
            self._device_step = self.step_count

    def _advanced(self, substeps):
        self.step_count += substeps
        self._device_step += substeps

    def _flag(self, name, value=None):
        idx = _native.FLAG[name]
        if value is None:
            return int(self._t["flags"][idx].item())
        self._t["flags"][idx] = value

    # --------------------------------------------------------------- views

    def _views(self):
        import torch

        T, n, K = self._t, self.n, self.config.tool_count
        o, r = self._order_t, self._rank_t

        def dirty_pairs():
            T["flags"][_native.FLAG["PAIR_DIRTY"]] = 1

        def dirty_all():
            T["flags"][_native.FLAG["PAIR_DIRTY"]] = 1
            T["flags"][_native.FLAG["TOPOLOGY_DIRTY"]] = 1
            T["flags"][_native.FLAG["HOST_DIRTY"]] = 1

        def dirty_topology():
            T["flags"][_native.FLAG["HOST_DIRTY"]] = 1

        self.x = particle_view(T["x"], o, r, (3,), np.float32, "x", dirty_pairs)
        self.v = particle_view(T["v"], o, r, (3,), np.float32, "v", dirty_pairs)
        self.ref = particle_view(T["ref"], o, r, (3,), np.float32, "ref", dirty_pairs)
        self.F = particle_view(T["F"], o, r, (3, 3), np.float32, "F")
        self.Fp = particle_view(T["Fp"], o, r, (3, 3), np.float32, "Fp", self._fp_written)
        self.stress = particle_view(T["stress"], o, r, (3, 3), np.float32, "stress")
        if self.maxwell:
            self.viscous = particle_view(T["viscous"], o, r, (3, 3), np.float64, "viscous")
        self.codes = particle_view(T["codes"], o, r, None, np.int64, "codes", dirty_all)
        self.single_field_codes = particle_view(T["zero_codes"], o, r, None, np.int64, "single_field_codes")
        self.tool_damage = [
            particle_view(T["damage"][k], o, r, None, np.float32, f"damage[{k}]") for k in range(K)
        ]
        self.damage = self.tool_damage[0]
        self.impulses = particle_view(T["impulses"], o, r, (3,), np.float32, "impulses")
        def histories_written():
            T["hist_mask"].fill_(-1)

        self.histories = particle_view(T["histories"][:2], o, r, (3,), np.float32, "histories", histories_written, leading=2)
        if K > 1:
            self.extra_histories = particle_view(
                T["histories"][1:], o, r, (3,), np.float32, "extra_histories", histories_written, leading=K
            )
        else:
            self.extra_histories = None
        self.mobility_view = None
        self.tool_mobility = plain_view(T["mobility"], (6, 6), np.float32, "tool_mobility")
        self.errors = plain_view(T["errors"], (3,), np.int32, "errors")
        self.speed = plain_view(T["speed"], (1,), np.float32, "speed")
        flags = T["flags"]
        # a host write of the flag asks for a full registration (HOST_DIRTY); the device's side
        # labelling sets it alone and registers only the nodes around the relabelled particles
        self.topology_dirty = plain_view(flags[_native.FLAG["TOPOLOGY_DIRTY"] : _native.FLAG["TOPOLOGY_DIRTY"] + 1], (1,), np.int32, "topology_dirty", dirty_topology)
        self.pair_list_dirty = plain_view(flags[_native.FLAG["PAIR_DIRTY"] : _native.FLAG["PAIR_DIRTY"] + 1], (1,), np.int32, "pair_list_dirty")
        self.pair_list_builds = plain_view(flags[_native.FLAG["PAIR_BUILDS"] : _native.FLAG["PAIR_BUILDS"] + 1], (1,), np.int32, "pair_list_builds")
        self.pair_count = [plain_view(T["pair_count"][i : i + 1], (1,), np.int32, f"pair_count[{i}]") for i in range(2)]
        self.pair_keys = [plain_view(T["pair_keys"][i], (self.pair_capacity,), np.int64, f"pair_keys[{i}]") for i in range(2)]
        self.pair_used = [plain_view(T["pair_used"][i], (self.pair_capacity,), np.int32, f"pair_used[{i}]") for i in range(2)]
        S = self.grid_capacity
        self.grid_mass = plain_view(T["grid_mass"], (S,), np.float32, "grid_mass")
        for name in ("momentum", "grid_impulse", "old_v", "new_v", "remapped"):
            setattr(self, name, soa_view(T[name], S, name))
        self.coupled_remapped = DeviceArray(
            (S, 3), np.float32, lambda: (T["remap_v"].t() * T["grid_mass"][:, None]).cpu().numpy(), None, None, "coupled_remapped"
        )
        self.tool_pos = self._tool_view(0, 3, "tool_pos")
        self.tool_vel = self._tool_view(3, 3, "tool_vel")
        self.tool_rot = self._tool_view(6, 4, "tool_rot")
        self.tool_omega = self._tool_view(10, 3, "tool_omega")
        self.tool_table_impulse = DeviceArray((K, 3), np.float32, lambda: T["table_impulse"].cpu().numpy(), None, None, "tool_table_impulse")
        self.reaction = self._acc_view("reaction")
        self.torque = self._acc_view("torque")
        self.board = self._acc_view("board")
        self.work = self._acc_view("work")
        self.interval_impulse = DeviceArray(
            (1, 3), np.float32, lambda: T["interval"][:3].cpu().numpy(), lambda a: T["interval"][:3].copy_(torch.as_tensor(a.reshape(3), dtype=torch.float64)), None, "interval_impulse"
        )
        self.interval_angular_impulse = DeviceArray(
            (1, 3), np.float32, lambda: T["interval"][3:].cpu().numpy(), lambda a: T["interval"][3:].copy_(torch.as_tensor(a.reshape(3), dtype=torch.float64)), None, "interval_angular_impulse"
        )
        self.weights = DeviceArray((n, 8), np.float32, lambda: T["stencil_w"][T["stencil_id"].long()].index_select(0, r).cpu().numpy(), None, None, "weights")
        self.gradients = DeviceArray((n, 8, 3), np.float32, lambda: T["stencil_g"][T["stencil_id"].long()].index_select(0, r).cpu().numpy(), None, None, "gradients")
        self.nodes = DeviceArray((n, 8), np.int32, lambda: self.node_numpy.astype(np.int32), None, None, "nodes")
        self.slots = DeviceArray((n, 8), np.int32, self._read_slots, None, None, "slots")
        self.keys = DeviceArray((S,), np.int64, self._read_keys, None, None, "keys")
        self.grid_keys = DeviceArray((S,), np.int64, self._read_grid_keys, None, None, "grid_keys")
        self.active_count = DeviceArray((1,), np.int32, lambda: np.array([int((self._read_keys() >= 0).sum())]), None, None, "active_count")
        self.ref_numpy = self.reference.astype(np.float32)

    def _fp_written(self):
        if not self._use_fp:
            self._use_fp = True
            self._rebind()

    def _tool_view(self, first, width, name):
        import torch

        T = self._t

        def read():
            return T["tool"][:, first : first + width].cpu().numpy()

        def write(value):
            T["tool"][:, first : first + width] = torch.as_tensor(value.astype(np.float32).astype(np.float64), device=self.device)
            self._call("bm_sync_tool_mirror", self._stream)

        return DeviceArray((self.config.tool_count, width), np.float32, read, write, None, name)

    def _acc_view(self, kind):
        import torch

        K = self.config.tool_count
        shape = {"reaction": (K, 3), "torque": (K, 3), "board": (1, 3), "work": (1,)}[kind]

        def read():
            out = torch.zeros(int(np.prod(shape)), dtype=torch.float32, device=self.device)
            args = [None, None, None, None]
            args[["reaction", "torque", "board", "work"].index(kind)] = out.data_ptr()
            self._call("bm_read_accumulators", *[ctypes.c_void_p(a) for a in args], self._stream)
            return out.cpu().numpy()

        def write(value):
            t = torch.as_tensor(np.ascontiguousarray(value, dtype=np.float32).reshape(-1), device=self.device)
            args = [None, None, None, None]
            args[["reaction", "torque", "board", "work"].index(kind)] = t.data_ptr()
            self._call("bm_write_accumulators", *[ctypes.c_void_p(a) for a in args], self._stream)
            torch.cuda.current_stream(self.device).synchronize()

        return DeviceArray(shape, np.float32, read, write, None, kind)

    def _read_slots(self):
        import torch

        T = self._t
        fidx = T["fidx"]
        offsets = torch.as_tensor(
            [int(np.ravel_multi_index(tuple(o), tuple(self.node_dims))) for o in OFFSETS], device=self.device
        )
        shifts = torch.arange(8, device=self.device) * 8
        field = (fidx[:, None] >> shifts[None]) & 0xFF
        slot = field * self.node_count + T["base_node"].long()[:, None] + offsets[None]
        return slot.index_select(0, self._rank_t).to(torch.int32).cpu().numpy()

    def _read_keys(self):
        import torch

        T = self._t
        f = torch.arange(self.fmax, device=self.device)[:, None]
        used = f < T["nfield"][None].long()
        node = torch.arange(self.node_count, device=self.device)[None]
        keys = torch.where(used, T["fcode"] * self.node_count + node, torch.full_like(T["fcode"], -1))
        return keys.reshape(-1).cpu().numpy()

    def _read_grid_keys(self):
        keys = self._read_keys()
        packed = np.sort(keys[keys >= 0])
        out = np.full(self.grid_capacity, -1, np.int64)
        out[: len(packed)] = packed
        return out

    # ------------------------------------------------------------- physics

    def refresh_stress(self):
        """Recompute the stored stress; needed after writing F, Fp or viscous from the host."""
        self._call("bm_refresh_stress", self._stream)

    def material_step(self):
        self._call("bm_material_step", int(self.single_field), self._stream)

    @property
    def single_field(self):
        return self.field_codes is self.single_field_codes

    def set_single_field(self, enabled):
        """Baseline of paper Fig. 4: particle-grid transfers ignore cut-side codes."""
        if bool(enabled) != self.single_field:
            self.field_codes = self.single_field_codes if enabled else self.codes
            self.topology_dirty.fill_(1)

    def _register_topology(self):
        self._call("bm_register_topology", int(self.single_field), self._stream)

    def step(self, target_edge=(0.0, 0.0, 0.042), cutting=True, cut_index=0, orientation=None):
        if self.config.external_tool:
            raise ValueError("Use ExternalToolPort.advance for an externally owned tool")
        cut_index = self._set_cut(cut_index)
        self._step_kernels(target_edge, cutting, cut_index, orientation=orientation)

    def _set_cut(self, cut_index):
        if isinstance(cut_index, (bool, np.bool_)) or not isinstance(cut_index, (int, np.integer)):
            raise ValueError("Cut index must be an integer")
        cut_index = int(cut_index)
        last = self.max_cut_index - (self.config.tool_count - 1)
        if cut_index < self.cut_index or cut_index > last:
            raise ValueError(f"Cut indices must be monotonic and within [0, {last}]")
        if cut_index != self.cut_index:
            for damage in self.tool_damage:
                damage.zero_()
            self.cut_index = cut_index
        return cut_index

    def _tool_model(self):
        cfg = self.config
        if cfg.external_tool:
            return -1
        return int(cfg.free_blade or cfg.pose_servo)

    def _cut_bits(self, cutting):
        if not cutting:
            return 0
        cfg = self.config
        return CUT_ON | (CUT_ADVANCE if cfg.cut_work == "advance" else 0) | (CUT_HOLD if cfg.cut_hold else 0)

    def rigid_contacts(self, cutting=True):
        """Gravity plus board and blade contact impulses on every particle."""
        self._call("bm_rigid_contacts", self._cut_bits(cutting), self._stream)

    def particle_contacts(self):
        """Contacts between particles on incompatible sides of a cut, with friction history."""
        self._sync_step()
        self._call("bm_particle_contacts", self._stream)

    def assign_sides(self, cut_index, cutting=True):
        self._call("bm_assign_sides", int(cut_index), int(bool(cutting)), self._stream)

    def _write_targets(self, targets, orientations):
        import torch

        k = len(targets)
        self._t["targets"][:k] = torch.as_tensor(np.asarray(targets, np.float32).reshape(k, 3), device=self.device)
        self._t["rotations"][:k] = torch.as_tensor(np.asarray(orientations, np.float32).reshape(k, 4), device=self.device)

    def _drive_tool(self, target_edge, orientation, buffer=None, rotations=None, index=0):
        """Pose servo, free rigid blade, or guided translation; all share the knife/board contact."""
        self._write_targets([target_edge], [orientation if orientation is not None else [0.0, 0.0, 0.0, 1.0]])
        self._call("bm_drive_tool", 0, self._stream)

    def components(self, codes=None):
        """Piece label of every particle and the piece sizes, computed on the device.

        topology.components (topology.py:17-57) of node_numpy, weight_numpy and
        ``codes`` ((n,) in reference order; default the current cut codes): the
        labels rank the pieces by their lowest particle index.  Returns int64
        (labels (n,), sizes (pieces,)) like the reference.
        """
        import torch

        n = self.n
        if getattr(self, "_pieces", None) is None:
            self._pieces = [torch.zeros(n, dtype=torch.int32, device=self.device) for _ in range(2)]
            self._pieces.append(torch.zeros(1, dtype=torch.int32, device=self.device))
        labels, sizes, count = self._pieces
        code_ptr = None
        if codes is not None:
            codes = np.asarray(codes, np.int64)
            if codes.shape != (n,):
                raise ValueError(f"codes must have shape ({n},)")
            device_codes = torch.as_tensor(codes, device=self.device).index_select(0, self._order_t)
            code_ptr = device_codes.data_ptr()
        self._call("bm_components", code_ptr, self._order_t.data_ptr(), labels.data_ptr(), sizes.data_ptr(),
                   count.data_ptr(), self._stream)
        pieces = int(count.item())
        if pieces < 0:
            raise RuntimeError("Piece labelling gave up (union retries exhausted)")
        return labels.cpu().numpy().astype(np.int64), sizes[:pieces].cpu().numpy().astype(np.int64)

    def embedded_particles(self):
        """Number of particles beside the blade body; zero once the blade has left the material."""
        self._call("bm_count_embedded", 1, self._stream)
        return self._flag("EMBEDDED")

    def embedded_particles_previous(self):
        """`embedded_particles` of the previous call (this call's count is read at the next)."""
        previous = getattr(self, "_embedded_previous", 0)
        self._embedded_previous = self.embedded_particles()
        return previous

    def _step_args(self, steps, cutting, cut_index, use_targets=1, **extra):
        a = _native.StepArgs()
        a.steps = steps
        a.cut_bits = self._cut_bits(cutting)
        a.cut_index = cut_index
        a.single_field = int(self.single_field)
        a.use_targets = use_targets
        for k, v in extra.items():
            setattr(a, k, int(v))
        return a

    def _step_kernels(self, target_edge, cutting, cut_index, buffer=None, index=0, rotations=None, orientation=None):
        """One substep: contacts, material update, tool update, side labels."""
        self._sync_step()
        self._write_targets([target_edge], [orientation if orientation is not None else [0.0, 0.0, 0.0, 1.0]])
        args = self._step_args(1, cutting, cut_index, use_targets=0)
        _native.check(self._lib.bm_substeps(self._handle, ctypes.byref(args), self._stream))
        self._advanced(1)

    def advance(self, targets, cutting=True, cut_index=0, graph=True, orientations=None):
        """Submit exact per-substep targets, including every intermediate contact (solver.py:942-973)."""
        if self.config.external_tool:
            raise ValueError("Use ExternalToolPort.advance for an externally owned tool")
        targets = np.ascontiguousarray(targets, dtype=np.float32)
        if targets.ndim != 2 or targets.shape[1] != 3 or not np.isfinite(targets).all() or not len(targets):
            raise ValueError("targets must be finite (substeps, 3) edge positions")
        orientations = np.tile([0.0, 0.0, 0.0, 1.0], (len(targets), 1)) if orientations is None else np.asarray(orientations)
        if orientations.shape != (len(targets), 4) or not np.isfinite(orientations).all():
            raise ValueError("orientations must be finite (substeps, 4) xyzw quaternions")
        lengths = np.linalg.norm(orientations, axis=1)
        if np.any(lengths < 1.0e-6):
            raise ValueError("Zero quaternion")
        orientations = np.ascontiguousarray(orientations / lengths[:, None], dtype=np.float32)
        cut_index = self._set_cut(cut_index)
        if not graph:
            for target, orientation in zip(targets, orientations):
                self._step_kernels(target, cutting, cut_index, orientation=orientation)
            return
        for start in range(0, len(targets), MAX_BATCH):
            chunk = slice(start, start + MAX_BATCH)
            self._sync_step()
            graph_handle = self.prepare(targets[chunk], cutting, cut_index, orientations[chunk])
            self._write_targets(targets[chunk], orientations[chunk])
            _native.check(self._lib.bm_graph_launch(graph_handle, self._stream))
            self._advanced(len(targets[chunk]))

    def prepare(self, targets, cutting=True, cut_index=0, orientations=None, tag=None, **extra):
        """Capture one batch of substeps as a CUDA graph, cached by its shape (solver.py:975-1019)."""
        steps = len(targets)
        key = (steps, bool(cutting), int(cut_index), self.single_field, tag, tuple(sorted(extra.items())))
        if key not in self._batches:
            start = time.perf_counter()
            args = self._step_args(steps, cutting, cut_index, **extra)
            handle = ctypes.c_void_p()
            _native.check(self._lib.bm_graph_create(self._handle, ctypes.byref(args), self._stream, ctypes.byref(handle)))
            self._batches[key] = handle
            self.graph_build_s += time.perf_counter() - start
        return self._batches[key]

    def state(self):
        errors = self.errors.numpy()
        if errors.any():
            raise RuntimeError(
                f"GPU errors [storage overflow, inverted material, coincident proxies]: {errors.tolist()}"
            )
        state = {
            k: getattr(self, a).numpy()
            for k, a in [
                ("position", "x"),
                ("velocity", "v"),
                ("deformation", "F"),
                ("plastic_deformation", "Fp"),
                ("sides", "codes"),
                ("damage", "damage"),
                ("blade_position", "tool_pos"),
                ("blade_velocity", "tool_vel"),
                ("blade_orientation", "tool_rot"),
                ("blade_omega", "tool_omega"),
            ]
        }
        if self.maxwell:
            state["viscous_deformation"] = np.eye(3) + self.viscous.numpy()
        if self.config.tool_count > 1:
            state["tool_damage"] = np.stack([damage.numpy() for damage in self.tool_damage])
        state["time"] = self.step_count * self.config.dt
        if any(not np.isfinite(v).all() for v in state.values()):
            raise RuntimeError("Nonfinite state; run is invalid")
        if np.linalg.det(state["deformation"]).min() <= 0:
            raise RuntimeError("Inverted material; run is invalid")
        return state

    def checkpoint(self):
        """A device-side copy of the whole solver state (no counterpart in the reference).

        Unlike ``state()``, which returns the reference's host dictionary, this
        keeps everything a later substep reads: particle and grid arrays, cut
        fields, pair lists, friction-history tables, knife state, accumulators
        and counters.  ``restore`` of it makes the following substeps repeat
        the ones that followed the checkpoint bit for bit.
        """
        import torch

        with torch.cuda.device(self.device):
            arrays = {name: t.clone() for name, t in self._t.items()}
        return {"arrays": arrays, "step_count": self.step_count, "device_step": self._device_step,
                "cut_index": self.cut_index, "single_field": self.single_field}

    def restore(self, checkpoint):
        """Copy a ``checkpoint()`` back in place (addresses, and so captured graphs, stay valid)."""
        for name, saved in checkpoint["arrays"].items():
            self._t[name].copy_(saved)
        self.step_count = checkpoint["step_count"]
        self._device_step = checkpoint["device_step"]
        self.cut_index = checkpoint["cut_index"]
        self.field_codes = self.single_field_codes if checkpoint["single_field"] else self.codes

    def synchronize(self):
        import torch

        torch.cuda.synchronize(self.device)
