"""CPU ORACLE wrapper - test infrastructure, not part of the product.

Loads oracle/oracle.c (built here with gcc -ffp-contract=off -fopenmp) and
drives it like the reference's Solver (blademaster_warp/solver.py), so tests
can run the same scene on the GPU product and on this restatement and
compare.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg use it.

Setup shared with the product: particle sampling and stencils come from
``blademaster_gb300.geometry`` (pinned bit-exactly against the reference's
geometry.points / stencil by tests/test_geometry.py), and the parameter
struct layout from include/blademaster_gb300.h.  The solver constants
(mass, Lame parameters, damage threshold, inertia, capacities) are derived
here again from solver.py:164-200, independently of the product.
"""

import ctypes
import os
import subprocess
import sys
import threading
from dataclasses import asdict
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT / "blademaster-lab_gb300"))

from blademaster_gb300 import _native  # noqa: E402  (header-driven struct layout only)
from blademaster_gb300.geometry import points, stencil, cell_sort  # noqa: E402

HERE = Path(__file__).resolve().parent
SOURCE = HERE / "oracle.c"
LIBRARY = HERE / "_build" / "liboracle.so"
# The same restatement built in float64 (-DORC_REAL64): the error reference of scene-level results.
LIBRARY64 = HERE / "_build" / "liboracle64.so"
_lock = threading.Lock()
_lib = None
_lib64 = None


def build(force=False, real64=False):
    """Compile the oracle (portable flags: it runs on x86_64 and aarch64); real64 builds the float64 one."""
    target = LIBRARY64 if real64 else LIBRARY
    with _lock:
        deps = [SOURCE, ROOT / "blademaster-lab_gb300" / "csrc" / "bm_scalar.h", ROOT / "include" / "blademaster_gb300.h"]
        if not force and target.exists() and all(d.stat().st_mtime <= target.stat().st_mtime for d in deps):
            return target
        target.parent.mkdir(exist_ok=True)
        tmp = target.with_suffix(".tmp.so")
        cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
               *(["-DORC_REAL64", "-Werror=incompatible-pointer-types"] if real64 else []),
               str(SOURCE), "-o", str(tmp), "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stderr)
        os.replace(tmp, target)
        return target


P = ctypes.c_void_p
_STATE_FIELDS = [
    "x", "v", "ref", "F", "Fp", "stress", "viscous", "codes", "damage", "histories", "impulses", "nodes",
    "weights", "gradients", "keys", "slots", "node_start", "node_slots", "slot_start", "contrib", "grid_mass",
    "momentum", "grid_impulse", "old_v", "new_v", "remapped", "coupled", "pair_keys", "pair_history", "pair_used",
    "pair_count", "cell_head", "cell_start", "cell_next", "tool", "mobility", "acc", "interval", "table_impulse", "speed",
    "errors", "flags", "result", "hold_side",
]


class State(ctypes.Structure):
    _fields_ = [(name, P) for name in _STATE_FIELDS] + [("capacity", ctypes.c_int64), ("buckets", ctypes.c_int64)]


def lib(real64=False):
    """The float32 oracle, or with real64 the float64 build (whose float arguments are doubles)."""
    global _lib, _lib64
    if real64:
        if _lib64 is None:
            build(real64=True)
            L = ctypes.CDLL(str(LIBRARY64))
            if L.orc_state_size() != ctypes.sizeof(State):
                raise RuntimeError("oracle state layout mismatch")
            pp, ps, vp, i = ctypes.POINTER(_native.Params), ctypes.POINTER(State), ctypes.c_void_p, ctypes.c_int
            for name, args in {"orc_register": [pp, ps, vp], "orc_refresh_stress": [pp, ps],
                               "orc_load_external": [pp, ps, vp], "orc_validate_interval": [pp, ps],
                               "orc_substep": [pp, ps, i, i, vp, i, vp, vp]}.items():
                getattr(L, name).argtypes = args
                getattr(L, name).restype = None
            L.orc_count_embedded.argtypes = [pp, ps]
            L.orc_count_embedded.restype = ctypes.c_int64
            L.orc_num_threads.restype = ctypes.c_int
            _lib64 = L
        return _lib64
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIBRARY))
        if L.orc_state_size() != ctypes.sizeof(State):
            raise RuntimeError("oracle state layout mismatch")
        pp, ps, vp, i, f = ctypes.POINTER(_native.Params), ctypes.POINTER(State), ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        sig = {
            "orc_register": [pp, ps, vp],
            "orc_refresh_stress": [pp, ps],
            "orc_plastic_project": [pp, ps, f],
            "orc_material_step": [pp, ps, vp, i],
            "orc_rigid_contacts": [pp, ps, i],
            "orc_particle_contacts": [pp, ps],
            "orc_assign": [pp, ps, i, i],
            "orc_drive_one": [pp, ps, i, vp, vp],
            "orc_accumulate_tool_impulses": [pp, ps],
            "orc_finish_external": [pp, ps],
            "orc_clear_step": [pp, ps],
            "orc_load_external": [pp, ps, vp],
            "orc_validate_interval": [pp, ps],
            "orc_hold_solve": [pp, ps],
            "orc_substep": [pp, ps, i, i, vp, i, vp, vp],
            "orc_friction": [vp, vp, vp, vp, i, f, f, f, f, f, f, vp, vp],
            "orc_blade_query": [vp, i, vp, f, vp, vp, vp],
            "orc_resist_cut": [vp, vp, vp, vp, vp, vp, vp, vp, f, f, vp, f, i, vp, vp, i],
        }
        for name, args in sig.items():
            getattr(L, name).argtypes = args
            getattr(L, name).restype = None
        L.orc_couple_fields.argtypes = [vp, vp, vp, vp, i, vp]
        L.orc_g2p.argtypes = [vp, vp, vp, vp, vp, vp, i, f, f]
        L.orc_math_f.argtypes = [vp, i, vp, vp]
        L.orc_math_d.argtypes = [vp, vp, i, vp, vp, vp]
        L.orc_svd.argtypes = [vp, i, vp, vp, vp, vp]
        L.orc_fx_roundtrip.argtypes = [vp, i, vp]
        L.orc_metrics.argtypes = [vp, vp, vp, vp, i, f, f, f, f, vp]
        for name in ("orc_couple_fields", "orc_g2p", "orc_math_f", "orc_math_d", "orc_svd", "orc_fx_roundtrip",
                     "orc_metrics"):
            getattr(L, name).restype = None
        L.orc_maxwell_hold.argtypes = [pp, ps, i]
        L.orc_maxwell_hold.restype = None
        L.orc_count_embedded.argtypes = [pp, ps]
        L.orc_count_embedded.restype = ctypes.c_int64
        L.orc_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def ptr(a):
    """Address of a C-contiguous array's data (the caller keeps the array alive across the call)."""
    if not a.flags.c_contiguous:
        raise ValueError("oracle arrays must be C-contiguous")
    return ctypes.c_void_p(a.ctypes.data)


def fx_to_float(lo, hi):
    v = (int(np.uint64(hi)) << 64) | int(np.uint64(lo))
    if v >= 1 << 127:
        v -= 1 << 128
    return v / 2.0**96


def _pow2_at_least(v):
    return 1 << (max(int(v), 1) - 1).bit_length()


class OracleSolver:
    """The reference's Solver restated on the CPU (device particle order, AoS arrays).

    real=np.float64 runs the float64 build of the same restatement (every float32 array and
    operation in double, the parameters the float32 values): the error reference that the
    float32 results (bit-exact with the GPU) are measured against.  Only the scene-stepping
    methods (step, advance, external_interval, get, set) are available there."""

    def __init__(self, config, real=np.float32):
        cfg = self.config = config
        self.R = R = np.dtype(real).type
        if R not in (np.float32, np.float64):
            raise ValueError("real must be float32 or float64")
        self.L = lib(R is np.float64)
        self.reference, self.origin, cells = points(cfg.size, cfg.grid_spacing, cfg.shape, cfg.sampling_seed)
        n = self.n = len(self.reference)
        nodes, w, g = stencil(self.reference, self.origin, cfg.grid_spacing, cells)
        order, cell_start = cell_sort(self.reference, self.origin, cfg.grid_spacing, cells)
        self.order = order
        self.rank = np.empty(n, np.int64)
        self.rank[order] = np.arange(n)
        self.node_count = int(np.prod(cells + 1))
        self.node_numpy, self.weight_numpy = nodes, w
        # solver.py:181-200
        volume = (cfg.grid_spacing / 2) ** 3
        mass = cfg.density * volume
        radius = cfg.grid_spacing / 4
        blade_offset = max(cfg.blade_contact_radius or radius, radius - cfg.blade_half_size[0])
        mu = cfg.young_modulus / (2 * (1 + cfg.poisson_ratio))
        lam = cfg.young_modulus * cfg.poisson_ratio / ((1 + cfg.poisson_ratio) * (1 - 2 * cfg.poisson_ratio))
        maxwell = cfg.maxwell_tau > 0 and cfg.maxwell_fraction > 0
        threshold = cfg.cutting_energy * volume ** (2 / 3) * (1 - cfg.sharpness) / cfg.sharpness
        ratio = 1.0 if cfg.contact_reference_dt == 0 else (cfg.dt / cfg.contact_reference_dt) ** 2
        sn, gk = cfg.normal_scale * ratio, cfg.tangent_stiffness * ratio
        hx, hy, hz = cfg.blade_half_size
        inertia_inv = 3 / (cfg.blade_mass * np.array([hy * hy + hz * hz, hx * hx + hz * hz, hx * hx + hy * hy]))
        self.mass, self.volume, self.radius, self.mu, self.lam = mass, volume, radius, mu, lam
        K = cfg.tool_count
        pair_list = cfg.pair_search in ("list", "auto")
        p = _native.Params()
        p.n, p.node_count, p.tool_count = n, self.node_count, K
        for i in range(3):
            p.node_dims[i], p.cell_dims[i] = int(cells[i] + 1), int(cells[i])
        p.pair_capacity = _pow2_at_least(max(64 * n, 16))
        p.tool_model = -1 if cfg.external_tool else int(cfg.free_blade or cfg.pose_servo)
        p.external_tool = int(cfg.external_tool)
        p.predict = int(cfg.tool_substep == "predict")
        p.free_blade = int(cfg.free_blade)
        p.lock_rotation = int(not (cfg.free_blade or cfg.pose_servo))
        p.accumulate_tool_impulses = int(cfg.accumulate_tool_impulses)
        p.plastic = int(cfg.yield_stress > 0)
        p.use_fp = int(cfg.yield_stress > 0 or maxwell)
        p.maxwell = int(maxwell)
        p.viscous = int(cfg.dynamic_viscosity > 0)
        p.pair_search = 0 if pair_list else 1
        p.cache_topology = int(cfg.cache_topology)
        p.dt, p.spacing, p.mass, p.volume, p.radius, p.mu, p.lam = cfg.dt, cfg.grid_spacing, mass, volume, radius, mu, lam
        p.mu_maxwell = cfg.maxwell_fraction * mu
        p.maxwell_relax = float(-np.expm1(-cfg.dt / cfg.maxwell_tau)) if maxwell else 0.0
        p.yield_stress, p.flip, p.dynamic_viscosity = cfg.yield_stress, cfg.flip_fraction, cfg.dynamic_viscosity
        p.normal_scale, p.tangent_stiffness = sn, gk
        p.friction_static, p.friction_dynamic, p.tangent_damping = cfg.friction_static, cfg.friction_dynamic, cfg.tangent_damping
        p.board_scale = cfg.board_normal_scale or sn
        p.board_half[0], p.board_half[1] = cfg.board_half_extent
        f32 = lambda v: float(np.float32(v))  # noqa: E731
        for i in range(3):
            p.half[i] = cfg.blade_half_size[i]
            p.inertia_inv[i] = f32(inertia_inv[i])
            p.half_d[i] = f32(cfg.blade_half_size[i])
            p.inertia_inv_d[i] = f32(inertia_inv[i])
        p.bevel, p.blade_offset, p.blade_mass, p.threshold = cfg.blade_bevel_height, blade_offset, cfg.blade_mass, threshold
        p.pair_skin = (cfg.pair_skin or radius) if pair_list else 0.0
        p.dt_d, p.blade_mass_d, p.bevel_d = f32(cfg.dt), f32(cfg.blade_mass), f32(cfg.blade_bevel_height)
        p.drive_stiffness, p.drive_damping = f32(cfg.drive_stiffness), f32(cfg.drive_damping)
        p.drive_force_limit = f32(cfg.drive_force_limit)
        p.rot_stiffness, p.rot_damping = f32(cfg.rotational_stiffness), f32(cfg.rotational_damping)
        p.friction_dynamic_d = f32(cfg.friction_dynamic)
        p.board_half_d[0], p.board_half_d[1] = f32(cfg.board_half_extent[0]), f32(cfg.board_half_extent[1])
        self.params = p
        cap = _pow2_at_least(max(16 * n, 16))
        A = self.arrays = {}
        A["x"] = np.ascontiguousarray(self.reference[order], R)
        A["v"] = np.zeros((n, 3), R)
        A["ref"] = A["x"].copy()
        A["F"] = np.tile(np.eye(3, dtype=R).reshape(9), (n, 1))
        A["Fp"] = A["F"].copy()
        A["stress"] = np.zeros((n, 9), R)
        A["viscous"] = np.zeros((n, 9), np.float64)
        A["codes"] = np.zeros(n, np.int64)
        A["zero_codes"] = np.zeros(n, np.int64)
        A["damage"] = np.zeros((K, n), R)
        A["histories"] = np.zeros((1 + K, n, 3), R)
        A["impulses"] = np.zeros((n, 3), R)
        A["nodes"] = np.ascontiguousarray(nodes[order], np.int32)
        A["weights"] = np.ascontiguousarray(w[order], R)
        A["gradients"] = np.ascontiguousarray(g[order], R)
        A["keys"] = np.full(cap, -1, np.int64)
        A["slots"] = np.zeros((n, 8), np.int32)
        A["node_start"] = np.zeros(self.node_count + 1, np.int32)
        A["node_slots"] = np.zeros(cap, np.int32)
        A["slot_start"] = np.zeros(cap + 1, np.int32)
        A["contrib"] = np.zeros(8 * n, np.int32)
        A["grid_mass"] = np.zeros(cap, R)
        for k in ("momentum", "grid_impulse", "old_v", "new_v", "remapped", "coupled"):
            A[k] = np.zeros((cap, 3), R)
        A["pair_keys"] = np.full((2, p.pair_capacity), -1, np.int64)
        A["pair_history"] = np.zeros((2, p.pair_capacity, 3), R)
        A["pair_used"] = np.zeros((2, p.pair_capacity), np.int32)
        A["pair_count"] = np.zeros(2, np.int32)
        buckets = _pow2_at_least(max(2 * n, 1024))
        A["cell_head"] = np.zeros(buckets, np.int32)
        A["cell_next"] = np.zeros(n, np.int32)
        A["cell_start"] = cell_start.astype(np.int32)
        tool = np.zeros((K, 13))
        tool[:, 2] = R(cfg.size[2] + 0.012 + hz)
        tool[:, 9] = 1.0
        A["tool"] = tool
        A["mobility"] = np.zeros(36, R)
        A["acc"] = np.zeros(_native.ACC_WORDS, np.uint64)
        A["interval"] = np.zeros(6)
        A["table_impulse"] = np.zeros((K, 3))
        A["speed"] = np.zeros(1, R)
        A["errors"] = np.zeros(3, np.int32)
        A["flags"] = np.zeros(_native.FLAG["WORDS"], np.int32)
        A["flags"][_native.FLAG["TOPOLOGY_DIRTY"]] = 1
        A["result"] = np.zeros(10 + 7 * 4097, R)
        A["hold_side"] = np.zeros(n, R)
        s = State()
        for name in _STATE_FIELDS:
            setattr(s, name, A[name].ctypes.data)
        s.capacity, s.buckets = cap, buckets
        self.S = s
        self.single_field = False
        self.step_count = 0
        self.cut_index = 0
        self.refresh_stress()

    # ------------------------------------------------------------- access

    def get(self, name):
        """Array in reference particle order (particle arrays) or as stored."""
        A = self.arrays
        if name in ("x", "v", "ref", "impulses"):
            return A[name][self.rank]
        if name in ("F", "Fp", "stress"):
            return A[name][self.rank].reshape(-1, 3, 3)
        if name == "hold_side":
            return A["hold_side"][self.rank]
        if name in ("codes", "damage"):
            return A[name][self.rank] if name == "codes" else A["damage"][0][self.rank]
        if name == "tool_damage":
            return A["damage"][:, self.rank]
        if name == "histories":
            return A["histories"][:2][:, self.rank]
        if name in ("reaction", "torque"):
            base = 0 if name == "reaction" else 2 * 3 * _native.MAX_TOOLS
            acc = A["acc"]
            return np.array(
                [[fx_to_float(acc[base + 6 * k + 2 * i], acc[base + 6 * k + 2 * i + 1]) for i in range(3)]
                 for k in range(self.config.tool_count)]
            )
        if name == "board":
            acc = A["acc"]
            b = 2 * 6 * _native.MAX_TOOLS
            return np.array([[fx_to_float(acc[b + 2 * i], acc[b + 2 * i + 1]) for i in range(3)]])
        if name == "work":
            acc = A["acc"]
            b = 2 * (6 * _native.MAX_TOOLS + 3)
            return np.array([fx_to_float(acc[b], acc[b + 1])])
        if name == "tool_pos":
            return A["tool"][:, 0:3]
        if name == "tool_vel":
            return A["tool"][:, 3:6]
        if name == "tool_rot":
            return A["tool"][:, 6:10]
        if name == "tool_omega":
            return A["tool"][:, 10:13]
        return A[name]

    def set(self, name, value):
        """Write an array given in reference particle order (particle arrays) or as stored."""
        A = self.arrays
        value = np.asarray(value)
        if name in ("x", "v", "ref", "impulses"):
            A[name][:] = value.reshape(-1, 3)[self.order]
        elif name in ("F", "Fp"):
            A[name][:] = value.reshape(-1, 9)[self.order]
            if name == "Fp" and not np.all(A["Fp"] == np.eye(3, dtype=self.R).reshape(9)):
                self.params.use_fp = 1
        elif name == "codes":
            A["codes"][:] = value[self.order]
            A["flags"][_native.FLAG["TOPOLOGY_DIRTY"]] = 1
        elif name == "damage":
            A["damage"][0][:] = value[self.order]
        elif name == "tool_pos":
            A["tool"][:, 0:3] = np.asarray(value, np.float32).reshape(-1, 3)
        elif name == "tool_vel":
            A["tool"][:, 3:6] = np.asarray(value, np.float32).reshape(-1, 3)
        elif name == "tool_rot":
            A["tool"][:, 6:10] = np.asarray(value, np.float32).reshape(-1, 4)
        elif name == "tool_omega":
            A["tool"][:, 10:13] = np.asarray(value, np.float32).reshape(-1, 3)
        elif name == "mobility":
            A["mobility"][:] = np.asarray(value, self.R).reshape(36)
        else:
            A[name][...] = value

    # ------------------------------------------------------------- physics

    def _field_codes(self):
        return ptr(self.arrays["zero_codes"] if self.single_field else self.arrays["codes"])

    def refresh_stress(self):
        self.L.orc_refresh_stress(ctypes.byref(self.params), ctypes.byref(self.S))

    def material_step(self):
        force = (not self.config.cache_topology) or self.arrays["flags"][_native.FLAG["TOPOLOGY_DIRTY"]]
        self.L.orc_material_step(ctypes.byref(self.params), ctypes.byref(self.S), self._field_codes(), int(bool(force)))

    def register(self):
        self.L.orc_register(ctypes.byref(self.params), ctypes.byref(self.S), self._field_codes())

    def rigid_contacts(self, cut_bits=1):
        self.L.orc_rigid_contacts(ctypes.byref(self.params), ctypes.byref(self.S), int(cut_bits))

    def particle_contacts(self):
        self.arrays["flags"][_native.FLAG["STEP"]] = self.step_count
        self.L.orc_particle_contacts(ctypes.byref(self.params), ctypes.byref(self.S))

    def assign_sides(self, cut_index, cutting=True):
        self.L.orc_assign(ctypes.byref(self.params), ctypes.byref(self.S), int(cut_index), int(bool(cutting)))

    def cut_bits(self, cutting):
        if not cutting:
            return 0
        cfg = self.config
        return 1 | (2 if cfg.cut_work == "advance" else 0) | (4 if cfg.cut_hold else 0)

    def set_cut(self, cut_index):
        if cut_index != self.cut_index:
            self.arrays["damage"][:] = 0
            self.cut_index = cut_index

    def step(self, target_edge=(0.0, 0.0, 0.042), cutting=True, cut_index=0, orientation=None):
        self.set_cut(cut_index)
        self.arrays["flags"][_native.FLAG["STEP"]] = self.step_count
        target = np.asarray(target_edge, np.float32).astype(self.R).reshape(3)
        rot = np.asarray(orientation if orientation is not None else [0, 0, 0, 1], np.float32).astype(self.R).reshape(4)
        self.L.orc_substep(ctypes.byref(self.params), ctypes.byref(self.S), self.cut_bits(cutting), int(cut_index),
                           self._field_codes(), int(self.config.cache_topology), ptr(target), ptr(rot))
        self.step_count += 1

    def advance(self, targets, cutting=True, cut_index=0, orientations=None):
        targets = np.asarray(targets, np.float32)
        if orientations is None:
            orientations = np.tile([0, 0, 0, 1.0], (len(targets), 1))
        orientations = np.asarray(orientations, np.float64)
        orientations = (orientations / np.linalg.norm(orientations, axis=1)[:, None]).astype(np.float32)
        for t, q in zip(targets, orientations):
            self.step(t, cutting, cut_index, q)

    def drive_tool(self, target_edge, orientation=None):
        """Solver._drive_tool (solver.py:824-831): tool.step of every knife with the current reaction sums."""
        target = np.asarray(target_edge, np.float32).reshape(3)
        rot = np.asarray(orientation if orientation is not None else [0, 0, 0, 1], np.float32).reshape(4)
        for k in range(self.config.tool_count):
            self.L.orc_drive_one(ctypes.byref(self.params), ctypes.byref(self.S), k, ptr(target), ptr(rot))

    def external_interval(self, state_packed, steps, cutting=True, cut_index=0):
        """ExternalToolPort.advance (coupling.py:88-189): returns (impulse, angular about the world origin, errors)."""
        self.set_cut(cut_index)
        packed = np.asarray(state_packed, np.float32).astype(self.R)
        self.L.orc_load_external(ctypes.byref(self.params), ctypes.byref(self.S), ptr(packed))
        dummy_t = np.zeros(3, self.R)
        dummy_q = np.array([0, 0, 0, 1], self.R)
        for _ in range(steps):
            self.arrays["flags"][_native.FLAG["STEP"]] = self.step_count
            self.L.orc_substep(ctypes.byref(self.params), ctypes.byref(self.S), self.cut_bits(cutting), int(cut_index),
                               self._field_codes(), int(self.config.cache_topology), ptr(dummy_t), ptr(dummy_q))
            self.step_count += 1
        self.L.orc_validate_interval(ctypes.byref(self.params), ctypes.byref(self.S))
        return self.arrays["interval"][:3].copy(), self.arrays["interval"][3:].copy(), self.arrays["errors"].copy()

    def hold_solve(self):
        """BladeConstraint.solve (blade_constraint.py:254-324) alone, on the current grid velocities and masses."""
        self.L.orc_hold_solve(ctypes.byref(self.params), ctypes.byref(self.S))

    def embedded_particles(self):
        """Solver.embedded_particles (solver.py:892-900): particles beside the blade body, inside the labelling band."""
        return int(self.L.orc_count_embedded(ctypes.byref(self.params), ctypes.byref(self.S)))

    def num_threads(self):
        return self.L.orc_num_threads()


def config_dict(cfg):
    return asdict(cfg)


class MlsState(ctypes.Structure):
    _fields_ = [(name, P) for name in ("x", "v", "C", "F", "yield_stress", "damage", "damage_reference", "grid_mass",
                                        "grid_momentum", "grid_v", "inversions")]


class MlsOracle:
    """MlsSolver (mlsmpm.py:232-446) restated on the CPU, particles in reference order (AoS)."""

    def __init__(self, cfg, params=None, damage_from_start=True):
        from blademaster_gb300.mlsmpm import TopoCutParams, fixed_shift, grid_layout

        params = params or TopoCutParams()
        L = self.L = lib()
        if L.orc_mls_state_size() != ctypes.sizeof(MlsState):
            raise RuntimeError("oracle MLS state layout mismatch")
        L.orc_mls_substep.argtypes = [ctypes.POINTER(_native.MlsParams), ctypes.POINTER(MlsState),
                                      ctypes.POINTER(_native.Params), ctypes.POINTER(State)]
        L.orc_mls_substep.restype = None
        self.config = cfg
        dx = cfg.grid_spacing
        reference, _, _ = points(cfg.size, dx, cfg.shape, cfg.sampling_seed)
        self.reference = reference
        n = self.n = len(reference)
        volume = (dx / 2) ** 3
        mass = cfg.density * volume
        radius = dx / 4
        blade_offset = max(cfg.blade_contact_radius or radius, radius - cfg.blade_half_size[0])
        ratio = 1.0 if cfg.contact_reference_dt == 0 else (cfg.dt / cfg.contact_reference_dt) ** 2
        sn, gk = cfg.normal_scale * ratio, cfg.tangent_stiffness * ratio
        mu = cfg.young_modulus / (2 * (1 + cfg.poisson_ratio))
        lam = cfg.young_modulus * cfg.poisson_ratio / ((1 + cfg.poisson_ratio) * (1 - 2 * cfg.poisson_ratio))
        self.mass, self.mu = mass, mu
        origin, dims = grid_layout(reference, dx, params)
        self.origin, self.dims = origin, dims
        nodes = int(np.prod(dims))
        A = self.arrays = {}
        A["x"] = np.ascontiguousarray(reference, np.float32)
        A["v"] = np.zeros((n, 3), np.float32)
        A["C"] = np.zeros((n, 9), np.float32)
        A["F"] = np.tile(np.eye(3, dtype=np.float32).reshape(9), (n, 1))
        A["yield_stress"] = np.full(n, cfg.yield_stress, np.float32)
        A["damage"] = np.zeros(n, np.float32)
        A["damage_reference"] = np.full(n, 1.0 if damage_from_start else 0.0, np.float32)
        A["grid_mass"] = np.zeros(nodes, np.int64)
        A["grid_momentum"] = np.zeros((nodes, 3), np.int64)
        A["grid_v"] = np.zeros((nodes, 3), np.float32)
        A["inversions"] = np.zeros(1, np.int32)
        M = self.mls_params = _native.MlsParams()
        M.n = n
        for i in range(3):
            M.dims[i], M.origin[i] = int(dims[i]), float(origin[i])
        M.plastic = int(cfg.yield_stress > 0)
        M.mass_shift = fixed_shift(float(np.float32(mass)))
        M.momentum_shift = fixed_shift(float(np.float32(mass)) * dx / cfg.dt)
        M.dx, M.dt, M.mass, M.volume, M.mu, M.lam = dx, cfg.dt, mass, volume, mu, lam
        M.damaged_shear, M.softening = params.damaged_shear, params.softening
        M.compressed = (1 - params.compression) ** params.sensitivity
        M.stretched = (1 + params.stretch) ** params.sensitivity
        T = self.mls_state = MlsState()
        for name, _ in MlsState._fields_:
            setattr(T, name, A[name].ctypes.data)
        # contact state: one held knife (tool model -1, zero mobility), cutting off
        p = self.contact_params = _native.Params()
        p.n, p.tool_count, p.tool_model, p.external_tool = n, 1, -1, 1
        p.dt, p.spacing, p.mass, p.volume, p.radius = cfg.dt, dx, mass, volume, radius
        p.normal_scale, p.tangent_stiffness = sn, gk
        p.friction_static, p.friction_dynamic, p.tangent_damping = cfg.friction_static, cfg.friction_dynamic, cfg.tangent_damping
        p.board_scale = cfg.board_normal_scale or sn
        p.board_half[0], p.board_half[1] = cfg.board_half_extent
        for i in range(3):
            p.half[i] = cfg.blade_half_size[i]
        p.bevel, p.blade_offset, p.blade_mass, p.threshold = cfg.blade_bevel_height, blade_offset, cfg.blade_mass, 1.0
        p.dt_d = float(np.float32(cfg.dt))
        CA = self.contact = {name: np.zeros(4, np.int64) for name in _STATE_FIELDS}
        CA["x"], CA["v"] = A["x"], A["v"]
        CA["histories"] = np.zeros((2, n, 3), np.float32)
        CA["damage"] = np.zeros((1, n), np.float32)
        CA["impulses"] = np.zeros((n, 3), np.float32)
        CA["tool"] = np.array([[0.0] * 9 + [1.0] + [0.0] * 3])
        CA["mobility"] = np.zeros(36, np.float32)
        CA["acc"] = np.zeros(_native.ACC_WORDS, np.uint64)
        CA["interval"] = np.zeros(6)
        CA["speed"] = np.zeros(1, np.float32)
        CA["errors"] = np.zeros(3, np.int32)
        CA["flags"] = np.zeros(_native.FLAG["WORDS"], np.int32)
        S = self.contact_state = State()
        for name in _STATE_FIELDS:
            setattr(S, name, CA[name].ctypes.data)
        S.capacity, S.buckets = 1, 1
        self.step_count = 0

    def advance(self, position, orientation_xyzw, velocity, angular, steps):
        """`steps` substeps with the knife held at this state; returns (impulse, angular impulse)."""
        packed = np.zeros(49, np.float32)
        packed[:3], packed[3:7], packed[7:10], packed[10:13] = position, orientation_xyzw, velocity, angular
        self.L.orc_load_external(ctypes.byref(self.contact_params), ctypes.byref(self.contact_state), ptr(packed))
        for _ in range(steps):
            self.L.orc_mls_substep(ctypes.byref(self.mls_params), ctypes.byref(self.mls_state),
                                   ctypes.byref(self.contact_params), ctypes.byref(self.contact_state))
        self.step_count += steps
        interval = self.contact["interval"]
        return interval[:3].copy(), interval[3:].copy()


def metrics(x, v, F, Fp, mass, volume, mu, lam):
    """diagnostics.metrics (diagnostics.py:7-32): the six values of Metrics.read as float64
    (exact energy sums, then the extrema), in the device kernel's operation order."""
    x, v = (np.ascontiguousarray(a, np.float32).reshape(-1, 3) for a in (x, v))
    F, Fp = (np.ascontiguousarray(a, np.float32).reshape(-1, 9) for a in (F, Fp))
    out = np.zeros(6, np.float64)
    lib().orc_metrics(ptr(x), ptr(v), ptr(F), ptr(Fp), len(x), mass, volume, mu, lam, ptr(out))
    return out
