"""Single-field MLS-MPM cutting baseline after TopoCut (blademaster_warp/mlsmpm.py).

Updated-Lagrangian MLS-MPM (quadratic B-splines, APIC, one velocity field) on
a dense grid around the material, with TopoCut damage (Eqs. 6, 7) and the
TLMPM solver's gravity, board and knife contact for a held knife (cutting
off).  ``MlsSolver`` keeps the reference's constructor, ``advance``,
``start_damage``, ``diagnostics`` and ``state``.  The kernels are the CUDA
ones in csrc/bm_mls.cu; grid sums are exact 64-bit fixed point.
"""

import ctypes
import math
from dataclasses import dataclass

import numpy as np

from . import _native
from .arrays import DeviceArray, plain_view, soa_view
from .coupling import Reaction
from .geometry import points


@dataclass(frozen=True)
class TopoCutParams:
    """TopoCut constants (mlsmpm.py:23-35)."""

    compression: float = 0.025  # epsilon_c, Eq. 6
    stretch: float = 0.01  # epsilon_s
    sensitivity: float = 1.0
    softening: float = 0.0  # gamma in Eq. 7, Pa per unit Hencky plastic strain
    damaged_shear: float = 0.0  # shear modulus factor of damaged particles
    margin: float = 0.06  # grid margin around the material, m
    headroom: float = 0.06  # grid height above the material, m


def fixed_shift(scale):
    """Exponent k with scale * 2^k in [2^40, 2^41): fixed-point units of 2^-k resolve 2^-40 of `scale`."""
    return 40 - (math.frexp(scale)[1] - 1)


def grid_layout(reference, dx, params):
    """Origin and node counts of the dense grid (mlsmpm.py:250-257)."""
    low = reference.min(0) - params.margin
    high = reference.max(0) + params.margin
    low[2] = -2 * dx
    high[2] = reference[:, 2].max() + params.headroom
    dims = np.ceil((high - low) / dx).astype(int) + 1
    return low, dims


class MlsSolver:
    """damage_from_start=True applies Eq. 6 to J of the reference configuration from the
    first step; False leaves damage off until `start_damage` (mlsmpm.py:232-238)."""

    def __init__(self, cfg, params=TopoCutParams(), device="cuda:0", damage_from_start=True):
        import torch

        if not str(device).startswith("cuda") or not torch.cuda.is_available():
            raise ValueError("CUDA device required")
        self.config, self.params = cfg, params
        self.device = torch.device(device)
        self._lib = _native.lib()
        dx = cfg.grid_spacing
        reference, _, _ = points(cfg.size, dx, cfg.shape, cfg.sampling_seed)
        self.reference = reference
        self.n = n = len(reference)
        self.volume = (dx / 2) ** 3
        self.mass = cfg.density * self.volume
        self.radius = dx / 4
        self.blade_offset = max(cfg.blade_contact_radius or self.radius, self.radius - cfg.blade_half_size[0])
        self.normal_scale, self.tangent_stiffness = cfg.contact_scales()
        self.mu = cfg.young_modulus / (2 * (1 + cfg.poisson_ratio))
        self.lam = cfg.young_modulus * cfg.poisson_ratio / ((1 + cfg.poisson_ratio) * (1 - 2 * cfg.poisson_ratio))
        self.origin, self.dims = grid_layout(reference, dx, params)
        self.compressed = (1 - params.compression) ** params.sensitivity
        self.stretched = (1 + params.stretch) ** params.sensitivity
        nodes = int(np.prod(self.dims))
        dev, f32, i32, i64 = self.device, torch.float32, torch.int32, torch.int64

        def zeros(*shape, dtype=f32):
            return torch.zeros(*shape, dtype=dtype, device=dev)

        T = self._t = {}
        T["x"] = torch.as_tensor(np.ascontiguousarray(reference.T, np.float32), device=dev)
        T["v"] = zeros(3, n)
        T["C"] = zeros(9, n)
        T["F"] = torch.eye(3, dtype=f32, device=dev).reshape(9, 1).repeat(1, n).contiguous()
        T["yield_stress"] = torch.full((n,), float(cfg.yield_stress), dtype=f32, device=dev)
        T["damage"] = zeros(n)
        T["damage_reference"] = torch.full((n,), 1.0 if damage_from_start else 0.0, dtype=f32, device=dev)
        T["grid_mass"] = zeros(nodes, dtype=i64)
        T["grid_momentum"] = zeros(3, nodes, dtype=i64)
        T["grid_v"] = zeros(3, nodes)
        T["inversions"] = zeros(1, dtype=i32)
        # contact state (contact.rigid_and_speed with one held knife)
        C = self._c = {}
        C["histories"] = zeros(2, 3, n)
        C["hist_mask"] = torch.full((n,), -1, dtype=torch.int16, device=dev)
        C["damage"] = zeros(n)
        C["impulses"] = zeros(3, n)
        C["tool"] = torch.tensor([[0.0] * 9 + [1.0] + [0.0] * 3], dtype=torch.float64, device=dev)
        C["tool_f"] = zeros(1, _native.TOOL_F_WORDS)
        C["mobility"] = zeros(36)
        C["acc"] = zeros(_native.ACC_WORDS, dtype=i64)
        C["interval"] = zeros(6, dtype=torch.float64)
        C["speed"] = zeros(1)
        C["errors"] = zeros(3, dtype=i32)
        C["flags"] = zeros(_native.FLAG["WORDS"], dtype=i32)
        C["packed"] = zeros(49)
        C["result"] = zeros(16)

        M = self._mls_params = _native.MlsParams()
        M.n = n
        for i in range(3):
            M.dims[i] = int(self.dims[i])
            M.origin[i] = float(self.origin[i])
        M.plastic = int(cfg.yield_stress > 0)
        M.mass_shift = fixed_shift(float(np.float32(self.mass)))
        M.momentum_shift = fixed_shift(float(np.float32(self.mass)) * dx / cfg.dt)
        M.dx, M.dt, M.mass, M.volume, M.mu, M.lam = dx, cfg.dt, self.mass, self.volume, self.mu, self.lam
        M.damaged_shear, M.softening = params.damaged_shear, params.softening
        M.compressed, M.stretched = self.compressed, self.stretched
        MB = self._mls_buffers = _native.MlsBuffers()
        for name, _ in _native.MlsBuffers._fields_:
            setattr(MB, name, T[name].data_ptr())
        P = self._contact_params = _native.Params()
        P.n, P.tool_count, P.tool_model, P.external_tool = n, 1, -1, 1
        P.dt, P.spacing, P.mass, P.volume, P.radius = cfg.dt, dx, self.mass, self.volume, self.radius
        P.mu, P.lam = self.mu, self.lam
        P.normal_scale, P.tangent_stiffness = self.normal_scale, self.tangent_stiffness
        P.friction_static, P.friction_dynamic, P.tangent_damping = cfg.friction_static, cfg.friction_dynamic, cfg.tangent_damping
        P.board_scale = cfg.board_normal_scale or self.normal_scale
        P.board_half[0], P.board_half[1] = cfg.board_half_extent
        for i in range(3):
            P.half[i] = cfg.blade_half_size[i]
            P.half_d[i] = float(np.float32(cfg.blade_half_size[i]))
        P.bevel, P.blade_offset, P.blade_mass, P.threshold = cfg.blade_bevel_height, self.blade_offset, cfg.blade_mass, 1.0
        P.dt_d = float(np.float32(cfg.dt))
        B = self._contact_buffers = _native.Buffers()
        B.x, B.v = T["x"].data_ptr(), T["v"].data_ptr()
        for name, tensor in C.items():
            setattr(B, name, tensor.data_ptr())
        handle = ctypes.c_void_p()
        _native.check(self._lib.bm_mls_create(ctypes.byref(M), ctypes.byref(MB), ctypes.byref(P), ctypes.byref(B),
                                              ctypes.byref(handle)))
        self._handle = handle
        self.graphs = {}
        self.step_count = 0
        self.x = soa_view(T["x"], n, "x", None)
        self.v = soa_view(T["v"], n, "v", None)
        self.F = _matrix_view(T["F"], n, "F")
        self.C = _matrix_view(T["C"], n, "C")
        self.damage = plain_view(T["damage"], (n,), np.float32, "damage")
        self.yield_stress = plain_view(T["yield_stress"], (n,), np.float32, "yield_stress")
        self.damage_reference = plain_view(T["damage_reference"], (n,), np.float32, "damage_reference")
        self.inversions = plain_view(T["inversions"], (1,), np.int32, "inversions")

    def __del__(self):
        lib = getattr(self, "_lib", None)
        if lib is None:
            return
        for g in getattr(self, "graphs", {}).values():
            lib.bm_graph_destroy(g)
        if getattr(self, "_handle", None) is not None:
            lib.bm_mls_destroy(self._handle)

    @property
    def _stream(self):
        import torch

        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def advance(self, state, duration_s, graph=True):
        """Hold the knife pose over duration_s (as ExternalToolPort with tool_substep='hold')."""
        import torch

        state = state.checked()
        dt = self.config.dt
        steps = int(round(duration_s / dt))
        if steps < 1 or not np.isclose(steps * dt, duration_s, rtol=1.0e-10, atol=1.0e-12):
            raise ValueError("Duration must be an integer number of substeps")
        packed = np.zeros(49, np.float32)
        packed[:3] = state.position
        packed[3:7] = state.orientation_xyzw
        packed[7:10] = state.linear_velocity
        packed[10:13] = state.angular_velocity  # the held knife ignores the mobility (stays zero)
        self._c["packed"].copy_(torch.as_tensor(packed, device=self.device))
        if graph:
            if steps not in self.graphs:
                handle = ctypes.c_void_p()
                _native.check(self._lib.bm_mls_graph_create(self._handle, steps, self._stream, ctypes.byref(handle)))
                self.graphs[steps] = handle
            _native.check(self._lib.bm_graph_launch(self.graphs[steps], self._stream))
        else:
            _native.check(self._lib.bm_mls_substeps(self._handle, steps, self._stream))
        self.step_count += steps
        interval = self._c["interval"].cpu().numpy()
        lost = self.diagnostics()["left_domain"]
        if lost:
            raise RuntimeError(
                f"MLS-MPM diverged by t = {self.step_count * dt:.3f} s: {lost} particles non-finite or outside the grid"
            )
        return Reaction(steps * dt, interval[:3].copy(), interval[3:6].copy(), np.asarray(state.position, dtype=float))

    def start_damage(self):
        """Enable Eq. 6 with each particle's current J as its reference volume."""
        self.damage_reference.assign(np.linalg.det(self.F.numpy().astype(np.float64)).astype(np.float32))

    def diagnostics(self):
        """Particles non-finite or outside the grid, and clamped inversions (particle-steps)."""
        local = (self.x.numpy() - self.origin) / self.config.grid_spacing
        with np.errstate(invalid="ignore"):
            base = np.floor(local - 0.5)
            outside = ~np.all(np.isfinite(base) & (base >= 0) & (base + 2 < self.dims), axis=1)
        return dict(left_domain=int(outside.sum()), clamped_inversions=int(self.inversions.numpy()[0]))

    def state(self):
        return dict(
            position=self.x.numpy(),
            velocity=self.v.numpy(),
            damage=self.damage.numpy(),
            deformation=self.F.numpy(),
            time=self.step_count * self.config.dt,
        )


def _matrix_view(tensor, n, name):
    """View of a [9][n] device tensor as (n, 3, 3)."""
    import torch

    def read():
        return tensor.t().reshape(n, 3, 3).cpu().numpy()

    def write(value):
        tensor.copy_(torch.as_tensor(np.ascontiguousarray(value), device=tensor.device).to(tensor.dtype).reshape(n, 9).t())

    return DeviceArray((n, 3, 3), np.float32, read, write, None, name)
