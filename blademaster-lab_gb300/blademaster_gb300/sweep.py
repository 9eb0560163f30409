"""Seeded sweep instances: the horizontal-cylinder cut sweep.

A 36 mm diameter, 120 mm long cylinder lying along x on the board
(E log-uniform in [5e4, 5e5] Pa, nu 0.35, rho 950 kg/m^3, Newtonian
viscosity 5 Pa s), grid spacing drawn from {3, 4, 4.5, 6} mm, a 1 mm
external knife at an x offset uniform in [0, h/2] descending at a speed
log-uniform in [0.02, 0.2] m/s, the material step from the banana_dt rule
(presets.py:50-60) for 1 ms coupling intervals.  Synthetic inputs: the
reference measures its sweeps on no dataset.
"""

import math
from dataclasses import dataclass, replace

import numpy as np

from .coupling import ToolState
from .presets import banana_dt
from .solver import Config

SPACINGS = (0.003, 0.004, 0.0045, 0.006)
RADIUS, LENGTH = 0.018, 0.12
KNIFE_HALF = (0.0005, 0.025, 0.02)
INTERVAL = 0.001


@dataclass(frozen=True)
class Instance:
    config: Config
    offset: float  # knife x position, m
    speed: float  # descent speed, m/s

    def state(self, interval_index, start_gap=0.002):
        """Knife state for coupling interval k: the edge starts start_gap above the cylinder."""
        edge = 2 * RADIUS + start_gap - self.speed * INTERVAL * interval_index
        return ToolState([self.offset, 0.0, edge + KNIFE_HALF[2]], [0, 0, 0, 1], [0, 0, -self.speed], [0, 0, 0])


def instances(count, seed=0, spacings=SPACINGS):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        h = float(rng.choice(spacings))
        cfg = Config(size=(LENGTH, 2 * RADIUS, 2 * RADIUS), shape="hcylinder", grid_spacing=h,
                     young_modulus=float(math.exp(rng.uniform(math.log(5.0e4), math.log(5.0e5)))), poisson_ratio=0.35,
                     density=950.0, dynamic_viscosity=5.0, external_tool=True, blade_half_size=KNIFE_HALF,
                     cache_topology=True)
        cfg = replace(cfg, dt=banana_dt(cfg, h, INTERVAL))
        out.append(Instance(cfg, float(rng.uniform(0.0, 0.5) * h), float(math.exp(rng.uniform(math.log(0.02), math.log(0.2))))))
    return out
