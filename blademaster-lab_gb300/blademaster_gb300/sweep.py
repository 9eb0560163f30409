"""Seeded sweep instances: the horizontal-cylinder cut sweep.

A 36 mm diameter, 120 mm long cylinder lying along x on the board
(E log-uniform in [5e4, 5e5] Pa, nu 0.35, rho 950 kg/m^3, Newtonian
viscosity 5 Pa s), grid spacing drawn from {3, 4, 4.5, 6} mm, a 1 mm
external knife at an x offset uniform in [0, h/2] descending at a speed
log-uniform in [0.02, 0.2] m/s, the material step from the banana_dt rule
(presets.py:50-60) for 1 ms coupling intervals.  Synthetic inputs: the
reference measures its sweeps on no dataset.

``impulse_bins`` integrates a sweep's per-interval force trace into impulse
bins of any width, as the reference's convergence studies compare runs of
different steps and intervals.
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


def impulse_bins(end_times, forces, edges):
    """convergence.impulse_bins (blademaster_warp/convergence.py:23-48): the impulse (N s) of a
    force trace in each bin [edges[k], edges[k + 1]].

    forces[i] is the average force over the coupling interval that ends at
    end_times[i] (the first interval starts at t = 0), so a bin takes the exact
    integral of that piecewise-constant force: the trace's impulse up to an edge
    is the impulse of the whole intervals before it plus the force of the
    interval that holds the edge times the time into it.  Bins of another
    width than the intervals therefore keep the total.  Raises ValueError for a
    trace that is empty, not (count, 3), not finite or not increasing from
    t > 0, and for bins that leave the trace (1e-10 s of slack at its end).
    """
    t = np.asarray(end_times, dtype=float)
    f = np.asarray(forces, dtype=float)
    e = np.asarray(edges, dtype=float)
    if not (t.ndim == 1 and t.size and f.shape == (t.size, 3) and np.isfinite(t).all() and np.isfinite(f).all()
            and t[0] > 0 and np.all(np.diff(t) > 0)):
        raise ValueError("Expected finite forces and increasing interval end times")
    if not (e.ndim == 1 and e.size >= 2 and np.isfinite(e).all() and e[0] >= 0 and e[-1] <= t[-1] + 1.0e-10
            and np.all(np.diff(e) > 0)):
        raise ValueError("Requested bins must lie within the complete trace")
    start = np.concatenate([[0.0], t[:-1]])
    before = np.concatenate([np.zeros((1, 3)), np.cumsum(f * (t - start)[:, None], axis=0)[:-1]])
    e = np.minimum(e, t[-1])
    i = np.searchsorted(t, e, side="left")  # the interval (start_i, t_i] that holds each edge
    at_edges = before[i] + f[i] * (e - start[i])[:, None]
    return np.diff(at_edges, axis=0)
