"""The three single-scene workloads the throughput metric is quoted on.

* ``gravity_knife`` - a free 0.2 kg knife released 5 mm above a block
  (0.14 x 0.10 x 0.08 m, 10 mm grid, 8960 particles on the regular 5 mm
  lattice, E = 2e5 Pa, nu = 0.3, rho = 1000 kg/m^3), gravity and material
  reaction only, as blademaster_warp/paper_freefall.py:20-157 runs its
  Fig. 3 knife (cutting energy 100, unit normal and board factors, identity
  orientation instead of the 25 degree tilt).  At the Table I step of 2 ms the
  grid CFL number is 3.3 and the material inverts on the fifth substep; the
  stable stand-in runs the same second at 0.25 ms (CFL 0.41).
* ``triple_cut`` - a horizontal Maxwell cylinder (r = 18 mm, L = 120 mm on
  the board, 6 mm grid, 4480 particles, E = 1e5 Pa, nu = 0.35,
  rho = 950 kg/m^3, Maxwell element of viscosity 5 Pa s holding half the
  shear modulus) cut three times by an externally prescribed 1 mm knife
  descending at 0.1 m/s to the board at x = +30, 0, -30 mm (cut indices
  0, 1, 2), each slice then pushed 20 mm towards +x, as the reference's
  scenarios drive ExternalToolPort from keyframes (scenarios.py:72-92,
  293-306, 309-434).
* ``block_8knives`` - the 1.6 M-particle block (0.20 x 0.10 x 0.08 m, 2 mm
  grid) with the gravity-knife material and 8 free knives at x = -70 ... +70
  mm, 20 mm apart, edges starting 1 mm into the top face and moving down at
  0.05 m/s, dt = 10 us (2000 substeps = 20 ms).

Inputs are synthetic and seeded; the reference measures on no dataset.
"""

from dataclasses import replace

import numpy as np

from .coupling import ToolState
from .solver import Config

# -------------------------------------------------------------- gravity knife

GRAVITY_KNIFE_STABLE_DT = 0.00025


def gravity_knife(dt=GRAVITY_KNIFE_STABLE_DT):
    """Config, initial knife centre (1, 3) and velocity (1, 3) of the gravity-knife scene."""
    cfg = Config(
        size=(0.14, 0.10, 0.08),
        grid_spacing=0.01,
        dt=dt,
        density=1000.0,
        young_modulus=2.0e5,
        poisson_ratio=0.3,
        free_blade=True,
        blade_mass=0.2,
        blade_half_size=(0.0005, 0.05, 0.02),
        cutting_energy=100.0,
        normal_scale=1.0,
        board_normal_scale=1.0,
        cache_topology=True,
    )
    return cfg, np.array([[0.0, 0.0, 0.08 + 0.005 + 0.02]]), np.zeros((1, 3))


def edge_height(position, orientation_xyzw, half_size):
    """Lowest point of the knife edge (paper_impact.edge_height): both edge ends, z."""
    q = np.asarray(orientation_xyzw, np.float64)
    u, w = q[:3], q[3]

    def rotate(v):
        return v * (2 * w * w - 1) + u * (2 * np.dot(u, v)) + np.cross(u, v) * (2 * w)

    ends = [np.asarray(position, np.float64) + rotate(np.array([0.0, s * half_size[1], -half_size[2]]))
            for s in (-1.0, 1.0)]
    return float(min(e[2] for e in ends))


# ----------------------------------------------------------------- triple cut

TRIPLE_CUT_RADIUS, TRIPLE_CUT_LENGTH = 0.018, 0.12
TRIPLE_CUT_KNIFE = (0.0005, 0.025, 0.02)
TRIPLE_CUT_POSITIONS = (0.03, 0.0, -0.03)
TRIPLE_CUT_INTERVAL = 0.002  # coupling interval: max(2 ms, dt) as scenarios.run (scenarios.py:319)


def triple_cut_config(maxwell_viscosity=5.0, maxwell_fraction=0.5):
    """The cylinder of the triple cut; the Maxwell element's viscosity is tau times its shear modulus."""
    cfg = Config(
        size=(TRIPLE_CUT_LENGTH, 2 * TRIPLE_CUT_RADIUS, 2 * TRIPLE_CUT_RADIUS),
        shape="hcylinder",
        grid_spacing=0.006,
        dt=0.0000625,
        density=950.0,
        young_modulus=1.0e5,
        poisson_ratio=0.35,
        cutting_energy=10.0,
        external_tool=True,
        blade_half_size=TRIPLE_CUT_KNIFE,
        cache_topology=True,
    )
    mu = cfg.young_modulus / (2 * (1 + cfg.poisson_ratio))
    return replace(cfg, maxwell_fraction=maxwell_fraction, maxwell_tau=maxwell_viscosity / (maxwell_fraction * mu))


def triple_cut_keyframes(speed=0.1, push=0.02, positions=TRIPLE_CUT_POSITIONS):
    """(time, knife centre, cut index or -1) keyframes: per cut a descent to the board, a hold, a
    rise to two thirds of the height, a push of the slice towards +x and a rise clear of it."""
    hz = TRIPLE_CUT_KNIFE[2]
    height = 2 * TRIPLE_CUT_RADIUS
    above, bottom, tip_over, clear = height + 0.002 + hz, 0.0003 + hz, 2 * height / 3 + hz, height + 0.01 + hz
    keys, t = [], 0.0
    for index, x in enumerate(positions):
        descent = (above - bottom) / speed
        keys += [
            (t, (x, 0.0, above), index),
            (t + 0.05, (x, 0.0, above), index),
            (t + 0.05 + descent, (x, 0.0, bottom), index),
            (t + 0.10 + descent, (x, 0.0, bottom), -1),
            (t + 0.20 + descent, (x, 0.0, tip_over), -1),
            (t + 0.20 + descent + push / speed, (x + push, 0.0, tip_over), -1),
            (t + 0.30 + descent + push / speed, (x + push, 0.0, clear), -1),
        ]
        t = keys[-1][0] + 0.05
    keys.append((t, keys[-1][1], -1))
    return keys


def command_at(t, keys):
    """Knife state, cutting flag and cut index at time t (scenarios.command_at, scenarios.py:293-306),
    with the identity orientation throughout."""
    times = np.array([k[0] for k in keys])
    j = min(int(np.searchsorted(times, t, side="right")) - 1, len(keys) - 2)
    j = max(j, 0)
    a, b = keys[j], keys[j + 1]
    duration = b[0] - a[0]
    u = float(np.clip((t - a[0]) / duration, 0.0, 1.0))
    p = (1 - u) * np.array(a[1]) + u * np.array(b[1])
    v = (np.array(b[1]) - np.array(a[1])) / duration
    index = max(k[2] for k in keys[: j + 1])
    return ToolState(p, [0.0, 0.0, 0.0, 1.0], v, [0.0, 0.0, 0.0]), a[2] >= 0, index


def triple_cut_schedule(keys=None, interval=TRIPLE_CUT_INTERVAL):
    """One (ToolState, cutting, cut_index) per coupling interval of the whole triple cut."""
    keys = keys or triple_cut_keyframes()
    count = int(round(keys[-1][0] / interval))
    return [command_at(i * interval, keys) for i in range(count)]


def packed_state(state):
    """The 49 floats ExternalToolPort.advance uploads for a ToolState (tool.load_external_state)."""
    state = state.checked()
    return np.concatenate([state.position, state.orientation_xyzw, state.linear_velocity, state.angular_velocity,
                           state.mobility.ravel()]).astype(np.float32)


# ------------------------------------------------------------ block, 8 knives


def block_8knives(spacing=0.002):
    """Config, knife centres (8, 3) and velocities (8, 3) of the 8-knife block."""
    cfg = Config(
        size=(0.20, 0.10, 0.08),
        grid_spacing=spacing,
        dt=1.0e-5,
        density=1000.0,
        young_modulus=2.0e5,
        poisson_ratio=0.3,
        free_blade=True,
        tool_count=8,
        blade_half_size=(0.0005, 0.06, 0.02),
        cache_topology=True,
    )
    knives = np.array([[x, 0.0, 0.079 + 0.02] for x in np.arange(-0.07, 0.0701, 0.02)])
    return cfg, knives, np.tile([0.0, 0.0, -0.05], (8, 1))
