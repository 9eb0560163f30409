"""An independent float64 restatement of the material step, against the oracle and the CUDA path.

The bit-exact parity tests compare the CUDA path with the oracle, and the two
compile the same arithmetic source (vector algebra, SVD, polar decomposition,
log and exp).  This leg shares nothing with either: its own particle lattice
and trilinear stencils (geometry.py:52-90 restated here), numpy's float64 SVD,
log, exp and expm1, and dense numpy scatters over the (node, code) fields.
It restates from the reference's sources:

* the corotated stress of the elastic part f = F Fp^-1 (material.py:78-112);
* the Hencky-strain von Mises return map (material.py:404-431);
* the Maxwell branch with its float64 viscous state (material.py:485-566);
* one material step: P2G over the (node, code) fields, the Eq. 8 exchange of
  compatible fields, grid velocities, G2P with the FLIP blend, the MUSL
  re-scatter and the F update (material.py:127-475, solver.py:334-376).

The state is a block with five cut fields (two cuts), a smooth rotation
field that turns the far end of the block by 2.5 rad, stretches that yield,
a Maxwell state and random velocities and impulses.  After one step the
float32 results agree with the float64 ones to 1e-5 relative (of each
array's largest value) for x, v, F, Fp and the viscous state; the stress to
2e-5 (1.05e-5 measured): its volumetric term lam (J - 1) J with J - 1 = 0.02
loses float32 digits to the cancellation in J - 1, as the reference's
float32 stress does.

This leg found that the stress refresh after host writes (refresh_stress)
ran the plastic return map when both plasticity and the Maxwell branch are
on; the reference's compute_stress_maxwell (material.py:569-589) does not,
and neither does this library now.
"""

from itertools import product

import numpy as np
import pytest

from blademaster_gb300.solver import Config
from oracle.oracle import OracleSolver

F32 = np.float32
RTOL = {"x": 1.0e-5, "v": 1.0e-5, "F": 1.0e-5, "Fp": 1.0e-5, "viscous": 1.0e-5, "stress": 2.0e-5}


# ---------------------------------------------------------- own geometry


def lattice(size, spacing):
    """Regular particles, two per cell and axis (geometry.points, seed 0, block)."""
    size = np.asarray(size, np.float64)
    cells = np.ceil(size / spacing - 1.0e-9).astype(int)
    origin = -np.array([size[0] / 2, size[1] / 2, 0.0])
    axes = [origin[i] + (np.arange(2 * cells[i]) + 0.5) * spacing / 2 for i in range(3)]
    x = np.array(list(product(*axes)))
    x = x[np.all(x - origin <= size, axis=1)]
    return x, origin, cells


def trilinear(x, origin, spacing, cells):
    """Nodes, weights and gradients of the 8 cell corners (geometry.stencil)."""
    u = (x - origin) / spacing
    base = np.floor(u).astype(int)
    t = u - base
    corners = np.array(list(product((0, 1), repeat=3)))
    f = np.where(corners[None] == 1, t[:, None, :], 1.0 - t[:, None, :])  # (n, 8, 3)
    w = f[..., 0] * f[..., 1] * f[..., 2]
    sign = 2.0 * corners - 1.0
    g = np.stack([sign[None, :, 0] * f[..., 1] * f[..., 2], sign[None, :, 1] * f[..., 0] * f[..., 2],
                  sign[None, :, 2] * f[..., 0] * f[..., 1]], axis=-1) / spacing
    ijk = base[:, None, :] + corners[None]
    nodes = (ijk[..., 0] * (cells[1] + 1) + ijk[..., 1]) * (cells[2] + 1) + ijk[..., 2]
    return nodes, w, g


# ------------------------------------------------------ float64 material


def compatible(a, b):
    while a or b:
        if a % 3 and b % 3 and a % 3 != b % 3:
            return False
        a, b = a // 3, b // 3
    return True


def svd_rotations(f):
    """f = U diag(s) V^T with U, V proper rotations (s[2] < 0 when det f < 0)."""
    U, s, Vt = np.linalg.svd(f)
    V = Vt.transpose(0, 2, 1).copy()
    U = U.copy()
    for M in (U, V):
        flip = np.linalg.det(M) < 0
        M[flip, :, 2] *= -1.0
        s[flip, 2] *= -1.0
    return U, s, V


def corotated(U, s, V, plastic_inverse, mu, lam):
    J = s.prod(1)
    d = 2.0 * mu * (s - 1.0) + (lam * (J - 1.0) * J)[:, None] / s
    return U @ (d[:, :, None] * V.transpose(0, 2, 1)) @ plastic_inverse.transpose(0, 2, 1)


def plastic(F, Fp, mu, yield_stress):
    U, s, V = svd_rotations(F @ np.linalg.inv(Fp))
    assert s.min() > 0
    e = np.log(s)
    dev = e - e.mean(1, keepdims=True)
    norm = np.linalg.norm(dev, axis=1)
    limit = yield_stress / (2.0 * mu) * np.sqrt(2.0 / 3.0)
    flow = norm > limit
    s = s.copy()
    Fp = Fp.copy()
    ep = e[flow] - (1.0 - limit / norm[flow])[:, None] * dev[flow]
    s[flow] = np.exp(ep)
    next_f = U[flow] @ (s[flow][:, :, None] * V[flow].transpose(0, 2, 1))
    Fp[flow] = np.linalg.inv(next_f) @ F[flow]
    return U, s, V, Fp, int(flow.sum())


def maxwell(U, s, V, F, Fp, D, mu, lam, mu_m, relax):
    f = U @ (s[:, :, None] * V.transpose(0, 2, 1))
    fm = f @ np.linalg.inv(np.eye(3) + D)
    Um, sm, Vm = svd_rotations(fm)
    assert sm.min() > 0
    e = np.log(sm)
    dev = e - e.mean(1, keepdims=True)
    if relax > 0:
        step = relax * dev
        dev = dev - step
        delta = Vm @ (np.expm1(step)[:, :, None] * Vm.transpose(0, 2, 1))
        D = D + delta + delta @ D
    kirchhoff = Um @ ((2.0 * mu_m * dev)[:, :, None] * Um.transpose(0, 2, 1))
    equilibrium = corotated(U, s, V, np.linalg.inv(Fp), mu - mu_m, lam + 2.0 / 3.0 * mu_m)
    return equilibrium + kirchhoff @ np.linalg.inv(F).transpose(0, 2, 1), D


def stress_of(F, Fp, D, k):
    """compute_stress_maxwell (material.py:569-589): no projection, no relaxation."""
    U, s, V = svd_rotations(F @ np.linalg.inv(Fp))
    return maxwell(U, s, V, F, Fp, D, k["mu"], k["lam"], k["mu_m"], 0.0)[0]


def material_step(x, v, F, Fp, D, codes, nodes, w, g, imp, k):
    n = len(x)
    keys = codes[:, None] * k["node_count"] + nodes
    unique, slot = np.unique(keys, return_inverse=True)
    slot = slot.reshape(n, 8)
    node_of, code_of = unique % k["node_count"], unique // k["node_count"]
    compat = np.array([[compatible(int(a), int(b)) for b in code_of] for a in code_of])
    compat &= node_of[:, None] == node_of[None, :]
    np.fill_diagonal(compat, False)
    S = len(unique)
    P = stress_of(F, Fp, D, k)
    mass, volume, dt = k["mass"], k["volume"], k["dt"]
    m = np.zeros(S)
    mom = np.zeros((S, 3))
    J = np.zeros((S, 3))
    np.add.at(m, slot, mass * w)
    np.add.at(mom, slot, mass * w[..., None] * v[:, None, :])
    np.add.at(J, slot, w[..., None] * imp[:, None, :] - dt * volume * np.einsum("pij,paj->pai", P, g))
    node_mass = np.zeros(k["node_count"])
    np.add.at(node_mass, node_of, m)
    total = node_mass[node_of]

    def couple(state):  # Eq. 8 (material.py:155-193)
        return state + (m[:, None] * (compat @ state) - (compat @ m)[:, None] * state) / total[:, None]

    coupled = couple(mom)
    old_v = coupled / m[:, None]
    new_v = (coupled + couple(J)) / m[:, None]
    pic = np.einsum("pa,pai->pi", w, new_v[slot])
    dv = np.einsum("pa,pai->pi", w, (new_v - old_v)[slot])
    v_new = (1.0 - k["flip"]) * pic + k["flip"] * (v + dv)
    x_new = x + dt * pic
    remapped = np.zeros((S, 3))
    np.add.at(remapped, slot, mass * w[..., None] * v_new[:, None, :])
    velocity = couple(remapped) / m[:, None]
    F_new = F + dt * np.einsum("pai,paj->pij", velocity[slot], g)
    U, s, V, Fp_new, flowing = plastic(F_new, Fp, k["mu"], k["yield_stress"])
    stress, D_new = maxwell(U, s, V, F_new, Fp_new, D, k["mu"], k["lam"], k["mu_m"], k["relax"])
    return dict(x=x_new, v=v_new, F=F_new, Fp=Fp_new, stress=stress, viscous=D_new), flowing


# ---------------------------------------------------------------- scene


def scene_config():
    cfg = Config(grid_spacing=0.005, yield_stress=300.0, maxwell_tau=0.002, maxwell_fraction=0.4)
    return cfg


def scene_state(cfg):
    x, origin, cells = lattice(cfg.size, cfg.grid_spacing)
    rng = np.random.default_rng(11)
    n = len(x)
    # a smooth rotation field: about (1, 1, 1) by up to 2.5 rad along the block
    angle = 2.5 * (x[:, 0] - x[:, 0].min()) / np.ptp(x[:, 0])
    axis = np.ones(3) / np.sqrt(3.0)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    R = np.eye(3) + np.sin(angle)[:, None, None] * K + (1 - np.cos(angle))[:, None, None] * (K @ K)
    stretch = np.diag([1.12, 0.93, 1.0 / (1.12 * 0.93) * 1.02])
    F = R @ (stretch + 0.01 * rng.normal(size=(n, 3, 3)))
    D = 0.03 * rng.normal(size=(n, 3, 3))
    D = 0.5 * (D + D.transpose(0, 2, 1))
    codes = (np.where(x[:, 0] < -0.005, 1, np.where(x[:, 0] > 0.005, 2, 0)) +
             3 * np.where(x[:, 1] < 0.0, 1, 2)).astype(np.int64)
    v = rng.normal(scale=0.01, size=(n, 3))
    imp = rng.normal(scale=1.0e-8, size=(n, 3))
    return dict(x=x, origin=origin, cells=cells, F=F.astype(F32), D=D, codes=codes, v=v.astype(F32),
                imp=imp.astype(F32))


def constants(cfg, node_count):
    mu = cfg.young_modulus / (2 * (1 + cfg.poisson_ratio))
    lam = cfg.young_modulus * cfg.poisson_ratio / ((1 + cfg.poisson_ratio) * (1 - 2 * cfg.poisson_ratio))
    volume = (cfg.grid_spacing / 2) ** 3
    f = lambda value: float(F32(value))  # noqa: E731  (the float32 constants the solver uses)
    return dict(mu=f(mu), lam=f(lam), mu_m=f(cfg.maxwell_fraction * mu), volume=f(volume),
                mass=f(cfg.density * volume), dt=f(cfg.dt), flip=f(cfg.flip_fraction),
                yield_stress=f(cfg.yield_stress), relax=f(-np.expm1(-cfg.dt / cfg.maxwell_tau)),
                node_count=node_count)


def expected(cfg):
    st = scene_state(cfg)
    cells = st["cells"]
    node_count = int(np.prod(cells + 1))
    nodes, w, g = trilinear(st["x"], st["origin"], cfg.grid_spacing, cells)
    k = constants(cfg, node_count)
    out, flowing = material_step(st["x"].astype(F32).astype(float), st["v"].astype(float),
                                 st["F"].astype(float), np.tile(np.eye(3), (len(st["x"]), 1, 1)), st["D"],
                                 st["codes"], nodes, w.astype(F32).astype(float), g.astype(F32).astype(float),
                                 st["imp"].astype(float), k)
    return st, out, flowing


def check(actual, out):
    for name, ref in out.items():
        got = np.asarray(actual[name], np.float64)
        scale = np.abs(ref).max()
        err = np.abs(got - ref).max() / scale
        assert err <= RTOL[name], f"{name}: {err:.3g} of its largest value"


def test_float64_leg_geometry_is_the_solvers():
    cfg = scene_config()
    o = OracleSolver(cfg)
    x, origin, cells = lattice(cfg.size, cfg.grid_spacing)
    np.testing.assert_array_equal(o.reference, x)
    nodes, w, g = trilinear(x, origin, cfg.grid_spacing, cells)
    np.testing.assert_array_equal(o.node_numpy, nodes)
    np.testing.assert_allclose(o.weight_numpy, w, rtol=0, atol=1e-15)


def _load(s, st, is_oracle):
    if is_oracle:
        s.set("v", st["v"])
        s.set("F", st["F"])
        s.set("codes", st["codes"])
        s.set("impulses", st["imp"])
        s.arrays["viscous"][:] = st["D"].reshape(-1, 9)[s.order]
    else:
        s.v.assign(st["v"])
        s.F.assign(st["F"])
        s.codes.assign(st["codes"])
        s.impulses.assign(st["imp"])
        s.viscous.assign(st["D"])
    s.refresh_stress()


def test_oracle_material_step_against_the_float64_leg():
    cfg = scene_config()
    st, out, flowing = expected(cfg)
    assert flowing > len(st["x"]) // 2  # the return map acts on most particles
    o = OracleSolver(cfg)
    _load(o, st, True)
    o.material_step()
    assert not o.get("errors").any()
    actual = {name: o.get(name) for name in ("x", "v", "F", "Fp", "stress")}
    actual["viscous"] = o.arrays["viscous"][o.rank].reshape(-1, 3, 3)
    check(actual, out)
    # the leg is sharp enough to see a planted mistake: a Maxwell step without relaxation
    k_wrong = dict(constants(cfg, int(np.prod(st["cells"] + 1))), relax=0.0)
    nodes, w, g = trilinear(st["x"], st["origin"], cfg.grid_spacing, st["cells"])
    wrong, _ = material_step(st["x"].astype(F32).astype(float), st["v"].astype(float), st["F"].astype(float),
                             np.tile(np.eye(3), (len(st["x"]), 1, 1)), st["D"], st["codes"], nodes,
                             w.astype(F32).astype(float), g.astype(F32).astype(float), st["imp"].astype(float),
                             k_wrong)
    with pytest.raises(AssertionError):
        check(actual, wrong)


@pytest.mark.gpu
def test_cuda_material_step_against_the_float64_leg():
    from blademaster_gb300.solver import Solver

    cfg = scene_config()
    st, out, _ = expected(cfg)
    s = Solver(cfg)
    _load(s, st, False)
    s.material_step()
    assert not s.errors.numpy().any()
    actual = {name: getattr(s, name).numpy() for name in ("x", "v", "F", "Fp", "stress", "viscous")}
    check(actual, out)
