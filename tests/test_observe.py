"""Observations between intervals: piece labels (topology.components,
topology.py:17-57) and energy metrics (diagnostics.Metrics, diagnostics.py:6-48).

CPU: the oracles against the reference's own cases (tests/test_topology.py:5-18,
tests/test_diagnostics.py:6-20) and the golden labels the reference wrote.
GPU: bm_components equals the pieces oracle (and the golden labels) exactly;
bm_metrics equals the metrics oracle to the bit.
"""

from dataclasses import replace
from pathlib import Path

import numpy as np
import pytest

from blademaster_gb300.solver import Config
from oracle import pieces
from oracle.oracle import metrics as metrics_oracle

GOLDEN = Path(__file__).parent / "golden" / "topology_default_block.npz"
CASES = ("uncut", "one_cut", "partial_cut", "two_cuts", "random27")


def constants(cfg):
    volume = (cfg.grid_spacing / 2) ** 3
    mu = cfg.young_modulus / (2 * (1 + cfg.poisson_ratio))
    lam = cfg.young_modulus * cfg.poisson_ratio / ((1 + cfg.poisson_ratio) * (1 - 2 * cfg.poisson_ratio))
    return cfg.density * volume, volume, mu, lam


# ------------------------------------------------------------------- CPU


def test_pieces_oracle_reference_cases():
    # tests/test_topology.py:5-18 of the reference
    nodes, weights = np.zeros((3, 1), dtype=int), np.ones((3, 1))
    assert pieces.components(nodes, weights, [1, 0, 2])[1].tolist() == [3]
    assert pieces.components(nodes, weights, [1, 1, 2])[1].tolist() == [2, 1]
    assert not pieces.compatible(1, 2) and not pieces.compatible(4, 7) and pieces.compatible(1, 4)
    nodes = np.array([[0, 1], [1, 2], [3, 4]])
    weights = np.array([[1.0, 0.0], [1.0, 0.0], [1.0, 0.0]])
    assert pieces.components(nodes, weights, [0, 0, 0])[1].tolist() == [1, 1, 1]


def test_pieces_oracle_matches_reference_fixture():
    f = np.load(GOLDEN)
    for key in CASES:
        labels, sizes = pieces.components(f["nodes"], f["weights"], f[f"{key}_codes"])
        np.testing.assert_array_equal(labels, f[f"{key}_labels"], err_msg=key)
        np.testing.assert_array_equal(sizes, f[f"{key}_sizes"], err_msg=key)


def test_metrics_oracle_uniform_analytic_states():
    # tests/test_diagnostics.py:6-20 of the reference, on the default block's particle count
    cfg = Config()
    mass, volume, mu, lam = constants(cfg)
    n = 1024
    x = np.zeros((n, 3), np.float32)
    x[:, 2] = 0.01
    v = np.tile(np.float32([0.2, -0.1, 0.3]), (n, 1))
    eye = np.tile(np.eye(3, dtype=np.float32), (n, 1, 1))
    values = metrics_oracle(x, v, eye, eye, mass, volume, mu, lam)
    np.testing.assert_allclose(values[0], 0.5 * n * mass * 0.14, rtol=2.0e-5)
    np.testing.assert_allclose(values[1], n * mass * 9.81 * 0.01, rtol=1.0e-6)
    assert abs(values[2]) < 1.0e-10
    np.testing.assert_allclose(values[3], np.sqrt(0.14), rtol=1.0e-6)
    assert values[4] == np.float32(0.01) and values[5] == 1.0
    R = np.tile(np.float32([[0, -1, 0], [1, 0, 0], [0, 0, 1]]), (n, 1, 1))
    assert abs(metrics_oracle(x, v, R, eye, mass, volume, mu, lam)[2]) < 1.0e-10
    dilated = np.tile(np.float32(1.01) * np.eye(3, dtype=np.float32), (n, 1, 1))
    expected = n * volume * (3 * mu * 0.01**2 + 0.5 * lam * (1.01**3 - 1) ** 2)
    np.testing.assert_allclose(metrics_oracle(x, v, dilated, eye, mass, volume, mu, lam)[2], expected, rtol=5.0e-5)
    # the elastic strain is measured against Fp: F = Fp is stress free
    assert abs(metrics_oracle(x, v, dilated, dilated, mass, volume, mu, lam)[2]) < 1.0e-10


def test_metrics_oracle_sums_do_not_depend_on_order():
    rng = np.random.default_rng(5)
    n = 4096
    x = rng.normal(0, 0.05, (n, 3)).astype(np.float32)
    v = rng.normal(0, 0.3, (n, 3)).astype(np.float32)
    F = (np.eye(3) + rng.normal(0, 0.05, (n, 3, 3))).astype(np.float32)
    Fp = np.tile(np.eye(3, dtype=np.float32), (n, 1, 1))
    mass, volume, mu, lam = constants(Config())
    a = metrics_oracle(x, v, F, Fp, mass, volume, mu, lam)
    order = rng.permutation(n)
    b = metrics_oracle(x[order], v[order], F[order], Fp[order], mass, volume, mu, lam)
    np.testing.assert_array_equal(a, b)
    assert abs(a[5] - np.linalg.det(F.astype(np.float64)).min()) < 1.0e-5
    assert abs(a[4] - x[:, 2].max()) == 0.0


# ------------------------------------------------------------------- GPU


@pytest.mark.gpu
def test_gpu_components_match_reference_fixture():
    from blademaster_gb300.solver import Solver

    f = np.load(GOLDEN)
    s = Solver(Config())
    np.testing.assert_array_equal(s.node_numpy, f["nodes"])
    for key in CASES:
        labels, sizes = s.components(f[f"{key}_codes"])
        np.testing.assert_array_equal(labels, f[f"{key}_labels"], err_msg=key)
        np.testing.assert_array_equal(sizes, f[f"{key}_sizes"], err_msg=key)


@pytest.mark.gpu
@pytest.mark.parametrize("cfg", [Config(), Config(size=(0.06, 0.04, 0.03), grid_spacing=0.003, sampling_seed=7)],
                         ids=["default", "jittered_3mm"])
def test_gpu_components_match_oracle_after_cuts(cfg):
    from blademaster_gb300.solver import Solver

    s = Solver(cfg)
    top = float(s.reference[:, 2].max())
    s.tool_pos.assign([[0.0, 0.0, top + 0.004]])
    rng = np.random.default_rng(3)
    for cut in range(2):
        for _ in range(40):
            s.step((0.0, 0.0, top - 0.6 * top), cutting=True, cut_index=cut)
        codes = s.codes.numpy()
        labels, sizes = s.components()
        want = pieces.components(s.node_numpy, s.weight_numpy, codes)
        np.testing.assert_array_equal(labels, want[0])
        np.testing.assert_array_equal(sizes, want[1])
        assert sizes.sum() == s.n
    # random codes with many distinct values per node (exercises the overflow path)
    codes = rng.integers(0, 3**6, s.n).astype(np.int64)
    labels, sizes = s.components(codes)
    want = pieces.components(s.node_numpy, s.weight_numpy, codes)
    np.testing.assert_array_equal(labels, want[0])
    np.testing.assert_array_equal(sizes, want[1])


@pytest.mark.gpu
def test_gpu_metrics_bitexact_with_oracle():
    from blademaster_gb300.diagnostics import Metrics
    from blademaster_gb300.solver import Solver

    cfg = replace(Config(), yield_stress=2000.0)
    s = Solver(cfg)
    meter = Metrics(s)
    s.tool_pos.assign([[0.0, 0.0, 0.047]])
    for _ in range(30):
        s.step((0.0, 0.0, 0.02), cutting=True)
    got = meter.read()
    want = metrics_oracle(s.x.numpy(), s.v.numpy(), s.F.numpy(), s.Fp.numpy(), s.mass, s.volume, s.mu, s.lam)
    np.testing.assert_array_equal(got, want.astype(np.float32))
    np.testing.assert_array_equal(meter.read(), got)  # the same state reads the same to the bit
    assert got[2] > 0.0


@pytest.mark.gpu
def test_gpu_metrics_uniform_analytic_states():
    # tests/test_diagnostics.py:6-20 of the reference
    from blademaster_gb300.diagnostics import Metrics
    from blademaster_gb300.solver import Solver

    s = Solver()
    meter = Metrics(s)
    s.v.assign(np.tile([0.2, -0.1, 0.3], (s.n, 1)))
    values = meter.read()
    np.testing.assert_allclose(values[0], 0.5 * s.n * s.mass * 0.14, rtol=2.0e-5)
    assert abs(values[2]) < 1.0e-10
    R = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]], float)
    s.F.assign(np.tile(R, (s.n, 1, 1)))
    assert abs(meter.read()[2]) < 1.0e-10
    s.F.assign(np.tile(1.01 * np.eye(3), (s.n, 1, 1)))
    expected = s.n * s.volume * (3 * s.mu * 0.01**2 + 0.5 * s.lam * (1.01**3 - 1) ** 2)
    np.testing.assert_allclose(meter.read()[2], expected, rtol=5.0e-5)
