"""Scene-level errors of the float32 results against a float64 run of the same scene.

The CUDA path reproduces the float32 oracle bit for bit; the oracle's float64
build (``OracleSolver(cfg, real=np.float64)``) runs the same restatement in
double precision.  These tests run the leading part of two benchmark scenes,
and of the 8-knife block at a coarse grid, in both and bound the float32
run's error on what the scenes report: the blade's impulse per coupling
interval (blade force and impulse are held to 0.5 %) and the knife's pose.
``oracle/fp64_scenes.py`` runs the whole scenes and reports the same errors,
and compares a float32 run against one whose knives start 10 nm lower.
"""

import numpy as np
import pytest

from oracle.fp64_scenes import block, freefall, triple_cut


def test_float64_build_runs_the_same_scene():
    from blademaster_gb300.solver import Config
    from oracle.oracle import OracleSolver

    cfg = Config()
    o32, o64 = OracleSolver(cfg), OracleSolver(cfg, real=np.float64)
    assert o64.get("x").dtype == np.float64 and o32.get("x").dtype == np.float32
    for o in (o32, o64):
        for _ in range(5):
            o.step((0.0, 0.0, 0.2), cutting=False)
    x32, x64 = o32.get("x").astype(np.float64), o64.get("x")
    # the reference positions differ by their float32 rounding (< 3e-9 m at these sizes)
    assert np.abs(x32 - x64).max() < 1e-7
    np.testing.assert_allclose(o32.get("v"), o64.get("v"), atol=1e-6)
    with pytest.raises(ValueError):
        OracleSolver(cfg, real=np.float16)


def test_gravity_knife_landing_against_float64():
    # the first 0.1 s of the gravity knife (8960 particles): the knife lands and starts cutting; 10 ms windows of its reaction impulse
    r = freefall(substeps=400)
    assert r["interval_error_of_largest"]["max"] < 1e-4
    assert r["total"]["relative_error"] < 1e-5
    assert r["knife_position_difference_m"] < 1e-6
    assert r["released_particles"]["float32"] == r["released_particles"]["float64"]
    assert r["device_errors"]["float32"] == r["device_errors"]["float64"] == [0, 0, 0]


def test_triple_cut_first_intervals_against_float64():
    # the first 60 port intervals of the triple cut (4480 particles): the knife descends through the Maxwell cylinder
    r = triple_cut(intervals=60)
    assert r["largest_interval_impulse"] > 1e-4  # the knife is in contact
    assert r["interval_error_of_largest"]["max"] < 1e-3
    assert r["total"]["relative_error"] < 5e-3  # blade impulse within 0.5 %
    assert r["released_particles"]["float32"] == r["released_particles"]["float64"] > 0


def test_knife_block_at_a_coarse_grid_against_float64_and_a_shifted_start():
    # the 8-knife block at a 10 mm grid (12,800 particles), its first 0.2 ms with the knives pressing in:
    # the float64 run, and a float32 run with the knives started 10 nm lower, both within 0.1 % on the
    # knives' total impulse
    r = block(substeps=20, window=10, spacing=0.01)
    assert r["second_run"] == "float64" and r["largest_interval_impulse"] > 1e-4
    assert r["total"]["relative_error"] < 1e-3
    assert r["knife_position_difference_m"] < 1e-8
    assert r["device_errors"]["float32"] == r["device_errors"]["float64"] == [0, 0, 0]
    p = block(substeps=20, window=10, spacing=0.01, perturb=1e-8)
    assert p["second_run"] == "float32, knives 1e-08 m lower"
    assert p["total"]["relative_error"] < 1e-3
    assert 0.0 < p["knife_position_difference_m"] < 2e-8
