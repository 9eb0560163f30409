"""Config validation mirrors blademaster_warp/solver.py:87-144 message for message."""

from dataclasses import replace

import pytest

from blademaster_gb300.solver import Config
from blademaster_gb300.presets import banana_config, banana_dt


@pytest.mark.parametrize(
    "kwargs, message",
    [
        (dict(grid_storage="dense"), "grid_storage must be hash or compact"),
        (dict(pair_search="grid"), "pair_search must be auto, hash, all or list"),
        (dict(pair_skin=-1.0), "pair_skin must be non-negative"),
        (dict(blade_contact_radius=-1.0), "blade_contact_radius must be non-negative"),
        (dict(cut_work="absolute"), "cut_work must be relative or advance"),
        (dict(tool_substep="jump"), "tool_substep must be hold or predict"),
        (dict(tool_substep="predict"), "tool_substep=predict requires external_tool"),
        (dict(dt=float("nan")), "Nonfinite configuration"),
        (dict(dt=0.0), "Invalid positive parameter"),
        (dict(poisson_ratio=0.5), "Invalid material/sharpness"),
        (dict(friction_dynamic=0.5), "Invalid transfer/friction"),
        (dict(yield_stress=-1.0), "Negative damping/plasticity/reference step"),
        (dict(maxwell_fraction=2.0), "maxwell_tau must be non-negative"),
        (dict(normal_scale=2.0), "Rescaled contact factor exceeds 1"),
        (dict(board_normal_scale=2.0), "Board normal scale must be in"),
        (dict(board_half_extent=(-1.0, 0.0)), "Board half extent must be non-negative"),
        (dict(blade_bevel_height=0.05), "Invalid blade geometry"),
        (dict(free_blade=True, pose_servo=True), "Choose free, pose-servo"),
        (dict(tool_count=2), "Several tools are supported only as free knives"),
        (dict(tool_count=0), "Several tools are supported only as free knives"),
        (dict(grid_spacing=0.05), "Grid spacing must be positive with at least two cells per axis"),
    ],
)
def test_invalid_configs_raise_reference_messages(kwargs, message):
    with pytest.raises(ValueError, match=message):
        Config(**kwargs)


def test_contact_scales_and_presets():
    cfg = Config(dt=0.001, contact_reference_dt=0.002, normal_scale=0.2, tangent_stiffness=0.1)
    assert cfg.contact_scales() == pytest.approx((0.05, 0.025))
    b = banana_config()
    assert b.dt == 0.0000625 and b.young_modulus == 400000.0
    # presets.py:50-60: at most 62.5 us and half the CFL limit, dividing 1 ms
    for spacing in (0.003, 0.004, 0.0045, 0.006):
        dt = banana_dt(b, spacing)
        assert dt <= 0.0000625 and abs(round(0.001 / dt) * dt - 0.001) < 1e-15
    assert replace(Config(), free_blade=True, tool_count=3).tool_count == 3
