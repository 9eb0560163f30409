"""Scene-level float64 errors of the float32 results - test infrastructure, not part of the product.

Runs a benchmark scene twice on the CPU oracle: the float32 restatement (whose
results the CUDA path reproduces bit for bit) and its float64 build
(``OracleSolver(cfg, real=np.float64)``: every float32 array and operation in
double, float64 stencils and reference positions), and reports the float32
run's error against the float64 one for the quantities the scenes report:
the blade's impulse (force times time) and angular impulse per coupling
interval, the knife's trajectory, cutting work, damage and pieces.

    python oracle/fp64_scenes.py freefall_8960      # the gravity knife: the whole simulated second
    python oracle/fp64_scenes.py triple_cut_4480    # the triple cut: all 1390 port intervals
    python oracle/fp64_scenes.py triple_cut_4480 --intervals 200
    python oracle/fp64_scenes.py block_1p6M_8knives --substeps 100   # 1.6 M particles: ~1 s per substep each
    python oracle/fp64_scenes.py block_1p6M_8knives --spacing 0.003 --substeps 1200 --perturb 1e-8

Prints one JSON object.  Relative errors of per-interval impulses are taken
against the largest interval impulse of the float64 run (intervals without
contact have no meaningful relative error of their own).
"""

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
# run as a script, this file's folder would shadow the oracle package with oracle/oracle.py
sys.path[:] = [p for p in sys.path if Path(p or ".").resolve() != Path(__file__).resolve().parent]
for p in (ROOT / "blademaster-lab_gb300", ROOT):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

from blademaster_gb300 import scenes  # noqa: E402
from oracle import pieces  # noqa: E402
from oracle.oracle import OracleSolver  # noqa: E402


def freefall(substeps=4000, window=40):
    """The gravity knife (8960 particles) at the stable step: the knife's reaction impulse per `window` substeps, its pose, work and damage."""
    cfg, pos, _ = scenes.gravity_knife()
    runs = {}
    for real in (np.float32, np.float64):
        o = OracleSolver(cfg, real=real)
        o.set("tool_pos", pos)
        impulses, begin = [], time.perf_counter()
        acc = np.zeros(3)
        for i in range(substeps):
            o.step((0.0, 0.0, 0.0), cutting=True)
            acc += o.get("reaction")[0]  # this substep's material impulse on the knife
            if (i + 1) % window == 0:
                impulses.append(acc.copy())
                acc[:] = 0.0
        runs[real.__name__] = {
            "impulses": np.array(impulses),
            "tool": o.get("tool").copy(),
            "work": float(o.get("work")[0]),
            "released": int(np.count_nonzero(o.get("damage") >= 1.0)),
            "pieces": len(pieces.components(o.node_numpy, o.weight_numpy, o.get("codes"))[1]),
            "x": o.get("x").astype(np.float64),
            "errors": o.get("errors").tolist(),
            "seconds": time.perf_counter() - begin,
        }
    a, b = runs["float32"], runs["float64"]
    edge32 = scenes.edge_height(a["tool"][0, 0:3], a["tool"][0, 6:10], cfg.blade_half_size)
    edge64 = scenes.edge_height(b["tool"][0, 0:3], b["tool"][0, 6:10], cfg.blade_half_size)
    return {
        "scene": "freefall_8960", "substeps": substeps, "window_substeps": window, **impulse_errors(a["impulses"], b["impulses"]),
        "edge_height_m": {"float32": edge32, "float64": edge64, "difference": edge32 - edge64},
        "knife_position_difference_m": float(np.abs(a["tool"][0, 0:3] - b["tool"][0, 0:3]).max()),
        "knife_tilt_deg": {"float32": tilt(a["tool"][0, 6:10]), "float64": tilt(b["tool"][0, 6:10])},
        "work_j": {"float32": a["work"], "float64": b["work"], "relative_error": (a["work"] - b["work"]) / b["work"]},
        "released_particles": {"float32": a["released"], "float64": b["released"]},
        "pieces": {"float32": a["pieces"], "float64": b["pieces"]},
        "particle_position_difference_m": float(np.abs(a["x"] - b["x"]).max()),
        "device_errors": {"float32": a["errors"], "float64": b["errors"]},
        "cpu_seconds": {"float32": a["seconds"], "float64": b["seconds"]},
    }


def block(substeps=100, window=10, spacing=0.002, perturb=0.0):
    """The block with 8 knives from t = 0 (1.6 M particles at the 2 mm grid): every knife's reaction
    impulse per `window` substeps, the knives' poses, damage and the particle positions.

    With perturb > 0 the second run is float32 again, its knives started `perturb` metres lower:
    a measure of how far the scene itself amplifies a tiny difference."""
    cfg, knives, velocity = scenes.block_8knives(spacing)
    runs = {}
    for label, real, shift in (("float32", np.float32, 0.0),
                               ("float64", np.float32 if perturb > 0 else np.float64, perturb)):
        o = OracleSolver(cfg, real=real)
        o.set("tool_pos", knives - np.array([0.0, 0.0, shift]))
        o.set("tool_vel", velocity)
        impulses, begin = [], time.perf_counter()
        acc = np.zeros((cfg.tool_count, 3))
        for i in range(substeps):
            o.step((0.0, 0.0, 0.0), cutting=True)
            acc += o.get("reaction")
            if (i + 1) % window == 0:
                impulses.append(acc.copy())
                acc[:] = 0.0
        runs[label] = {
            "impulses": np.array(impulses),  # [windows][knives][3]
            "tool": o.get("tool").copy(),
            "released": int(np.count_nonzero(o.get("tool_damage") >= 1.0)),
            "x": o.get("x").astype(np.float64), "errors": o.get("errors").tolist(),
            "seconds": time.perf_counter() - begin,
        }
    a, b = runs["float32"], runs["float64"]
    # all knives' windows as one series of 3-vectors
    per_knife = {f"knife_{k}": impulse_errors(a["impulses"][:, k], b["impulses"][:, k])["total"]["relative_error"]
                 for k in range(cfg.tool_count)}
    return {
        "scene": f"block_{o.n}_8knives", "substeps": substeps, "window_substeps": window,
        "second_run": f"float32, knives {perturb} m lower" if perturb > 0 else "float64",
        **impulse_errors(a["impulses"].reshape(-1, 3), b["impulses"].reshape(-1, 3)),
        "total_relative_error_per_knife": per_knife,
        "knife_position_difference_m": float(np.abs(a["tool"][:, 0:3] - b["tool"][:, 0:3]).max()),
        "released_particles": {"float32": a["released"], "float64": b["released"]},
        "particle_position_difference_m": float(np.abs(a["x"] - b["x"]).max()),
        "device_errors": {"float32": a["errors"], "float64": b["errors"]},
        "cpu_seconds": {"float32": a["seconds"], "float64": b["seconds"]},
    }


def triple_cut(intervals=None):
    """The triple cut of the Maxwell cylinder (4480 particles) through the port: every interval's impulse and angular impulse, final damage and pieces."""
    cfg = scenes.triple_cut_config()
    schedule = scenes.triple_cut_schedule()[:intervals]
    steps = int(round(scenes.TRIPLE_CUT_INTERVAL / cfg.dt))
    runs = {}
    for real in (np.float32, np.float64):
        o = OracleSolver(cfg, real=real)
        imp, ang, begin = [], [], time.perf_counter()
        for state, cutting, index in schedule:
            i, a, _ = o.external_interval(scenes.packed_state(state), steps, cutting, index)
            imp.append(i)
            ang.append(a)
        runs[real.__name__] = {
            "impulses": np.array(imp), "angular": np.array(ang),
            "released": int(np.count_nonzero(o.get("damage") >= 1.0)),
            "pieces": len(pieces.components(o.node_numpy, o.weight_numpy, o.get("codes"))[1]),
            "x": o.get("x").astype(np.float64), "errors": o.get("errors").tolist(),
            "seconds": time.perf_counter() - begin,
        }
    a, b = runs["float32"], runs["float64"]
    return {
        "scene": "triple_cut_4480", "intervals": len(schedule), "substeps_per_interval": steps,
        **impulse_errors(a["impulses"], b["impulses"]),
        "angular": impulse_errors(a["angular"], b["angular"]),
        "released_particles": {"float32": a["released"], "float64": b["released"]},
        "pieces": {"float32": a["pieces"], "float64": b["pieces"]},
        "particle_position_difference_m": float(np.abs(a["x"] - b["x"]).max()),
        "device_errors": {"float32": a["errors"], "float64": b["errors"]},
        "cpu_seconds": {"float32": a["seconds"], "float64": b["seconds"]},
    }


def tilt(q):
    """Angle (degrees) between the knife's axis z and the vertical, from its xyzw quaternion."""
    x, y, z, w = (float(c) for c in q)
    zz = 1.0 - 2.0 * (x * x + y * y)  # world z component of the rotated local z axis
    return float(np.degrees(np.arccos(np.clip(zz / max(np.sqrt(x * x + y * y + z * z + w * w) ** 2, 1e-300), -1, 1))))


def impulse_errors(f32, f64):
    """Errors of a series of 3-vectors (per interval) and of their sum, against the float64 series."""
    scale = float(np.linalg.norm(f64, axis=1).max())
    per = np.linalg.norm(f32 - f64, axis=1) / scale if scale > 0 else np.zeros(len(f64))
    total32, total64 = f32.sum(0), f64.sum(0)
    return {
        "largest_interval_impulse": scale,
        "interval_error_of_largest": {"median": float(np.median(per)), "p99": float(np.percentile(per, 99)),
                                      "max": float(per.max())},
        "total": {"float32": total32.tolist(), "float64": total64.tolist(),
                  "relative_error": float(np.linalg.norm(total32 - total64) / max(np.linalg.norm(total64), 1e-300))},
    }


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("scene", choices=["freefall_8960", "triple_cut_4480", "block_1p6M_8knives"])
    ap.add_argument("--substeps", type=int, default=None,
                    help="freefall_8960: substeps (default 4000 = 1 s); block_1p6M_8knives: substeps (default 100)")
    ap.add_argument("--intervals", type=int, default=None, help="triple_cut_4480: leading port intervals (all 1390)")
    ap.add_argument("--spacing", type=float, default=0.002, help="block_1p6M_8knives: grid spacing (0.003: 0.47 M)")
    ap.add_argument("--perturb", type=float, default=0.0,
                    help="block_1p6M_8knives: compare with float32 again, knives started this much lower (m)")
    args = ap.parse_args()
    if args.scene == "freefall_8960":
        out = freefall(args.substeps or 4000)
    elif args.scene == "block_1p6M_8knives":
        out = block(args.substeps or 100, spacing=args.spacing, perturb=args.perturb)
    else:
        out = triple_cut(args.intervals)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
