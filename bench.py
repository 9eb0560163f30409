"""Throughput of the TLMPM material substep on one GB300 (particle-substeps/s).

Workload (default): the plain TLMPM block cut by 8 knives at scale -
block 0.20 x 0.10 x 0.08 m, 2 mm grid, 1 mm particle lattice (1.6 M
particles), E = 2e5 Pa, nu = 0.3, rho = 1000 kg/m^3, float32, dt = 10 us;
8 free knives (1 mm thick, 120 mm long) at x = -70 ... +70 mm, 20 mm apart,
edges starting 1 mm into the top face, moving down at 0.05 m/s; sorted-cell
transfers and the skin-list pair search.  Synthetic inputs (the reference
measures on no dataset).

One step = one coupling interval of the workload (1 ms = 100 substeps for the
block), replayed as one CUDA graph.  The warm-up steps run from t = 0; the
solver is then restored to its t = 0 checkpoint, so the K timed steps are the
scene's first K intervals (K = 20: the whole 2000-substep run of the block,
with its settling, pair-list rebuilds and any re-registrations).  `value`
times them with all state resident in HBM; `e2e` restores t = 0 again and
times the same intervals through the public API (Solver.advance per interval)
with the knife targets copied from pinned host memory and the knife state
read back every call; `e2e_single_substep` does one substep per call.
The CPU baseline runs the C oracle (the reference's algorithm restated, all
host threads) on a bounded number of substeps of the same workload.

--impl reference times that CPU restatement alone, on the same workload and
metric (the reference's own implementation needs Warp 1.18, which is not
installed, and refuses CPU devices, blademaster_warp/solver.py:161-162).
"""

import argparse
from dataclasses import replace
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for p in (ROOT, ROOT / "blademaster-lab_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

METRIC = "TLMPM particle-substeps/s (1 GB300); batched & learned vs plain at <1% force err"
UNIT = "particle-substeps/s"


def workload(name):
    """(Config, knife centres, knife velocities) of a scene workload (blademaster_gb300.scenes)."""
    from blademaster_gb300 import scenes

    if name == "block_1p6M_8knives":
        return scenes.block_8knives()
    if name == "block_3mm_8knives":
        # the same scene at 3 mm spacing (0.5 M particles, still larger than L2): profiling case
        return scenes.block_8knives(spacing=0.003)
    if name == "freefall_8960":
        # the gravity knife at the stable 0.25 ms step (the Table I step of 2 ms inverts the material)
        return scenes.gravity_knife()
    raise ValueError(name)


# Substeps of one bench step: one coupling interval of the workload (1 ms for the block,
# so that 20 steps are its whole 2000-substep run; 50 ms for the gravity knife, 20 steps = 1 s).
SUBSTEPS_PER_STEP = {"block_1p6M_8knives": 100, "block_3mm_8knives": 100, "freefall_8960": 200}

# Algorithmic bytes of each stage: per particle, per registered (node, code) slot.
STAGE_BYTES = {
    "rigid": (36, 0),      # read x, v; write impulse (knife/board histories of contacting particles not counted)
    "p2g": (68, 28),       # read v, impulse, stress, code; write mass, old_v, new_v per slot
    "g2p": (56, 24),       # read+write x, v; read field indices; read old_v, new_v per slot
    "remap": (20, 16),     # read v, field indices; read mass, write coupled velocity per slot
    "fupdate": (124, 12),  # read+write F, write stress, read stencil id, base node, field indices; coupled velocity per slot
    "assign": (12, 0),     # read x (v and codes only for particles in a knife's band, not counted)
}
# Stages that are one kernel each; the largest of them is the roofline's dominant kernel.
SINGLE_KERNEL_STAGES = {"rigid": "k_rigid", "fupdate": "k_fupdate", "assign": "k_assign"}
# Whole-substep byte model: 296 B per particle, 156 B per slot (+108 B per particle with plasticity).
SUBSTEP_BYTES = (296, 156)


def sample_clocks(path):
    cmd = [
        "nvidia-smi",
        "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
        "--format=csv,noheader,nounits",
        "-lms",
        "200",
    ]
    try:
        return subprocess.Popen(cmd, stdout=open(path, "w"), stderr=subprocess.DEVNULL)
    except OSError:
        return None


def summarize_clocks(path, gpu_index):
    rows = []
    for line in Path(path).read_text().splitlines():
        parts = [p.strip() for p in line.split(",")]
        if len(parts) >= 9 and parts[0] == str(gpu_index):
            rows.append(parts)
    if not rows:
        return None
    sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
    reasons = set()
    for r in rows:
        for name, value in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), r[5:9]):
            if value.lower() == "active":
                reasons.add(name)
    return {
        "sm_mhz": float(np.median(sm)) if sm else None,
        "sm_max_mhz": float(rows[0][2]) if rows[0][2].replace(".", "").isdigit() else None,
        "reasons": sorted(reasons),
        "samples": len(rows),
    }


def peaks():
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        data = json.loads(path.read_text())
        return float(data["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_launch(stage, n, slots):
    """DRAM bytes per launch of `stage` from the committed ncu summary, scaled to this workload."""
    path = ROOT / "profiles" / "traffic.json"
    if not path.exists():
        return None
    data = json.loads(path.read_text()).get(stage)
    if not data:
        return None
    return float(data["bytes_per_particle"]) * n + float(data.get("bytes_per_slot", 0.0)) * slots


def cpu_baseline(name, seconds=15.0, max_steps=None, warmup=1):
    from oracle.oracle import OracleSolver

    cfg, knives, velocity = workload(name)
    o = OracleSolver(cfg)
    o.set("tool_pos", knives)
    o.set("tool_vel", velocity)
    zero = np.zeros(3, np.float32)
    warmup = max(1, warmup)
    for _ in range(warmup):  # registration and first-touch outside the timing
        o.step(zero, cutting=True)
    steps, begin = 0, time.perf_counter()
    while time.perf_counter() - begin < seconds and (max_steps is None or steps < max_steps):
        o.step(zero, cutting=True)
        steps += 1
    elapsed = time.perf_counter() - begin
    return {
        "value": o.n * steps / elapsed,
        "unit": UNIT,
        "cores": o.num_threads(),
        "kind": "port",
        "sample": f"{steps} substeps of the full {o.n}-particle workload after {warmup} untimed "
                  f"substep{'s' if warmup > 1 else ''}, C oracle with OpenMP",
    }


def run_sweep(args, rank, world):
    """Batched sweep of independent cutting instances (one graph launch per 1 ms interval) against the
    same instances advanced one ExternalToolPort call at a time, as the reference's sweeps run."""
    import torch

    from blademaster_gb300.batch import BatchTuner, SolverBatch
    from blademaster_gb300.coupling import ExternalToolPort
    from blademaster_gb300.solver import Solver
    from blademaster_gb300.sweep import instances

    from blademaster_gb300 import replicas

    dist, rank, world, local = replicas.init()
    torch.cuda.set_device(local)
    # weak scaling: each rank takes its share of one list of instances per rank
    everything = instances(args.instances * world, seed=0)
    sweep = [everything[i] for i in replicas.shard(len(everything), rank, world)]
    solvers = [Solver(i.config, device=f"cuda:{local}") for i in sweep]
    batch = SolverBatch(solvers)
    steps = [int(round(0.001 / s.config.dt)) for s in solvers]
    work = sum(s.n * k for s, k in zip(solvers, steps))
    k = 0

    def states():
        nonlocal k
        out = [i.state(k, start_gap=-0.001) for i in sweep]
        k += 1
        return out

    tuner = BatchTuner(cache=os.path.join(tempfile.gettempdir(), "bm_tune.json"))
    for lanes in tuner.candidates:  # first replays upload the graphs: keep them out of the tuning
        if lanes <= len(solvers):
            batch.advance(states(), 0.001, lanes=lanes, strict=False)
    tuner.tune(batch, lambda i: states(), 0.001, strict=False)
    for _ in range(args.warmup):
        batch.advance(states(), 0.001, strict=False)
    replicas.barrier(dist, torch.cuda.current_device())
    begin = time.perf_counter()
    for _ in range(args.steps):
        batch.advance(states(), 0.001, strict=False)
    replicas.barrier(dist, torch.cuda.current_device())
    batched = replicas.max_over_ranks(dist, (time.perf_counter() - begin) / args.steps)
    work = replicas.sum_over_ranks(dist, work)
    ports = [ExternalToolPort(s) for s in solvers]

    def port_interval(port, state):
        try:
            port.advance(state, 0.001)
        except RuntimeError:  # the same checks as the batch's strict=False: the interval still ran
            pass

    for p, i in zip(ports, sweep):  # warm the per-instance graphs
        port_interval(p, i.state(k, start_gap=-0.001))
    k += 1
    replicas.barrier(dist, torch.cuda.current_device())
    begin = time.perf_counter()
    for _ in range(max(1, args.steps // 4)):
        for p, s_ in zip(ports, states()):
            port_interval(p, s_)
    replicas.barrier(dist, torch.cuda.current_device())
    single = replicas.max_over_ranks(dist, (time.perf_counter() - begin) / max(1, args.steps // 4))
    failures = replicas.sum_over_ranks(dist, len(batch.failures))
    particles = replicas.sum_over_ranks(dist, sum(s.n for s in solvers))
    # The held-blade constraint's residual is a lifetime maximum (as the reference's
    # BladeConstraint.max_violation): an instance that once ends a solve above 1e-6 m/s
    # reports it at every later interval.  Listed per instance with its first interval.
    from blademaster_gb300 import _native

    residuals = batch._flags[:, _native.FLAG["HOLD_RESIDUAL"]].cpu().numpy().view(np.float32)
    first = {}
    for i, interval in batch.failures:
        first.setdefault(i, interval)
    failed_instances = [{"instance": int(rank * len(sweep) + i), "first_interval": int(k),
                         "residual_m_per_s": float(residuals[i]), "spacing_m": sweep[i].config.grid_spacing,
                         "young_modulus": sweep[i].config.young_modulus, "speed_m_per_s": sweep[i].speed}
                        for i, k in sorted(first.items())]
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": work / batched, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": batched * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"sweep_{args.instances}_hcylinders", "instances": args.instances,
                       "particles": int(particles), "substeps_per_interval": steps[0],
                       "lanes": batch.lanes, "tuned": getattr(tuner, "timings", {}),
                       "step": "one 1 ms coupling interval of every instance, host knife states in, reactions out"},
            "per_instance": {"value": work / single, "ms_per_step": single * 1e3,
                             "mode": "one ExternalToolPort.advance (graph) per instance per interval"},
            "batched_speedup": single / batched,
            "failed_instance_intervals": int(failures),
            "failed_instances": failed_instances,
            "failure_note": "the held-blade constraint ends its 8 x 48 iterations above 1e-6 m/s; the C oracle "
                            "gives the same residual on the same instance and interval, and the reference's port "
                            "raises there (coupling.py:187-188); intervals are counted, not re-run",
            "parallelism": f"replicas x{world}, {args.instances} instances per rank",
        }), flush=True)
    if dist:
        dist.destroy_process_group()


def run_learned(args, rank, world):
    """The learned tool predictor against the plain intervals it stands in for.

    Data come from the batched solver: instances of the horizontal-cylinder
    sweep at 6 mm, the knife in the reference's predict mode
    (tool_substep="predict", tool.py:97-113: inside each 1 ms interval of 16
    substeps the knife's twist follows the material reaction through a
    mobility matrix, here a compliant tool of 0.5 kg and 1e-4 kg m^2),
    descending at the instance's speed to 0.3 mm above the board and resting
    there.  `--learned-instances` instances x `--learned-intervals` intervals
    are the training set (256 x 800 = 204,800 by default); 64 other instances
    x 100 intervals are held out.  The MLP (tcgen05 GEMMs) predicts the
    interval's force and torque and the knife's twist change (12 outputs)
    from the state at the interval's start.  On each held-out interval the
    plain interval is the referee: a prediction is accepted when force and
    torque are each within 1 % of the plain ones.  `value` is the learned
    path's throughput on the held-out intervals: feature extraction and
    inference for every instance plus the plain interval for the rejected
    share (that share of the batched interval's time); `plain` is the batched
    plain intervals alone.
    """
    import torch

    from blademaster_gb300 import replicas
    from blademaster_gb300.batch import SolverBatch
    from blademaster_gb300.coupling import ToolState
    from blademaster_gb300.predictor import OUT_WITH_STATE, ToolPredictor, features_batch
    from blademaster_gb300.sweep import KNIFE_HALF, RADIUS, instances
    from blademaster_gb300.solver import Solver

    dist, rank, world, local = replicas.init()
    torch.cuda.set_device(local)
    top = 2 * RADIUS
    mobility = np.diag([2.0, 2.0, 2.0, 1.0e4, 1.0e4, 1.0e4])

    def state_at(inst, k):
        edge = max(2 * RADIUS - 0.0005 - inst.speed * 0.001 * k, 0.0003)
        moving = edge > 0.0003
        return ToolState([inst.offset, 0.0, edge + KNIFE_HALF[2]], [0, 0, 0, 1],
                         [0.0, 0.0, -inst.speed if moving else 0.0], [0.0, 0.0, 0.0], mobility)

    def sync():
        torch.cuda.synchronize(local)

    def generate(sweep, intervals, timed=False):
        solvers = [Solver(replace(i.config, tool_substep="predict"), device=f"cuda:{local}") for i in sweep]
        batch = SolverBatch(solvers, lanes=min(64, len(solvers)))
        xs, ys, times = [], [], []
        for k in range(intervals):
            states = [state_at(i, k) for i in sweep]
            sync()
            t0 = time.perf_counter()
            x = features_batch(solvers, states, top)
            sync()
            t1 = time.perf_counter()
            reactions = batch.advance(states, 0.001, strict=False)
            sync()
            t2 = time.perf_counter()
            tools = torch.stack([s._t["tool"][0] for s in solvers]).cpu().numpy()
            twist = np.concatenate([tools[:, 3:6] - [st.linear_velocity for st in states],
                                    tools[:, 10:13] - [st.angular_velocity for st in states]], axis=1)
            wrench = np.array([np.concatenate([r.impulse_ns, r.angular_impulse_nms]) / 0.001 for r in reactions])
            xs.append(x)
            ys.append(np.concatenate([wrench, twist], axis=1))
            times.append((t1 - t0, t2 - t1))
        work = sum(s.n * 16 for s in solvers)
        failures = len(batch.failures)
        del batch, solvers
        return np.concatenate(xs), np.concatenate(ys), times, work, failures

    count = args.learned_instances
    everything = instances(count * world, seed=11, spacings=(0.006,))
    sweep = [everything[i] for i in replicas.shard(len(everything), rank, world)]
    begin = time.perf_counter()
    train_x, train_y = [], []
    for start in range(0, len(sweep), 128):  # batches of at most 128 instances
        x, y, _, _, _ = generate(sweep[start:start + 128], args.learned_intervals)
        train_x.append(x)
        train_y.append(y)
    train_x, train_y = np.concatenate(train_x), np.concatenate(train_y)
    generation_s = time.perf_counter() - begin
    held = instances(64, seed=12345, spacings=(0.006,))
    test_x, test_y, times, work, failures = generate(held, args.learned_held_intervals)
    predictor = ToolPredictor(device=f"cuda:{local}", seed=0, outputs=OUT_WITH_STATE)
    begin = time.perf_counter()
    history = predictor.fit(train_x, train_y, epochs=args.learned_epochs, batch=512, lr=1e-3)
    sync()
    training_s = time.perf_counter() - begin
    predictor.predict(test_x[:64])  # first call outside the timing
    rows = len(held)
    learned_s = plain_s = 0.0
    accepted = 0
    force_err, torque_err, twist_err, mean_err = [], [], [], []
    mean = train_y.mean(0)
    for k, (t_features, t_plain) in enumerate(times):
        x, y = test_x[k * rows:(k + 1) * rows], test_y[k * rows:(k + 1) * rows]
        sync()
        t0 = time.perf_counter()
        predicted = predictor.predict(x)
        sync()
        t_infer = time.perf_counter() - t0

        def rel(a, b):
            return np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-12)

        fe, te = rel(predicted[:, :3], y[:, :3]), rel(predicted[:, 3:6], y[:, 3:6])
        ok = (fe <= 0.01) & (te <= 0.01)
        force_err.extend(fe.tolist())
        torque_err.extend(te.tolist())
        twist_err.extend(rel(predicted[:, 6:9], y[:, 6:9]).tolist())
        mean_err.extend(rel(mean[None, :3], y[:, :3]).tolist())
        accepted += int(ok.sum())
        learned_s += t_features + t_infer + (1.0 - ok.mean()) * t_plain
        plain_s += t_plain
    intervals = len(times)
    gemm = ToolPredictor(device=f"cuda:{local}", seed=1, outputs=OUT_WITH_STATE)
    big = gemm._inputs(np.random.default_rng(0).normal(size=(32768, 81)).astype(np.float32))
    gemm.forward(big)
    sync()
    t0 = time.perf_counter()
    for _ in range(20):
        gemm.forward(big)
    sync()
    forward_s = (time.perf_counter() - t0) / 20
    flops = 2 * 32768 * (96 * 256 + 2 * 256 * 256 + 256 * 16)
    # the tcgen05 GEMM alone (hidden-layer shape, bf16 operands, fp32 out), CUDA events on its stream
    import torch
    gemm_rates = {}
    for rows_g in (32768, 131072):
        a = torch.randn(rows_g, 256, device=f"cuda:{local}").to(torch.bfloat16).view(torch.int16)
        b = torch.randn(256, 256, device=f"cuda:{local}").to(torch.bfloat16).view(torch.int16)
        d = torch.empty(rows_g, 256, dtype=torch.float32, device=f"cuda:{local}")
        for _ in range(5):
            gemm._gemm(a, b, rows_g, 256, 256, D=d)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(50):
            gemm._gemm(a, b, rows_g, 256, 256, D=d)
        e1.record()
        sync()
        gemm_ms = e0.elapsed_time(e1) / 50
        gemm_rates[f"{rows_g}x256x256"] = {"us": gemm_ms * 1e3, "tflops": 2 * rows_g * 256 * 256 / (gemm_ms * 1e-3) / 1e12}
    gemm_status = int(gemm.status.item())
    learned_s = replicas.max_over_ranks(dist, learned_s)
    plain_s = replicas.max_over_ranks(dist, plain_s)
    held_work = replicas.sum_over_ranks(dist, work * intervals)
    peak_tf = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["bf16_tflops"] if (ROOT / "MEASURED_PEAKS.json").exists() else 1900.0
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": held_work / learned_s, "unit": UNIT, "n_gpus": world, "steps": intervals,
            "warmup": 0, "ms_per_step": learned_s / intervals * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (MLP) + f32 (plain referee)", "data": "synthetic",
            "config": {"workload": f"learned_{count}_hcylinders_6mm_predict", "instances": count,
                       "training_intervals": int(len(train_x)), "held_out_instances": rows,
                       "held_out_intervals": int(len(test_x)), "epochs": args.learned_epochs,
                       "outputs": "force 3, torque 3, knife twist change 6",
                       "tool": "predict mode, mobility diag(2 /kg x3, 1e4 /(kg m^2) x3)",
                       "step": "one held-out 1 ms interval of 64 instances: features, MLP, and the plain interval "
                               "for the rejected share"},
            "plain": {"value": held_work / plain_s, "ms_per_step": plain_s / intervals * 1e3},
            "learned": {"acceptance": accepted / max(len(force_err), 1), "tolerance": 0.01,
                        "force_rel_err_median": float(np.median(force_err)),
                        "force_rel_err_p90": float(np.percentile(force_err, 90)),
                        "torque_rel_err_median": float(np.median(torque_err)),
                        "twist_change_rel_err_median": float(np.median(twist_err)),
                        "mean_predictor_force_rel_err_median": float(np.median(mean_err)),
                        "training_loss": [float(history[0]), float(history[-1])],
                        "generation_s": generation_s, "training_s": training_s,
                        "held_out_failed_instance_intervals": failures},
            "mlp_forward": {"rows": 32768, "ms": forward_s * 1e3, "tflops": flops / forward_s / 1e12,
                            "frac_of_bf16_burst": flops / forward_s / 1e12 / peak_tf},
            "gemm_tn_bf16": {**gemm_rates, "status": gemm_status, "peak_bf16_tflops": peak_tf},
            "parallelism": f"replicas x{world}, {count} instances per rank",
        }), flush=True)
    if dist:
        dist.destroy_process_group()


def run_triple_cut(args, rank, world):
    """The triple cut of the Maxwell cylinder through ExternalToolPort, as the reference's scenarios
    drive it: one step = one 2 ms coupling interval (32 substeps, one graph replay and one readback
    of the interval's impulses).  The warm-up intervals run from t = 0; the solver is then restored
    to t = 0 and the first `--steps` intervals of the schedule are timed on the host clock around
    each port call (whole-job, device-synchronised by the readback)."""
    import torch

    from blademaster_gb300 import replicas, scenes
    from blademaster_gb300.coupling import ExternalToolPort
    from blademaster_gb300.solver import Solver

    dist, rank, world, local = replicas.init()
    torch.cuda.set_device(local)
    cfg = scenes.triple_cut_config()
    s = Solver(cfg, device=f"cuda:{local}")
    port = ExternalToolPort(s)
    schedule = scenes.triple_cut_schedule()
    steps = min(args.steps, len(schedule))
    start_of_run = s.checkpoint()
    for state, cutting, index in schedule[: max(args.warmup, 3)]:
        port.advance(state, scenes.TRIPLE_CUT_INTERVAL, cutting=cutting, cut_index=index)
    s.restore(start_of_run)
    torch.cuda.synchronize()
    replicas.barrier(dist, torch.cuda.current_device())
    begin = time.perf_counter()
    for state, cutting, index in schedule[:steps]:
        port.advance(state, scenes.TRIPLE_CUT_INTERVAL, cutting=cutting, cut_index=index)
    seconds = replicas.max_over_ranks(dist, time.perf_counter() - begin, torch.cuda.current_device())
    per = int(round(scenes.TRIPLE_CUT_INTERVAL / cfg.dt))
    simulated = steps * scenes.TRIPLE_CUT_INTERVAL
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": world * s.n * per * steps / seconds, "unit": UNIT, "n_gpus": world,
            "steps": steps, "warmup": args.warmup, "ms_per_step": seconds / steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "triple_cut_4480", "particles": s.n, "substeps_per_step": per, "dt_s": cfg.dt,
                       "schedule_intervals": len(schedule),
                       "step": "one 2 ms ExternalToolPort.advance (graph replay + interval readback) from t = 0"},
            "wall_s_per_simulated_s": seconds / simulated,
            "parallelism": f"replicas x{world}",
        }), flush=True)
    if dist:
        dist.destroy_process_group()


# MLS-MPM step: per particle P2G reads x, v, C, F, damage + impulse (112 B); G2P reads x, F, yield,
# damage, damage_ref (60 B) and writes x, v, C, F, damage, yield (104 B); per touched dense-grid node 56 B.
MLS_BYTES = (276, 56)


def run_gemm(args, rank, world):
    """The predictor's tensor-core GEMM alone (bm_gemm_tn_bf16: bf16 operands, fp32 result) at its
    hidden-layer shape (N = K = 256) over large row counts, CUDA events on the launching stream."""
    import torch

    from blademaster_gb300 import _native, replicas

    dist, rank, world, local = replicas.init()
    torch.cuda.set_device(local)
    lib = _native.lib()
    peak_tf = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["bf16_tflops"] if (ROOT / "MEASURED_PEAKS.json").exists() else 1900.0
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    status = torch.zeros(1, dtype=torch.int32, device=f"cuda:{local}")
    shapes = {}
    for rows in (4096, 32768, 131072):
        a = torch.randn(rows, 256, device=f"cuda:{local}").to(torch.bfloat16).view(torch.int16)
        b = torch.randn(256, 256, device=f"cuda:{local}").to(torch.bfloat16).view(torch.int16)
        d = torch.empty(rows, 256, dtype=torch.float32, device=f"cuda:{local}")
        call = lambda: _native.check(lib.bm_gemm_tn_bf16(p(a), p(b), p(d), rows, 256, 256, None, 0, None, p(status),
                                                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
        for _ in range(max(args.warmup, 3)):
            call()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(args.steps):
            call()
        e1.record()
        torch.cuda.synchronize()
        us = e0.elapsed_time(e1) / args.steps * 1e3
        tflops = 2 * rows * 256 * 256 / (us * 1e-6) / 1e12
        shapes[f"{rows}x256x256"] = {"us": us, "tflops": tflops, "frac_of_bf16_burst": tflops / peak_tf}
    big = shapes["131072x256x256"]
    if rank == 0:
        print(json.dumps({
            "metric": "bm_gemm_tn_bf16 TFLOP/s (predictor hidden layer)", "value": big["tflops"], "unit": "TFLOP/s",
            "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": big["us"] / 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (fp32 accumulate)",
            "data": "synthetic", "config": {"workload": "gemm_tn_bf16", "shapes": shapes, "status": int(status.item())},
            "roofline": {"bound": "tensor", "achieved": big["tflops"], "peak": peak_tf, "unit": "TFLOP/s",
                         "frac": big["frac_of_bf16_burst"], "peak_kind": "of measured bf16 burst"},
        }), flush=True)
    if dist:
        dist.destroy_process_group()


def run_mls(args, rank, world):
    """The MLS-MPM baseline step at the block's scale (1.6 M particles, 2 mm grid, dt 10 us): one held
    knife 1 mm into the top face, one 1 ms interval (100 substeps) per step, replayed as one graph."""
    import torch

    from blademaster_gb300 import replicas, scenes, _native
    from blademaster_gb300.coupling import ToolState
    from blademaster_gb300.mlsmpm import MlsSolver

    dist, rank, world, local = replicas.init()
    torch.cuda.set_device(local)
    cfg, knives, _ = scenes.block_8knives()
    s = MlsSolver(cfg, device=f"cuda:{local}")
    knife = ToolState(knives[3], [0.0, 0.0, 0.0, 1.0], [0.0, 0.0, -0.05], [0.0, 0.0, 0.0])
    per_step = args.substeps or 100
    s.advance(knife, per_step * cfg.dt)  # captures and uploads the interval graph
    graph = s.graphs[per_step]
    for _ in range(args.warmup):
        _native.check(s._lib.bm_graph_launch(graph, s._stream))
    torch.cuda.synchronize()
    clock_file = tempfile.NamedTemporaryFile(suffix=".csv", delete=False).name
    sampler = sample_clocks(clock_file)
    time.sleep(0.5)
    replicas.barrier(dist, torch.cuda.current_device())
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(args.steps):
        _native.check(s._lib.bm_graph_launch(graph, s._stream))
    end.record()
    replicas.barrier(dist, torch.cuda.current_device())
    if sampler:
        time.sleep(0.3)
        sampler.terminate()
        sampler.wait()
    ms = replicas.max_over_ranks(dist, start.elapsed_time(end), torch.cuda.current_device())
    count = ctypes.c_int64()
    _native.check(s._lib.bm_graph_kernel_count(graph, ctypes.byref(count)))
    substeps = args.steps * per_step
    touched = int((s._t["grid_mass"] != 0).sum().item())
    algo = MLS_BYTES[0] * s.n + MLS_BYTES[1] * touched
    rate = algo / (ms / substeps * 1e-3) / 1e9
    peak, peak_kind = peaks()
    diag = s.diagnostics()
    line = {
        "metric": METRIC, "value": world * s.n * substeps / (ms / 1e3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "mls_block_1p6M", "particles": s.n, "grid_nodes": int(np.prod(s.dims)),
                   "touched_nodes": touched, "substeps_per_step": per_step, "dt_s": cfg.dt,
                   "step": f"one {per_step * cfg.dt * 1e3:g} ms interval of the held knife, one graph replay",
                   "l2": "inputs larger than L2 (particle state > 400 MB per substep), no flush",
                   "parallelism": f"replicas x{world}"},
        "ms_per_substep": ms / substeps,
        "gpu_launches": args.steps * count.value,
        "roofline": {"kernel": "whole MLS-MPM substep", "bound": "hbm", "achieved": rate, "peak": peak,
                     "unit": "GB/s", "frac": rate / peak, "peak_kind": f"of {peak_kind}",
                     "algorithmic_bytes": algo, "traffic": None},
        "left_domain": diag["left_domain"], "clamped_inversions": diag["clamped_inversions"],
    }
    line["clocks"] = summarize_clocks(clock_file, torch.cuda.current_device()) if sampler else None
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle.oracle import MlsOracle

        o = MlsOracle(cfg)
        o.advance(knife.position, knife.orientation_xyzw, knife.linear_velocity, knife.angular_velocity, 1)
        steps, begin = 0, time.perf_counter()
        while time.perf_counter() - begin < args.cpu_seconds:
            o.advance(knife.position, knife.orientation_xyzw, knife.linear_velocity, knife.angular_velocity, 1)
            steps += 1
        elapsed = time.perf_counter() - begin
        line["cpu_baseline"] = {"value": o.n * steps / elapsed, "unit": UNIT, "cores": o.L.orc_num_threads(),
                                "kind": "port", "sample": f"{steps} MLS-MPM substeps of the full {o.n}-particle "
                                                          "workload after 1 untimed substep, C oracle with OpenMP"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_reference(args, rank, world):
    if rank != 0:
        return
    name = args.workload
    cfg, _, _ = workload(name)
    budget = max(10.0, min(120.0, 0.5 * (args.steps + args.warmup)))
    base = cpu_baseline(name, seconds=budget, max_steps=args.steps, warmup=args.warmup)
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": base["value"],
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "higher_is_better": True,
        "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": name},
        "cpu_baseline": base,
        "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "vs_baseline": None,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20, help="timed steps (coupling intervals)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--substeps", type=int, default=0,
                    help="substeps per step (default: the workload's coupling interval)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="block_1p6M_8knives")
    ap.add_argument("--e2e-steps", type=int, default=100)
    ap.add_argument("--profile-steps", type=int, default=20)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--eager", action="store_true", help="launch substeps without CUDA graphs (profiling)")
    ap.add_argument("--profile-window", type=int, default=-1,
                    help="profiling: advance this many substeps from t = 0 (graphs), then run --profile-steps eager "
                         "substeps inside a CUDA profiler range (for ncu --profile-from-start off) and exit; "
                         "for triple_cut_4480 this many 2 ms port intervals, then one eager interval")
    ap.add_argument("--instances", type=int, default=256, help="instances of the sweep_c4 workload")
    ap.add_argument("--learned-instances", type=int, default=256, help="training instances of the learned_c5 workload")
    ap.add_argument("--learned-intervals", type=int, default=800, help="training intervals per learned_c5 instance")
    ap.add_argument("--learned-held-intervals", type=int, default=100, help="held-out intervals of learned_c5")
    ap.add_argument("--learned-epochs", type=int, default=25, help="training epochs of the learned_c5 predictor")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "sweep_c4":
        run_sweep(args, rank, world)
        return
    if args.workload == "learned_c5":
        run_learned(args, rank, world)
        return
    if args.workload == "mls_block_1p6M":
        run_mls(args, rank, world)
        return
    if args.workload == "gemm_tn_bf16":
        run_gemm(args, rank, world)
        return
    if args.profile_window >= 0:
        run_profile_window(args)
        return
    if args.workload == "triple_cut_4480":
        run_triple_cut(args, rank, world)
        return
    run_scene(args)


def run_profile_window(args):
    """Eager substeps of a scene workload at a given time, inside a CUDA profiler range."""
    import torch

    from blademaster_gb300 import _native
    from blademaster_gb300.solver import Solver

    if args.workload == "triple_cut_4480":
        # the window counts 2 ms port intervals; the profiled one runs its 32 substeps eagerly
        from blademaster_gb300 import scenes
        from blademaster_gb300.coupling import ExternalToolPort

        s = Solver(scenes.triple_cut_config())
        port = ExternalToolPort(s)
        schedule = scenes.triple_cut_schedule()
        for state, cutting, index in schedule[:args.profile_window]:
            port.advance(state, scenes.TRIPLE_CUT_INTERVAL, cutting=cutting, cut_index=index)
        state, cutting, index = schedule[args.profile_window]
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        port.advance(state, scenes.TRIPLE_CUT_INTERVAL, cutting=cutting, cut_index=index, graph=False)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        print(json.dumps({"workload": args.workload, "particles": s.n, "window_start_interval": args.profile_window,
                          "cutting": bool(cutting), "cut_index": int(index),
                          "eager_substeps": int(round(scenes.TRIPLE_CUT_INTERVAL / s.config.dt))}), flush=True)
        return
    cfg, knives, velocity = workload(args.workload)
    s = Solver(cfg)
    s.tool_pos.assign(knives)
    s.tool_vel.assign(velocity)
    per = SUBSTEPS_PER_STEP.get(args.workload, 100)
    done = 0
    while done < args.profile_window:
        k = min(per, args.profile_window - done)
        s.advance(np.zeros((k, 3)), cutting=True)
        done += k
    torch.cuda.synchronize()
    before = s._t["flags"].cpu().numpy().copy()
    torch.cuda.profiler.start()
    s.advance(np.zeros((args.profile_steps, 3)), cutting=True, graph=False)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    after = s._t["flags"].cpu().numpy()
    events = {k: int(after[_native.FLAG[k]] - before[_native.FLAG[k]]) for k in ("PAIR_BUILDS", "RELISTS", "REGISTRATIONS")}
    print(json.dumps({"workload": args.workload, "particles": s.n, "window_start": args.profile_window,
                      "eager_substeps": args.profile_steps, "events": events}), flush=True)


def run_scene(args):
    import torch

    from blademaster_gb300 import replicas

    dist, rank, world, local = replicas.init()
    torch.cuda.set_device(local)

    from blademaster_gb300 import _native
    from blademaster_gb300.solver import Solver

    cfg, knives, velocity = workload(args.workload)
    s = Solver(cfg, device=f"cuda:{local}")
    s.tool_pos.assign(knives)
    s.tool_vel.assign(velocity)
    per_step = args.substeps or SUBSTEPS_PER_STEP.get(args.workload, 100)
    zeros = np.zeros((per_step, 3))
    start_of_run = s.checkpoint()  # t = 0: the timed steps and the end-to-end steps both start here

    def run(steps, graph=True):
        for _ in range(steps):
            s.advance(zeros, cutting=True, graph=graph and not args.eager)

    run(args.warmup)  # graph capture and upload, first touch of every array

    count = ctypes.c_int64()
    _native.check(s._lib.bm_graph_kernel_count(s.prepare(zeros, True, 0), ctypes.byref(count)))
    timed_launches = args.steps * count.value  # eager runs launch the same kernels
    s.restore(start_of_run)
    torch.cuda.synchronize()
    clock_file = tempfile.NamedTemporaryFile(suffix=".csv", delete=False).name
    sampler = sample_clocks(clock_file)
    time.sleep(0.5)
    replicas.barrier(dist, torch.cuda.current_device())
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    counters_before = s._t["flags"].cpu().numpy().copy()
    start.record()
    run(args.steps)
    end.record()
    replicas.barrier(dist, torch.cuda.current_device())
    if sampler:
        time.sleep(0.3)
        sampler.terminate()
        sampler.wait()
    ms = replicas.max_over_ranks(dist, start.elapsed_time(end), torch.cuda.current_device())
    substeps = args.steps * per_step
    slots = int(s._t["nfield"].sum().item())
    counters_after = s._t["flags"].cpu().numpy()
    errors = s.errors.numpy().tolist()
    final_tool = s._t["tool"].cpu().numpy()

    def delta(name):
        return int(counters_after[_native.FLAG[name]] - counters_before[_native.FLAG[name]])

    events = {
        "pair_list_builds": delta("PAIR_BUILDS"),
        "relists": delta("RELISTS"),
        "registrations": delta("REGISTRATIONS"),
        "multi_field_nodes": int(counters_after[_native.FLAG["MULTI"]]),
        "mixed_cells": int(counters_after[_native.FLAG["MIXED_CELLS"]]),
        "simulated_s": substeps * cfg.dt,
    }
    value = world * s.n * substeps / (ms / 1e3)

    # per-stage device time (CUDA events around each stage, eager launches), after the timed run
    stage_ms = (ctypes.c_float * len(_native.STAGES))()
    a = s._step_args(args.profile_steps, True, 0, use_targets=0)
    s._sync_step()
    _native.check(s._lib.bm_substeps_profiled(s._handle, ctypes.byref(a), stage_ms, s._stream))
    s._advanced(args.profile_steps)
    stages = {name: stage_ms[i] / args.profile_steps for i, name in enumerate(_native.STAGES)}
    dominant = max(SINGLE_KERNEL_STAGES, key=lambda k: stages[k])
    per_particle, per_slot = STAGE_BYTES[dominant]
    algo = per_particle * s.n + per_slot * slots
    achieved = algo / (stages[dominant] * 1e-3) / 1e9
    peak, peak_kind = peaks()
    stage_rooflines = {}
    for name, (bp, bs) in STAGE_BYTES.items():
        rate = (bp * s.n + bs * slots) / (stages[name] * 1e-3) / 1e9
        stage_rooflines[name] = {"achieved_gbs": round(rate, 1), "frac": round(rate / peak, 4),
                                 "traffic": traffic_per_launch(name, s.n, slots)}
    substep_bytes = SUBSTEP_BYTES[0] * s.n + SUBSTEP_BYTES[1] * slots
    substep_rate = substep_bytes / (ms / substeps * 1e-3) / 1e9

    # End to end through the public API, as a caller drives the solver, over
    # the same intervals from the same t = 0 state as the timed region: each
    # Solver.advance call copies its host targets in (targets and orientations,
    # 28 B a substep) and replays the interval's graph, and the caller reads
    # the float64 knife state back to pinned host memory and synchronises.
    pinned_state = torch.zeros(s._t["tool"].shape, dtype=torch.float64).pin_memory()

    def end_to_end(per_call, calls):
        host_targets = np.zeros((per_call, 3))
        s.advance(host_targets, True, 0)  # the graph exists before the timing
        s.restore(start_of_run)
        torch.cuda.synchronize()
        begin = time.perf_counter()
        for _ in range(calls):
            s.advance(host_targets, True, 0)
            pinned_state.copy_(s._t["tool"], non_blocking=True)
            torch.cuda.current_stream().synchronize()
        seconds = replicas.max_over_ranks(dist, time.perf_counter() - begin, torch.cuda.current_device())
        return world * s.n * per_call * calls / seconds

    e2e_value = end_to_end(per_step, args.steps)
    e2e_same = bool(np.array_equal(pinned_state.numpy(), final_tool))
    e2e_single = end_to_end(1, args.e2e_steps)

    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {
            "workload": args.workload,
            "particles": s.n,
            "registered_slots": slots,
            "substeps_per_step": per_step,
            "dt_s": cfg.dt,
            "step": f"one {per_step * cfg.dt * 1e3:g} ms interval ({per_step} substeps, one graph replay); the "
                    "timed steps restart from the t = 0 checkpoint after the warm-up",
            "l2": "inputs larger than L2 (particle state > 400 MB per substep), no flush"
                  if s.n > 1_000_000 else "small scene: the particle state fits in L2",
            "parallelism": f"replicas x{world}",
        },
        "ms_per_substep": ms / substeps,
        "gpu_launches": timed_launches,
        "stage_ms": {k: round(v, 5) for k, v in stages.items()},
        "roofline": {
            "kernel": SINGLE_KERNEL_STAGES[dominant],
            "bound": "hbm",
            "achieved": achieved,
            "peak": peak,
            "unit": "GB/s",
            "frac": achieved / peak,
            "peak_kind": f"of {peak_kind}",
            "algorithmic_bytes": algo,
            "traffic": traffic_per_launch(dominant, s.n, slots),
        },
        "stage_rooflines": stage_rooflines,
        "substep_roofline": {"algorithmic_bytes": substep_bytes, "achieved_gbs": round(substep_rate, 1),
                             "frac": round(substep_rate / peak, 4)},
        "e2e": {
            "value": e2e_value,
            "unit": UNIT,
            "h2d_bytes_per_step": 28 * per_step,
            "d2h_bytes_per_step": int(pinned_state.numel() * 8),
            "substeps_per_step": per_step,
            "call": "Solver.advance(host targets) per interval + knife state read back, same intervals from t = 0",
            "same_final_knife_state": e2e_same,
        },
        "e2e_single_substep": {"value": e2e_single, "unit": UNIT, "h2d_bytes_per_step": 28,
                               "d2h_bytes_per_step": int(pinned_state.numel() * 8)},
        "device_errors": errors,
        "timed_region_events": events,
    }
    clocks = summarize_clocks(clock_file, torch.cuda.current_device()) if sampler else None
    line["clocks"] = clocks
    if rank == 0 and world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args.workload, seconds=args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
