"""Learned tool predictor: tensor-core forward/backward checked against the
float64 oracle, training on intervals the batched solver generates, the gain
over the method without it (predicting the training mean), and the 1 % gate
against the plain substeps."""

import numpy as np
import pytest

from oracle import mlp as ref

pytestmark = pytest.mark.gpu


def test_gradients_match_the_float64_oracle():
    import torch

    from blademaster_gb300.predictor import IN, IN_PAD, OUT, ToolPredictor

    p = ToolPredictor(seed=1)
    rng = np.random.default_rng(2)
    rows = 128
    x = rng.normal(size=(rows, IN)).astype(np.float32)
    target = rng.normal(size=(rows, OUT)).astype(np.float32)
    xh = p._inputs(x)
    y = p.forward(xh)
    p.backward(y, torch.as_tensor(target, device=p.device))
    weights = [w.cpu().numpy().astype(np.float64) for w in p.w]
    biases = [b.cpu().numpy().astype(np.float64) for b in p.b]
    xin = np.zeros((rows, IN_PAD))
    xin[:, :IN] = ref.bf16(x)
    acts, y_ref = ref.forward(xin, weights, biases)
    np.testing.assert_allclose(y.cpu().numpy(), y_ref, rtol=2e-3, atol=2e-3 * np.abs(y_ref).max())
    grads = ref.backward(acts, y_ref, target.astype(np.float64), weights)
    for i, ((gw, gb), (rw, rb)) in enumerate(zip(p.grads, grads)):
        gw, gb = gw.cpu().numpy(), gb.cpu().numpy()
        assert np.linalg.norm(gw - rw) <= 1e-2 * np.linalg.norm(rw), f"dW layer {i}"
        assert np.linalg.norm(gb - rb) <= 1e-2 * np.linalg.norm(rb), f"db layer {i}"


def collect(count, intervals, seed):
    """(features, wrench) of every interval of a small batched sweep."""
    from blademaster_gb300.batch import SolverBatch
    from blademaster_gb300.predictor import features
    from blademaster_gb300.solver import Solver
    from blademaster_gb300.sweep import RADIUS, instances

    sweep = instances(count, seed=seed, spacings=(0.006,))
    solvers = [Solver(i.config) for i in sweep]
    batch = SolverBatch(solvers, lanes=count)
    xs, ys = [], []
    for k in range(intervals):
        states = [i.state(k, start_gap=-0.0005) for i in sweep]
        xs.extend(features(s, st, 2 * RADIUS) for s, st in zip(solvers, states))
        for r in batch.advance(states, 0.001, strict=False):
            ys.append(np.concatenate([r.impulse_ns, r.angular_impulse_nms]) / 0.001)
    return np.array(xs), np.array(ys)


def test_training_beats_the_mean_predictor_on_held_out_intervals():
    from blademaster_gb300.predictor import ToolPredictor

    x, y = collect(16, 48, seed=11)
    interval = np.arange(len(x)) // 16  # rows are interval-major, 16 instances each
    train, test = interval % 2 == 0, interval % 2 == 1
    p = ToolPredictor(seed=0)
    history = p.fit(x[train], y[train], epochs=80, batch=64, lr=2e-3)
    assert history[-1] < 0.5 * history[0]
    mean_error = np.linalg.norm(y[test] - y[train].mean(0), axis=1).mean()
    mlp_error = np.linalg.norm(p.predict(x[test]) - y[test], axis=1).mean()
    print(f"held-out wrench error: MLP {mlp_error:.4g}, training mean {mean_error:.4g}")
    assert mlp_error < 0.5 * mean_error


def test_gate_accepts_only_predictions_within_one_percent():
    from blademaster_gb300.coupling import ExternalToolPort
    from blademaster_gb300.predictor import GatedPredictor, ToolPredictor
    from blademaster_gb300.solver import Solver
    from blademaster_gb300.sweep import RADIUS, instances

    inst = instances(1, seed=5, spacings=(0.006,))[0]
    s = Solver(inst.config)
    gate = GatedPredictor(ExternalToolPort(s), ToolPredictor(seed=3), 2 * RADIUS)
    for k in range(4):
        reaction, predicted, ok = gate.advance(inst.state(k, start_gap=-0.0005), 0.001)
        plain = np.concatenate([reaction.impulse_ns, reaction.angular_impulse_nms]) / 0.001
        close = np.linalg.norm(predicted[:3] - plain[:3]) <= 0.01 * np.linalg.norm(plain[:3])
        assert ok == (close and np.linalg.norm(predicted[3:] - plain[3:]) <= 0.01 * max(np.linalg.norm(plain[3:]), 1e-12))
    assert gate.intervals == 4
