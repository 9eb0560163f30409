"""Learned tool predictor: an MLP that predicts the knife wrench of a coupling interval.

It stands in for the linear mobility prediction of ``tool_substep="predict"``
(blademaster_warp/tool.py:97-113): inputs are the knife pose and velocity
(13), the cut depth (1), the material (3) and 64 pooled occupancies of the
particles around the edge; the output is the interval's force and torque
(6).  Layers 81 -> 256 -> 256 -> 256 -> 6 with ReLU, bf16 weights and
activations, fp32 accumulation.  Every GEMM of training and inference runs on
the tensor cores through bm_gemm_tn_bf16 (tcgen05); the elementwise steps
(transposes, ReLU backward, loss gradient, bias sums, Adam) are the library's
own kernels.  The plain substeps stay the referee: ``GatedPredictor`` accepts a
prediction only within 1 % of the plain interval's wrench.
"""

import ctypes
import math

import numpy as np

from . import _native

IN, HIDDEN, OUT = 81, 256, 6
IN_PAD, OUT_PAD = 96, 16  # GEMM K multiple of 32 for the input, N multiple of 16 for the output
OUT_WITH_STATE = 12  # the wrench and the knife's twist change over the interval
LAYERS = ((HIDDEN, IN_PAD), (HIDDEN, HIDDEN), (HIDDEN, HIDDEN), (OUT_PAD, HIDDEN))  # (out, in) of each weight


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class ToolPredictor:
    """The MLP with its training state; tensors live on `device`."""

    def __init__(self, device="cuda:0", seed=0, outputs=OUT):
        import torch

        if not 1 <= outputs <= OUT_PAD:
            raise ValueError(f"outputs must be in [1, {OUT_PAD}]")
        self.outputs = outputs
        self.device = torch.device(device)
        self._lib = _native.lib()
        rng = np.random.default_rng(seed)
        self.w, self.b, self.wh, self.wt = [], [], [], []
        for i, (fan_out, fan_in) in enumerate(LAYERS):
            real_in = IN if i == 0 else fan_in
            real_out = outputs if i == len(LAYERS) - 1 else fan_out
            w = np.zeros((fan_out, fan_in), np.float32)
            w[:real_out, :real_in] = rng.normal(0.0, math.sqrt(2.0 / real_in), (real_out, real_in))
            self.w.append(torch.as_tensor(w, device=self.device))
            self.b.append(torch.zeros(fan_out, dtype=torch.float32, device=self.device))
            self.wh.append(torch.zeros(fan_out, fan_in, dtype=torch.int16, device=self.device))
            self.wt.append(None)
        self.adam = [[torch.zeros_like(t) for t in (w, w, b, b)] for w, b in zip(self.w, self.b)]
        self.steps = 0
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.feature_mean = np.zeros(IN, np.float32)
        self.feature_std = np.ones(IN, np.float32)
        self.target_mean = np.zeros(outputs, np.float32)
        self.target_std = np.ones(outputs, np.float32)
        self._refresh()

    @property
    def _stream(self):
        import torch

        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _refresh(self):
        """bf16 copies of the weights and the transposes the backward GEMMs use."""
        import torch

        for i, w in enumerate(self.w):
            out, inp = w.shape
            _native.check(self._lib.bm_mlp_cast_bf16(_p(w), out, inp, inp, _p(self.wh[i]), self._stream))
            if i == 0:
                continue
            # W^T with the reduction (out) padded to a multiple of 32 for dX = dY W
            pad = -(-out // 32) * 32
            wt = torch.zeros(inp, pad, dtype=torch.int16, device=self.device)
            t = torch.empty(inp, out, dtype=torch.int16, device=self.device)
            _native.check(self._lib.bm_mlp_transpose16(_p(self.wh[i]), _p(t), out, inp, self._stream))
            wt[:, :out] = t
            self.wt[i] = wt

    def _gemm(self, A, B, M, N, K, D=None, bias=None, relu=False, Dh=None):
        _native.check(self._lib.bm_gemm_tn_bf16(_p(A), _p(B), _p(D), M, N, K, _p(bias), int(relu), _p(Dh), _p(self.status),
                                                self._stream))

    def _transpose(self, x):
        import torch

        rows, cols = x.shape
        out = torch.empty(cols, rows, dtype=torch.int16, device=self.device)
        _native.check(self._lib.bm_mlp_transpose16(_p(x), _p(out), rows, cols, self._stream))
        return out

    def forward(self, xh):
        """xh: [B x 96] bf16 inputs; returns fp32 outputs [B x 16] and keeps the activations."""
        import torch

        rows = xh.shape[0]
        acts = [xh]
        for i in range(3):
            h = torch.empty(rows, HIDDEN, dtype=torch.int16, device=self.device)
            self._gemm(acts[-1], self.wh[i], rows, HIDDEN, LAYERS[i][1], bias=self.b[i], relu=True, Dh=h)
            acts.append(h)
        y = torch.empty(rows, OUT_PAD, dtype=torch.float32, device=self.device)
        self._gemm(acts[-1], self.wh[3], rows, OUT_PAD, HIDDEN, D=y, bias=self.b[3])
        self._acts = acts
        return y

    def backward(self, y, target):
        """Gradients of the mean squared error against target [B x 6] (fp32); returns the loss."""
        import torch

        rows = y.shape[0]
        if rows % 32:
            raise ValueError("training batches must hold a multiple of 32 samples")
        dev = self.device
        loss = torch.zeros(1, dtype=torch.float32, device=dev)
        g = torch.empty(rows, OUT_PAD, dtype=torch.float32, device=dev)
        gh = torch.zeros(rows, 32, dtype=torch.int16, device=dev)  # reduction padded to 32 for dH = dY W
        gh16 = torch.empty(rows, OUT_PAD, dtype=torch.int16, device=dev)
        _native.check(self._lib.bm_mlp_mse_grad(_p(y), _p(target), rows, self.outputs, OUT_PAD, _p(g), _p(gh16), _p(loss),
                                                self._stream))
        gh[:, :OUT_PAD] = gh16
        self.grads = [None] * 4
        for i in range(3, -1, -1):
            out, inp = LAYERS[i]
            grad_w = torch.empty(out, inp, dtype=torch.float32, device=dev)
            grad_b = torch.empty(out, dtype=torch.float32, device=dev)
            g_half = gh[:, :out] if i == 3 else gh
            self._gemm(self._transpose(g_half.contiguous()), self._transpose(self._acts[i]), out, inp, rows, D=grad_w)
            _native.check(self._lib.bm_mlp_colsum(_p(g), rows, out, _p(grad_b), self._stream))
            self.grads[i] = (grad_w, grad_b)
            if i == 0:
                break
            # dH = dY W (fp32), then through the ReLU of the layer below
            dh = torch.empty(rows, inp, dtype=torch.float32, device=dev)
            self._gemm(gh, self.wt[i], rows, inp, gh.shape[1], D=dh)
            g = dh
            gh = torch.empty(rows, inp, dtype=torch.int16, device=dev)
            _native.check(self._lib.bm_mlp_relu_grad(_p(g), _p(self._acts[i]), _p(gh), g.numel(), self._stream))
        return float(loss.item())

    def step(self, lr=1.0e-3, beta1=0.9, beta2=0.999, eps=1.0e-8):
        self.steps += 1
        for (w, b), (gw, gb), (mw, vw, mb, vb), wh in zip(zip(self.w, self.b), self.grads, self.adam, self.wh):
            _native.check(self._lib.bm_mlp_adam(_p(w), _p(gw), _p(mw), _p(vw), _p(wh), w.numel(), lr, beta1, beta2, eps,
                                                self.steps, self._stream))
            _native.check(self._lib.bm_mlp_adam(_p(b), _p(gb), _p(mb), _p(vb), None, b.numel(), lr, beta1, beta2, eps,
                                                self.steps, self._stream))
        self._refresh()

    def _inputs(self, features):
        import torch

        x = (np.asarray(features, np.float32) - self.feature_mean) / self.feature_std
        xf = torch.as_tensor(np.ascontiguousarray(x, np.float32), device=self.device)
        xh = torch.empty(x.shape[0], IN_PAD, dtype=torch.int16, device=self.device)
        _native.check(self._lib.bm_mlp_cast_bf16(_p(xf), x.shape[0], IN, IN_PAD, _p(xh), self._stream))
        return xh

    def fit(self, features, wrenches, epochs=200, batch=256, lr=1.0e-3, seed=0):
        """Train on (features [S x 81], targets [S x outputs]); returns the loss of each epoch."""
        import torch

        features = np.asarray(features, np.float32)
        wrenches = np.asarray(wrenches, np.float32)
        self.feature_mean, self.feature_std = features.mean(0), features.std(0) + 1.0e-6
        self.target_mean, self.target_std = wrenches.mean(0), wrenches.std(0) + 1.0e-9
        xh = self._inputs(features)
        t = torch.as_tensor((wrenches - self.target_mean) / self.target_std, device=self.device)
        rng = np.random.default_rng(seed)
        count = (len(features) // batch) * batch
        if count == 0:
            raise ValueError(f"need at least {batch} samples")
        history = []
        for _ in range(epochs):
            order = torch.as_tensor(rng.permutation(len(features))[:count], device=self.device)
            total = 0.0
            for start in range(0, count, batch):
                idx = order[start : start + batch]
                y = self.forward(xh[idx].contiguous())
                total += self.backward(y, t[idx].contiguous())
                self.step(lr)
            history.append(total / (count // batch))
        return history

    def predict(self, features):
        """Outputs [B x outputs] (force and torque first) for feature rows [B x 81]."""
        y = self.forward(self._inputs(np.atleast_2d(features)))
        if int(self.status.item()):
            raise RuntimeError("tensor-core GEMM did not complete")
        return y[:, : self.outputs].cpu().numpy() * self.target_std + self.target_mean


def features_batch(solvers, states, material_top):
    """``features`` of many solvers, their pooling kernels queued back to back and read with one copy."""
    import torch

    solvers, states = list(solvers), [st.checked() for st in states]
    if not solvers:
        return np.zeros((0, IN), np.float32)
    device = solvers[0].device
    lib = _native.lib()
    counts = torch.zeros(len(solvers), 64, dtype=torch.int32, device=device)
    records = np.zeros((len(solvers), _native.TOOL_F_WORDS), np.float32)
    for i, (solver, st) in enumerate(zip(solvers, states)):
        records[i] = _knife_record(solver, st)
    tools = torch.as_tensor(records, device=device)
    for i, solver in enumerate(solvers):
        cfg = solver.config
        _native.check(lib.bm_mlp_pool(_p(solver._t["x"]), solver.n, _p(tools[i]), cfg.grid_spacing,
                                      cfg.blade_half_size[1], _p(counts[i]), solver._stream))
    counts = counts.cpu().numpy()
    return np.stack([_assemble(solver, st, material_top, c) for solver, st, c in zip(solvers, states, counts)])


def _knife_record(solver, st):
    """float32 knife record of the upcoming pose: orientation (words 6-9) and edge centre (15-17)."""
    cfg = solver.config
    record = np.zeros(_native.TOOL_F_WORDS, np.float32)
    q = np.asarray(st.orientation_xyzw, np.float64)
    record[0:3], record[6:10] = st.position, q
    x, y, z, w = q
    down = np.array([-(2 * (x * z + w * y)), -(2 * (y * z - w * x)), -(1 - 2 * (x * x + y * y))])
    record[15:18] = np.asarray(st.position) + cfg.blade_half_size[2] * down
    return record


def _assemble(solver, st, material_top, counts):
    cfg = solver.config
    h, half_y = cfg.grid_spacing, cfg.blade_half_size[1]
    full = (2 * h) * (0.5 * half_y) * (2 * h) / solver.volume
    centroid = solver.reference.mean(0)
    edge_z = st.position[2] - cfg.blade_half_size[2]
    head = np.concatenate([np.asarray(st.position) - centroid, st.orientation_xyzw, st.linear_velocity, st.angular_velocity,
                           [material_top - edge_z], [math.log10(cfg.young_modulus), cfg.poisson_ratio, cfg.density / 1000.0]])
    return np.concatenate([head, counts / full]).astype(np.float32)


def features(solver, state, material_top):
    """Predictor inputs for a solver whose knife 0 is at `state` (81 values).

    Pose (position relative to the reference centroid, orientation) and twist,
    the cut depth (material top minus edge height), the material (log10 E,
    nu, rho / 1000) and the 64 bin occupancies (count / particles a full bin holds).
    """
    return features_batch([solver], [state], material_top)[0]


class GatedPredictor:
    """The plain substeps as the referee of the predictor (1 % wrench tolerance).

    ``advance`` predicts the interval's wrench, runs the plain interval through
    the port, and accepts the prediction only if the force and torque are each
    within `tolerance` of the plain ones (relative to the plain magnitude);
    otherwise the plain wrench is used.  Counts the accepted intervals.
    """

    def __init__(self, port, predictor, material_top, tolerance=0.01):
        self.port, self.predictor, self.material_top, self.tolerance = port, predictor, material_top, tolerance
        self.accepted = 0
        self.intervals = 0

    def advance(self, state, duration_s, **kw):
        predicted = self.predictor.predict(features(self.port.solver, state, self.material_top))[0]
        reaction = self.port.advance(state, duration_s, **kw)
        plain = np.concatenate([reaction.impulse_ns, reaction.angular_impulse_nms]) / duration_s
        ok = all(
            np.linalg.norm(predicted[i : i + 3] - plain[i : i + 3]) <= self.tolerance * max(np.linalg.norm(plain[i : i + 3]), 1e-12)
            for i in (0, 3)
        )
        self.intervals += 1
        self.accepted += int(ok)
        return reaction, predicted, ok
