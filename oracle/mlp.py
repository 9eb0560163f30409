"""CPU ORACLE of the learned tool predictor - test infrastructure, not part of the product.

Float64 numpy forward and backward of the MLP (81 -> 256 -> 256 -> 256 -> 6,
ReLU, mean squared error) with bf16 rounding at the same points as the GPU
kernels: the inputs, the weights, each hidden activation, and each loss /
layer gradient before it enters a GEMM.  Used to check the GPU gradients.
"""

import numpy as np


def bf16(x):
    """Round to bfloat16 (nearest even) and return float64 values."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint32)
    return (rounded << 16).view(np.float32).astype(np.float64)


def forward(x, weights, biases):
    """x [B x 96] (already bf16 values), weights [(out x in)], biases [(out,)]: activations and outputs."""
    acts = [x]
    for w, b in zip(weights[:3], biases[:3]):
        acts.append(bf16(np.maximum(acts[-1] @ bf16(w).T + b, 0.0)))
    y = acts[-1] @ bf16(weights[3]).T + biases[3]
    return acts, y


def backward(acts, y, target, weights, outputs=6):
    """Gradients (dW, db) of the mean squared error over the first `outputs` columns."""
    rows = y.shape[0]
    g = np.zeros_like(y)
    g[:, :outputs] = 2.0 * (y[:, :outputs] - target) / (rows * outputs)
    grads = [None] * 4
    for i in range(3, -1, -1):
        gh = bf16(g)
        grads[i] = (gh.T @ acts[i], g.sum(0))
        if i == 0:
            break
        g = (gh @ bf16(weights[i])) * (acts[i] > 0)
    return grads
