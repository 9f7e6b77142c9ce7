"""CPU reference of the surrogate MLP's forward and backward passes.

TEST INFRASTRUCTURE ONLY (gradient checks of the GPU kernels).  Float64
arithmetic throughout, with bf16 rounding applied exactly where the GPU
kernels store bf16 (activations, output, activation gradients), so the
comparison isolates the kernels' FP32 accumulation order.
"""
import numpy as np

C = np.sqrt(2.0 / np.pi)


def bf16_round(x):
    """Round float values to bfloat16 (round to nearest even), returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = ((u + 0x7FFF + lsb) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def bf16_bits(x):
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    return (((u + 0x7FFF + lsb) >> 16) & 0xFFFF).astype(np.uint16)


def from_bits(b):
    return (np.asarray(b, dtype=np.uint32) << 16).view(np.float32).astype(np.float64)


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(C * (x + 0.044715 * x ** 3)))


def gelu_grad(x):
    t = np.tanh(C * (x + 0.044715 * x ** 3))
    return 0.5 * (1 + t) + 0.5 * x * (1 - t * t) * C * (1 + 3 * 0.044715 * x * x)


def forward(weights, biases, x, acts):
    """weights: list of [N, K] float64 (already bf16-valued); x: [M, K0]
    bf16-valued.  Returns (inputs, pres, y): the hidden activations are
    bf16-rounded as the GPU stores them; the output y is the last layer's
    pre-activation, kept in full precision (the GPU keeps it in FP32)."""
    h = x
    inputs, pres = [], []
    for w, b, act in zip(weights, biases, acts):
        inputs.append(h)
        pre = h @ w.T + b
        pres.append(pre)
        h = bf16_round(gelu(pre) if act else pre)
    return inputs, pres, pres[-1]


def backward(weights, inputs, pres, dy, acts):
    """dy bf16-valued [M, N_last].  Returns (dW list, db list) in float64."""
    dws, dbs = [None] * len(weights), [None] * len(weights)
    g = dy
    for i in range(len(weights) - 1, -1, -1):
        dpre = g * gelu_grad(pres[i]) if acts[i] else g
        dbs[i] = dpre.sum(0)
        dpre_b = bf16_round(dpre)
        dws[i] = dpre_b.T @ inputs[i]
        if i > 0:
            g = bf16_round(dpre_b @ weights[i])
    return dws, dbs


def loss_grad(y, t, n_valid, mode=0, scale=1.0, weights=None, clip=4.0):
    """Loss and bf16-rounded output gradient of mcgb_mlp_loss_grad: mode 0
    squared error, mode 1 relative error of exp(scale*y) against a linear
    target (the gradient clips the ratio at ``clip``)."""
    m, n = y.shape
    w = np.ones(n) if weights is None else np.asarray(weights, np.float64)
    yv, tv = y[:, :n_valid], t[:, :n_valid]
    g = np.zeros_like(y)
    if mode == 0:
        d = yv - tv
        loss = (w[:n_valid] * d ** 2).sum() / (m * n_valid)
        g[:, :n_valid] = 2.0 * w[:n_valid] * d / (m * n_valid)
    else:
        ratio = tv * np.exp(-scale * yv)
        loss = (w[:n_valid] * (ratio - 1.0) ** 2).sum() / (m * n_valid)
        g[:, :n_valid] = -2.0 * scale * w[:n_valid] * (np.minimum(ratio, clip) - 1.0) / (m * n_valid)
    return bf16_round(g), loss
