"""FP64 restatement of the surrogate MLP with the CUDA path's BF16 roundings.

TEST INFRASTRUCTURE ONLY: the checker for the tensor-core MLP kernels.
The GPU rounds to bfloat16 (round to nearest even) at exactly these points:
the packed input, the weight copies, every hidden activation after ReLU,
the output gradient dY and every masked pre-activation gradient.  This
oracle rounds at the same points and does all arithmetic in FP64, so the
two differ only by the GPU's FP32 accumulation order.
"""
import numpy as np


def bf16(x):
    """Round float values to bfloat16 (nearest even), returned as float64."""
    f = np.ascontiguousarray(np.asarray(x, np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params, dims):
    out, o = [], 0
    for l in range(1, len(dims)):
        n = dims[l] * dims[l - 1]
        W = params[o:o + n].reshape(dims[l], dims[l - 1]).astype(np.float64)
        o += n
        b = params[o:o + dims[l]].astype(np.float64)
        o += dims[l]
        out.append((W, b))
    return out


def forward(params, dims, X):
    layers = unpack(params, dims)
    H = bf16(X)
    acts = [H]
    for i, (W, b) in enumerate(layers):
        Z = H @ bf16(W).T + b
        if i < len(layers) - 1:
            H = bf16(np.maximum(Z, 0.0))
            acts.append(H)
        else:
            return Z, acts
    raise AssertionError


def loss_and_grads(params, dims, X, T):
    """MSE loss and its gradient in the flat parameter layout."""
    layers = unpack(params, dims)
    Y, acts = forward(params, dims, X)
    B, d = Y.shape
    E = Y - T
    loss = float(np.sum(E * E) / (B * d))
    dZ = bf16(2.0 * E / (B * d))
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        W, _ = layers[l]
        Hp = acts[l]
        gW = dZ.T @ Hp
        gb = dZ.sum(0)
        grads[l] = (gW, gb)
        if l > 0:
            dH = dZ @ bf16(W)
            dZ = bf16(dH * (Hp > 0))
    flat = np.concatenate([np.concatenate([g[0].ravel(), g[1]]) for g in grads])
    return loss, flat
