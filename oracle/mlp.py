"""FP64 restatement of the learned subpixel network.  TEST INFRASTRUCTURE ONLY.

The checker for the library's own network kernels (libbicos_gb300/csrc/
learned.cu): the forward pass, the loss 0.5 (y - target)^2 summed over a
batch and its gradient with respect to every parameter, written out by hand
in float64 numpy, plus the inference path with the BF16 roundings the
tensor-core kernel applies.  Nothing in the product imports it.

The network has no counterpart in libBICOS; its inputs come from the
correlations the reference's agreement stage computes (include/impl/cuda/
agree.cuh:35-97 at integer offsets), and its target is the offset the
reference's subpixel sweep picks (agree.cuh:161-259).

Model layout (floats): W1[64][7], b1[64], W2[64][64], b2[64], w3[64], b3,
then mean[7], std[7] of the network inputs.
"""
from __future__ import annotations

import math

import numpy as np

N_IN, N_H = 7, 64
W1, B1 = 0, N_H * N_IN
W2 = B1 + N_H
B2 = W2 + N_H * N_H
W3 = B2 + N_H
B3 = W3 + N_H
N_PARAMS = B3 + 1
NORM = N_PARAMS
MODEL_FLOATS = N_PARAMS + 2 * N_IN

GELU_C = math.sqrt(2.0 / math.pi)
GELU_A = 0.044715


def unpack(model):
    m = np.asarray(model, np.float64)
    return (m[W1:B1].reshape(N_H, N_IN), m[B1:W2], m[W2:B2].reshape(N_H, N_H), m[B2:W3], m[W3:B3], m[B3],
            m[NORM:NORM + N_IN], m[NORM + N_IN:NORM + 2 * N_IN])


def raw_inputs(feats):
    """Network inputs before normalisation from (N, >=7) feature rows."""
    f = np.asarray(feats, np.float64)
    r = np.where(np.isfinite(f[:, :5]), f[:, :5], -1.0)
    return np.stack([r[:, 2], r[:, 1] - r[:, 2], r[:, 3] - r[:, 2], r[:, 0] - r[:, 2], r[:, 4] - r[:, 2],
                     np.log1p(np.maximum(np.nan_to_num(f[:, 5], nan=0.0), 0.0)),
                     np.log1p(np.maximum(np.nan_to_num(f[:, 6], nan=0.0), 0.0))], axis=1)


def inputs(feats, mean, std):
    return (raw_inputs(feats) - mean) / std


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(GELU_C * (z + GELU_A * z ** 3)))


def gelu_grad(z):
    t = np.tanh(GELU_C * (z + GELU_A * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * GELU_C * (1.0 + 3.0 * GELU_A * z * z)


def forward(model, feats):
    w1, b1, w2, b2, w3, b3, mean, std = unpack(model)
    x = inputs(feats, mean, std)
    z1 = x @ w1.T + b1
    h1 = gelu(z1)
    z2 = h1 @ w2.T + b2
    h2 = gelu(z2)
    y = np.tanh(h2 @ w3 + b3)
    return y, (x, z1, h1, z2, h2)


def loss_and_grad(model, samples):
    """samples: (N, 8), feature rows with the target offset in the last
    column.  Returns (sum of 0.5 (y - t)^2, gradient over the parameters)."""
    s = np.asarray(samples, np.float64)
    w1, b1, w2, b2, w3, b3, mean, std = unpack(model)
    y, (x, z1, h1, z2, h2) = forward(model, s)
    dy = y - s[:, 7]
    loss = 0.5 * float(np.sum(dy * dy))
    dz3 = dy * (1.0 - y * y)
    dz2 = np.outer(dz3, w3) * gelu_grad(z2)
    dz1 = (dz2 @ w2) * gelu_grad(z1)
    g = np.zeros(N_PARAMS)
    g[W1:B1] = (dz1.T @ x).ravel()
    g[B1:W2] = dz1.sum(0)
    g[W2:B2] = (dz2.T @ h1).ravel()
    g[B2:W3] = dz2.sum(0)
    g[W3:B3] = h2.T @ dz3
    g[B3] = dz3.sum()
    return loss, g


def bf16(a):
    """float32 values rounded to the nearest BF16 (ties to even), as float32."""
    b = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return b.astype(np.uint32).view(np.float32)


def propose(model, feats):
    """Inference as the tensor-core kernel evaluates it: parameters rounded
    to BF16, layer 1 in (here) float64, its activations rounded to BF16
    for the tensor-core layer, the rest in float64."""
    m = np.array(model, np.float32)
    m[:N_PARAMS] = bf16(m[:N_PARAMS])
    w1, b1, w2, b2, w3, b3, mean, std = unpack(m)
    x = inputs(feats, mean, std)
    h1 = bf16(gelu(x @ w1.T + b1)).astype(np.float64)
    h2 = gelu(h1 @ w2.T + b2)
    return np.tanh(h2 @ w3 + b3)


def adam_step(params, grad, m, v, step, lr, scale):
    """Adam with bias correction (Kingma & Ba 2015), as k_mlp_adam."""
    g = grad * scale
    m = 0.9 * m + 0.1 * g
    v = 0.999 * v + 0.001 * g * g
    mh = m / (1.0 - 0.9 ** step)
    vh = v / (1.0 - 0.999 ** step)
    return params - lr * mh / (np.sqrt(vh) + 1e-8), m, v
