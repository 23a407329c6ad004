"""CPU restatement of the learned block-screening MLP (test infrastructure only).

Checks the GPU forward / backward kernels of librpa_gb300/csrc/screen.cu: a 9-64-64-1 network
with GELU activations, parameters rounded to FP16 (the GPU stores FP16 weights and
accumulates in FP32; this restatement accumulates in FP64), normalised inputs and targets,
and the mean squared error on normalised targets.  The network has no counterpart in the
reference; its inputs are block norms the reference's own filter rule acts on
(LibRI LRI.hpp:20-25: a block is kept when its max-norm exceeds the threshold).
"""
import math

import numpy as np

IN, H = 9, 64
NPARAM = H * IN + H + H * H + H + H + 1
NNORM = 2 * IN + 3
_ERF = np.vectorize(math.erf)


def unpack(params, round16=True):
    # FP16 weights, as the kernels read them (round16=False keeps FP64, for derivative checks)
    p = np.asarray(params, np.float16 if round16 else np.float64).astype(np.float64)
    o = 0
    W1 = p[o:o + H * IN].reshape(H, IN); o += H * IN
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + H]; o += H
    b3 = p[o]
    return W1, b1, W2, b2, W3, b3


def gelu(z):
    return 0.5 * z * (1.0 + _ERF(z / math.sqrt(2.0)))


def gelu_d(z):
    return 0.5 * (1.0 + _ERF(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def forward(params, norm, x):
    """Prediction in target units (log10 max |chi0|) for features x [n, 9]."""
    W1, b1, W2, b2, W3, b3 = unpack(params)
    norm = np.asarray(norm, np.float64)
    xn = (np.asarray(x, np.float64) - norm[:IN]) / norm[IN:2 * IN]
    h1 = gelu(xn @ W1.T + b1)
    h2 = gelu(h1 @ W2.T + b2)
    return (h2 @ W3 + b3) * norm[2 * IN + 1] + norm[2 * IN]


def loss_grad(params, norm, x, y, round16=True):
    """Mean squared error on normalised targets and its gradient (layout of screen.cu)."""
    W1, b1, W2, b2, W3, b3 = unpack(params, round16)
    norm = np.asarray(norm, np.float64)
    n = len(y)
    xn = (np.asarray(x, np.float64) - norm[:IN]) / norm[IN:2 * IN]
    tn = (np.asarray(y, np.float64) - norm[2 * IN]) / norm[2 * IN + 1]
    z1 = xn @ W1.T + b1
    h1 = gelu(z1)
    z2 = h1 @ W2.T + b2
    h2 = gelu(z2)
    out = h2 @ W3 + b3
    r = out - tn
    loss = float(np.mean(r * r))
    dy = 2.0 * r / n
    gW3 = h2.T @ dy
    gb3 = dy.sum()
    dz2 = dy[:, None] * W3[None, :] * gelu_d(z2)
    gW2 = dz2.T @ h1
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ W2) * gelu_d(z1)
    gW1 = dz1.T @ xn
    gb1 = dz1.sum(0)
    grad = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3, [gb3]])
    return loss, grad
