"""TEST INFRASTRUCTURE ONLY: CPU restatement of the warm-start MLP.

Forward and backward of the 64 -> 128 -> 128 -> 3 GELU network in float64,
with the inputs, weights and hidden activations rounded to BF16 as the GPU
path stores them (tensor-core operands), so GPU gradients can be compared
with a tolerance that reflects BF16 storage only.  The network has no
counterpart in the reference; this is the project's own restatement.

Parameter blob layout: W1 [64x128], b1 [128], W2 [128x128], b2 [128],
W3 [128x3], b3 [3], row-major (input x output).
"""
import math

import numpy as np

IN, HID, OUT = 64, 128, 3


def bf16(x):
    """Round float64/float32 values to the nearest BF16 (ties to even)."""
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    u = ((u + rounding) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    out = []
    for shape in ((IN, HID), (HID,), (HID, HID), (HID,), (HID, OUT), (OUT,)):
        n = int(np.prod(shape))
        out.append(p[o:o + n].reshape(shape))
        o += n
    return out


_erf = np.vectorize(math.erf)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def forward(X, p, round_bf16=True):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    r = bf16 if round_bf16 else (lambda a: np.asarray(a, np.float64))
    X = r(X)
    z1 = X @ r(W1) + b1
    h1 = r(gelu(z1))
    z2 = h1 @ r(W2) + b2
    h2 = r(gelu(z2))
    y = h2 @ r(W3) + b3
    return y, (X, z1, h1, z2, h2)


def loss_grad(X, T, p, round_bf16=True):
    """Mean over rows of the summed squared error of the 3 outputs, and its gradient."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    r = bf16 if round_bf16 else (lambda a: np.asarray(a, np.float64))
    y, (Xr, z1, h1, z2, h2) = forward(X, p, round_bf16)
    B = X.shape[0]
    e = y - np.asarray(T, np.float64)
    loss = float(np.sum(e * e) / B)
    dy = 2.0 * e / B
    gW3 = h2.T @ dy
    gb3 = dy.sum(0)
    dz2 = (dy @ r(W3).T) * gelu_grad(z2)
    gW2 = h1.T @ dz2
    gb2 = dz2.sum(0)
    dz1 = (dz2 @ r(W2).T) * gelu_grad(z1)
    gW1 = Xr.T @ dz1
    gb1 = dz1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g
