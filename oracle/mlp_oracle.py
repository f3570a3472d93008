"""TEST INFRASTRUCTURE ONLY: NumPy FP64 restatement of the warm-start
network of rootpwa_gb300 (forward, mean-squared-error gradient), with the
same BF16 rounding points as the CUDA kernels (inputs, weights, hidden
activations and the backward signals are rounded to BF16; sums are exact
here), used to check the GPU gradients.  The network has no reference
counterpart."""
import numpy as np


EXACT = False  # when True the rounding points are skipped (finite-difference checks)


def bf16(x):
    """Round-to-nearest-even to bfloat16, returned as float64."""
    if EXACT:
        return np.asarray(x, dtype=np.float64)
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def f32(x):
    if EXACT:
        return np.asarray(x, dtype=np.float64)
    return np.asarray(x, dtype=np.float32).astype(np.float64)


def unpack(p, shape):
    nIn, h1, h2, nOut = shape
    o = 0
    out = []
    for rows, cols in ((h1, nIn), (h2, h1), (nOut, h2)):
        W = p[o:o + rows * cols].reshape(rows, cols)
        o += rows * cols
        b = p[o:o + rows]
        o += rows
        out += [W.astype(np.float64), b.astype(np.float64)]
    return out


def loss_and_gradient(p, shape, X, T):
    """Mean squared error and its gradient (parameter layout of pwa_mlp)."""
    W1, b1, W2, b2, W3, b3 = unpack(p, shape)
    W1b, W2b, W3b = bf16(W1), bf16(W2), bf16(W3)
    x = bf16(X)
    h1 = bf16(np.maximum(f32(x @ W1b.T + b1), 0.0))
    h2 = bf16(np.maximum(f32(h1 @ W2b.T + b2), 0.0))
    y = f32(h2 @ W3b.T + b3)
    n = y.size
    d = y - np.asarray(T, dtype=np.float64)
    loss = float(np.sum(d * d) / n)
    dy = f32(2.0 * d / n)
    dy16 = bf16(dy)
    gW3 = dy16.T @ h2
    gb3 = dy.sum(axis=0)
    dh2 = f32(dy16 @ W3b) * (h2 > 0)
    gb2 = dh2.sum(axis=0)
    dh2b = bf16(dh2)
    gW2 = dh2b.T @ h1
    dh1 = f32(dh2b @ W2b) * (h1 > 0)
    gb1 = dh1.sum(axis=0)
    gW1 = bf16(dh1).T @ x
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g


def forward(p, shape, X):
    W1, b1, W2, b2, W3, b3 = unpack(p, shape)
    h1 = bf16(np.maximum(f32(bf16(X) @ bf16(W1).T + b1), 0.0))
    h2 = bf16(np.maximum(f32(h1 @ bf16(W2).T + b2), 0.0))
    return f32(h2 @ bf16(W3).T + b3)
