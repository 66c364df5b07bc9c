"""FP64 numpy restatement of the learned-correction MLP (test infrastructure only).

Mirrors particular_gb300/csrc/pt_mlp.cuh (parameter layout, GELU tanh form) and the
loss of the training kernel (mean over samples of the squared error of the scaled
targets), with exact derivatives by hand. It has no counterpart in the reference.
"""
import numpy as np

IN, H, OUT = 12, 64, 3
W1 = 0
B1 = W1 + H * IN
W2 = B1 + H
B2 = W2 + H * H
W3 = B2 + H
B3 = W3 + OUT * H
SCALE = B3 + OUT
NPARAM = SCALE + 1
C = np.sqrt(2.0 / np.pi)
A = 0.044715


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[W1:B1].reshape(H, IN), p[B1:W2], p[W2:B2].reshape(H, H), p[B2:W3],
            p[W3:B3].reshape(OUT, H), p[B3:SCALE], p[SCALE])


def gelu(x):
    u = C * (x + A * x ** 3)
    t = np.tanh(u)
    return 0.5 * x * (1 + t), 0.5 * (1 + t) + 0.5 * x * (1 - t * t) * C * (1 + 3 * A * x * x)


def forward(p, f):
    w1, b1, w2, b2, w3, b3, scale = unpack(p)
    h1, _ = gelu(f @ w1.T + b1)
    h2, _ = gelu(h1 @ w2.T + b2)
    return (h2 @ w3.T + b3) * scale


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    b = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def forward_bf16(p, f):
    """The tensor-core inference path: features and both hidden layers' activations
    rounded to BF16 before each product, everything else exact."""
    w1, b1, w2, b2, w3, b3, scale = unpack(p)
    h1, _ = gelu(bf16(f) @ w1.T + b1)
    h2, _ = gelu(bf16(h1) @ w2.T + b2)
    return (bf16(h2) @ w3.T + b3) * scale


def loss_grad(p, f, t):
    """Loss and gradient of the training kernel for features f (b, 12), raw targets t."""
    w1, b1, w2, b2, w3, b3, scale = unpack(p)
    f = np.asarray(f, np.float64)
    t = np.asarray(t, np.float64) / scale
    b = f.shape[0]
    z1 = f @ w1.T + b1
    h1, d1 = gelu(z1)
    z2 = h1 @ w2.T + b2
    h2, d2 = gelu(z2)
    y = h2 @ w3.T + b3
    e = y - t
    loss = (e * e).sum() / b
    dy = 2 * e / b
    g = np.zeros(NPARAM)
    g[W3:B3] = (dy.T @ h2).ravel()
    g[B3:SCALE] = dy.sum(0)
    g2 = (dy @ w3) * d2
    g[W2:B2] = (g2.T @ h1).ravel()
    g[B2:W3] = g2.sum(0)
    g1 = (g2 @ w2) * d1
    g[W1:B1] = (g1.T @ f).ravel()
    g[B1:W2] = g1.sum(0)
    return loss, g
