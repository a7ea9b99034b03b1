"""Float64 CPU restatement of the cost model's forward pass and gradient.

TEST INFRASTRUCTURE ONLY: the GPU kernels of acctricnt_gb300/csrc/model.cu are
checked against it (same parameter layout: W1[IN][H], b1, W2[H][H], b2,
W3[H][OUT], b3; ReLU hidden layers; mean squared error on the output of each
sample's kind).
"""
import numpy as np

IN, H, OUT = 8, 32, 3


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    W1 = p[o:o + IN * H].reshape(IN, H); o += IN * H
    b1 = p[o:o + H]; o += H
    W2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    W3 = p[o:o + H * OUT].reshape(H, OUT); o += H * OUT
    b3 = p[o:o + OUT]
    return W1, b1, W2, b2, W3, b3


def forward(p, x):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    x = np.asarray(x, np.float64)
    a1 = x @ W1 + b1
    h1 = np.maximum(a1, 0)
    a2 = h1 @ W2 + b2
    h2 = np.maximum(a2, 0)
    return h2 @ W3 + b3, (x, a1, h1, a2, h2)


def loss_grad(p, x, kind, target):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    y, (x, a1, h1, a2, h2) = forward(p, x)
    k = len(kind)
    yk = y[np.arange(k), kind]
    err = yk - np.asarray(target, np.float64)
    loss = float(np.mean(err ** 2))
    dy = np.zeros_like(y)
    dy[np.arange(k), kind] = 2 * err / k
    gW3 = h2.T @ dy
    gb3 = dy.sum(0)
    dh2 = (dy @ W3.T) * (a2 > 0)
    gW2 = h1.T @ dh2
    gb2 = dh2.sum(0)
    dh1 = (dh2 @ W2.T) * (a1 > 0)
    gW1 = x.T @ dh1
    gb1 = dh1.sum(0)
    return loss, np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
