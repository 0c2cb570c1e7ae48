"""CPU restatement of the learned models' network (test infrastructure only).

The GPU kernels in madam_gb300/csrc/mlp.cu are checked against this: the same
network x -> tanh(W1 x + b1) -> tanh(W2 . + b2) -> w3 . + b3, the same packed
parameter vector [W1 (h1 x d, row-major) | b1 | W2 (h2 x h1) | b2 | w3 | b3],
mean squared error, reverse-mode gradient written out by hand, and Adam
(Kingma & Ba, 2015: beta1 0.9, beta2 0.999, eps 1e-8, bias-corrected).
Computed in float64 so that it serves as the reference for the FP32 kernels.
"""
import numpy as np


def unpack(p, d, h1, h2):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + h1 * d].reshape(h1, d); o += h1 * d
    b1 = p[o:o + h1]; o += h1
    W2 = p[o:o + h2 * h1].reshape(h2, h1); o += h2 * h1
    b2 = p[o:o + h2]; o += h2
    w3 = p[o:o + h2]; o += h2
    b3 = p[o]
    return W1, b1, W2, b2, w3, b3


def forward(p, X, d, h1, h2):
    W1, b1, W2, b2, w3, b3 = unpack(p, d, h1, h2)
    X = np.asarray(X, dtype=np.float64)
    A1 = np.tanh(X @ W1.T + b1)
    A2 = np.tanh(A1 @ W2.T + b2)
    return A2 @ w3 + b3, (X, A1, A2)


def loss_and_grad(p, X, Y, d, h1, h2):
    W1, b1, W2, b2, w3, b3 = unpack(p, d, h1, h2)
    y, (X, A1, A2) = forward(p, X, d, h1, h2)
    n = len(y)
    r = y - np.asarray(Y, dtype=np.float64)
    loss = float(np.mean(r * r))
    dy = 2.0 * r / n                                   # dL/dy
    D2 = (dy[:, None] * w3[None, :]) * (1.0 - A2 * A2)  # dL/d(pre-activation 2)
    D1 = (D2 @ W2) * (1.0 - A1 * A1)                    # dL/d(pre-activation 1)
    g = np.concatenate([(D1.T @ X).ravel(), D1.sum(0), (D2.T @ A1).ravel(), D2.sum(0), A2.T @ dy, [dy.sum()]])
    return loss, g


def adam(p, m, v, g, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v
