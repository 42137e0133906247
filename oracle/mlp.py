"""NumPy restatement of the learned-guess network (FP64). TEST INFRASTRUCTURE ONLY.

Same network and parameter layout as opencmp_gb300/csrc/ocmp_guess.cu:
    y = w3 . tanh(W2 tanh(W1 x + b1) + b2) + b3 + c . x,   hidden width 32,
flat parameters [W1 (32 x F, row-major), b1, W2 (32 x 32), b2, w3, b3, c (F)]; loss = mean((y - t)^2).
Used to check the GPU forward pass and gradients.
"""
import numpy as np

H = 32


def layout(F):
    o = {'W1': 0}
    o['b1'] = o['W1'] + H * F
    o['W2'] = o['b1'] + H
    o['b2'] = o['W2'] + H * H
    o['w3'] = o['b2'] + H
    o['b3'] = o['w3'] + H
    o['c'] = o['b3'] + 1
    o['n'] = o['c'] + F
    return o


def unpack(P, F):
    o = layout(F)
    P = np.asarray(P, np.float64)
    return (P[o['W1']:o['b1']].reshape(H, F), P[o['b1']:o['W2']], P[o['W2']:o['b2']].reshape(H, H),
            P[o['b2']:o['w3']], P[o['w3']:o['b3']], P[o['b3']], P[o['c']:o['n']])


def forward(P, X):
    F = X.shape[1]
    W1, b1, W2, b2, w3, b3, c = unpack(P, F)
    h1 = np.tanh(X @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    return h2 @ w3 + b3 + X @ c, (h1, h2)


def loss_grad(P, X, T):
    X = np.asarray(X, np.float64)
    T = np.asarray(T, np.float64)
    F = X.shape[1]
    N = X.shape[0]
    W1, b1, W2, b2, w3, b3, c = unpack(P, F)
    y, (h1, h2) = forward(P, X)
    e = y - T
    loss = float(np.mean(e * e))
    dy = 2.0 * e / N
    d2 = np.outer(dy, w3) * (1 - h2 * h2)
    d1 = (d2 @ W2) * (1 - h1 * h1)
    g = np.concatenate([(d1.T @ X).ravel(), d1.sum(0), (d2.T @ h1).ravel(), d2.sum(0), dy @ h2, [dy.sum()], dy @ X])
    return loss, g
