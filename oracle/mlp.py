"""NumPy restatement of the learned-guess network (FP64). TEST INFRASTRUCTURE ONLY.

Same network and parameter layout as opencmp_gb300/csrc/ocmp_guess.cu:
    y = w3 . tanh(W2 tanh(W1 x + b1) + b2) + b3 + c . x,   hidden width 16,
flat parameters [W1 (16 x F, row-major), b1, W2 (16 x 16), b2, w3, b3, c (F)]; loss = mean((y - t)^2).
Used to check the GPU forward pass and gradients, and (backward differences, features, prediction,
training target, residual loss) the guess built on the network.
"""
import numpy as np

H = 16


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


def backward(P, X, dY):
    """Parameter gradient of sum_r dY_r y_r (the vector-Jacobian product of the network)."""
    X = np.asarray(X, np.float64)
    dy = np.asarray(dY, np.float64)
    F = X.shape[1]
    W1, b1, W2, b2, w3, b3, c = unpack(P, F)
    _, (h1, h2) = forward(P, X)
    d2 = np.outer(dy, w3) * (1 - h2 * h2)
    d1 = (d2 @ W2) * (1 - h1 * h1)
    return np.concatenate([(d1.T @ X).ravel(), d1.sum(0), (d2.T @ h1).ravel(), d2.sum(0), dy @ h2, [dy.sum()], dy @ X])


def back_diffs(hist):
    """D_0 = u^n and the backward differences D_j = nabla^j u^n of the history [u^n, u^{n-1}, ...]."""
    v = [np.asarray(h, np.float64).copy() for h in hist]
    D = [v[0].copy()]
    for j in range(1, len(v)):
        v = [v[m] - v[m + 1] for m in range(len(v) - 1)]
        D.append(v[0].copy())
    return D


def scales(hist, free):
    """S_j = root mean square of D_j over the free dofs, j = 1..k-1."""
    D = back_diffs(hist)
    nf = max(int(free.sum()), 1)
    return np.array([max(np.sqrt((D[j][free] ** 2).sum() / nf), 1e-300) for j in range(1, len(D))])


def features(hist, free):
    D = back_diffs(hist)
    S = scales(hist, free)
    X = np.stack([D[j] / S[j - 1] for j in range(1, len(D))], 1)
    X[~free] = 0
    return X, S


def predict(P, hist, free, base):
    """u^n + D_1 + ... + D_base (+ S_{k-1} y(X) when P is given) on free dofs, u^n elsewhere."""
    D = back_diffs(hist)
    x = D[0] + sum(D[j] for j in range(1, base + 1))
    if P is not None:
        X, S = features(hist, free)
        y, _ = forward(P, X.astype(np.float32).astype(np.float64))
        x = x + S[-1] * y
    return np.where(free, x, D[0])


def target(hist, free, base, unext):
    D = back_diffs(hist)
    S = scales(hist, free)
    base_v = D[0] + sum(D[j] for j in range(1, base + 1))
    return np.where(free, (unext - base_v) / S[-1], 0.0)


def residual_loss(A, Y, T, S, b, free, weight=1.0):
    """weight |(A e)_free|^2 / |b_free|^2 with e = S (Y - T) on free dofs, and its gradient in Y."""
    e = np.where(free, S * (np.asarray(Y, np.float64) - np.asarray(T, np.float64)), 0.0)
    v = np.where(free, A @ e, 0.0)
    bb = float((b[free] ** 2).sum())
    c = weight / bb
    return c * float(v @ v), np.where(free, 2 * c * S * (A.T @ v), 0.0)
