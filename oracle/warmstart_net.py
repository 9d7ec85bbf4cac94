"""Float64 numpy restatement of the warm-start network and its gradients.

TEST INFRASTRUCTURE ONLY: the checker for the GPU forward/backward kernels
(``pot_gb300/csrc/mlp.cu``).  The network has no counterpart in the
reference; its gradients are pinned here by central finite differences
(``tests/test_oracle.py``), and the GPU gradients are compared with these.
"""
import numpy as np


def _relu(x):
    return np.maximum(x, 0.0)


def forward(params, X, Y, Z=None):
    """X: (P, n, d), Y: (P, m, d) normalised clouds, Z: (P, n, dz) head
    inputs (default X); returns f (P, n) and a cache for ``backward``."""
    p = {k: np.asarray(v, dtype=np.float64) for k, v in params.items()}
    X = np.asarray(X, dtype=np.float64)
    Y = np.asarray(Y, dtype=np.float64)
    hx1 = _relu(X @ p["W1x"] + p["b1x"])
    hx2 = _relu(hx1 @ p["W2x"] + p["b2x"])
    hy1 = _relu(Y @ p["W1y"] + p["b1y"])
    hy2 = _relu(hy1 @ p["W2y"] + p["b2y"])
    sX = hx2.mean(1)
    sY = hy2.mean(1)
    P, n, _ = X.shape
    Zi = X if Z is None else np.asarray(Z, dtype=np.float64)
    z = np.concatenate([Zi, np.repeat(sX[:, None, :], n, 1), np.repeat(sY[:, None, :], n, 1)], 2)
    h3 = _relu(z @ p["W3"] + p["b3"])
    h4 = _relu(h3 @ p["W4"] + p["b4"])
    f = (h4 @ p["W5"] + p["b5"])[..., 0]
    return f, (p, X, Y, hx1, hx2, hy1, hy2, z, h3, h4)


def centered_mse(f, t):
    """Mean over pairs of sum_i ((f_i - mean f) - t_i)^2 / n, and d/df."""
    P, n = f.shape
    e = (f - f.mean(1, keepdims=True)) - t
    loss = float(np.sum(e * e) / (P * n))
    df = 2.0 * (e - e.mean(1, keepdims=True)) / (P * n)
    return loss, df


def backward(cache, df):
    p, X, Y, hx1, hx2, hy1, hy2, z, h3, h4 = cache
    g = {}
    P, n, _ = X.shape
    m = Y.shape[1]
    H = p["W2x"].shape[1]
    d = z.shape[2] - 2 * H
    dfe = df[..., None]
    g["W5"] = np.einsum("pnh,pno->ho", h4, dfe)
    g["b5"] = dfe.sum((0, 1))
    dh4 = (dfe @ p["W5"].T) * (h4 > 0)
    g["W4"] = np.einsum("pnh,pno->ho", h3, dh4)
    g["b4"] = dh4.sum((0, 1))
    dh3 = (dh4 @ p["W4"].T) * (h3 > 0)
    g["W3"] = np.einsum("pnh,pno->ho", z, dh3)
    g["b3"] = dh3.sum((0, 1))
    dz = dh3 @ p["W3"].T
    dsX = dz[:, :, d:d + H].sum(1)
    dsY = dz[:, :, d + H:].sum(1)
    for side, ds, h1, h2, rows, inp in (("x", dsX, hx1, hx2, n, X), ("y", dsY, hy1, hy2, m, Y)):
        dh2 = np.repeat(ds[:, None, :] / rows, rows, 1) * (h2 > 0)
        g["W2" + side] = np.einsum("pnh,pno->ho", h1, dh2)
        g["b2" + side] = dh2.sum((0, 1))
        dh1 = (dh2 @ p["W2" + side].T) * (h1 > 0)
        g["W1" + side] = np.einsum("pnh,pno->ho", inp, dh1)
        g["b1" + side] = dh1.sum((0, 1))
    return g


def loss_and_grads(params, X, Y, t, Z=None):
    f, cache = forward(params, X, Y, Z)
    loss, df = centered_mse(f, np.asarray(t, dtype=np.float64))
    return loss, backward(cache, df), f
