"""Oracle (test infrastructure only): NumPy FP64 restatement of the learned
proposal's features, forward pass and backward pass (graph-cut-ransac_gb300/
csrc/gcr_learned.cu), used to check the device kernels and their gradients.
The network reads the same BF16-rounded weights as the device."""
import numpy as np

K = 8
FEAT = 20
IN = 32
H = 128


def offsets_of():
    o = {}
    o["W1"] = 0
    o["b1"] = o["W1"] + IN * H
    o["W2"] = o["b1"] + H
    o["b2"] = o["W2"] + H * H
    o["W3"] = o["b2"] + H
    o["b3"] = o["W3"] + H * H
    o["W4"] = o["b3"] + H
    o["b4"] = o["W4"] + H
    o["count"] = o["b4"] + 1
    return o


OFF = offsets_of()


def bf16_round(x):
    """Round-to-nearest-even of float32 values to bfloat16, returned as float64."""
    x = np.asarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(P):
    P = np.asarray(P, np.float64)
    return (P[OFF["W1"]:OFF["b1"]].reshape(IN, H), P[OFF["b1"]:OFF["W2"]],
            P[OFF["W2"]:OFF["b2"]].reshape(H, H), P[OFF["b2"]:OFF["W3"]],
            P[OFF["W3"]:OFF["b3"]].reshape(H, H), P[OFF["b3"]:OFF["W4"]],
            P[OFF["W4"]:OFF["b4"]], P[OFF["b4"]])


MISSING = 65536.0


def features(corr, size):
    """Features of one pair: [n, IN] float32 (gcr_learned.cu, features_kernel).
    Neighbours: the K nearest first-image points by FP32 squared distance
    (coordinates rounded to float32, each operation rounded), ties by index;
    per neighbour (sqrt|d_j - d_i| / 4, sqrt|x1_j - x1_i| / 4) in pixels,
    ordered by the first value, missing neighbours (4, 4) last."""
    corr = np.asarray(corr, np.float64)
    h1, w1, h2, w2 = size
    n = len(corr)
    out = np.zeros((n, IN), np.float32)
    p = corr[:, :2].astype(np.float32)
    ex = p[None, :, 0] - p[:, None, 0]
    ey = p[None, :, 1] - p[:, None, 1]
    d2 = ex * ex + ey * ey
    np.fill_diagonal(d2, np.inf)
    out[:, 0] = corr[:, 0] / w1 - 0.5
    out[:, 1] = corr[:, 1] / h1 - 0.5
    out[:, 2] = corr[:, 2] / w2 - 0.5
    out[:, 3] = corr[:, 3] / h2 - 0.5
    dx = corr[:, 2] - corr[:, 0]
    dy = corr[:, 3] - corr[:, 1]
    for i in range(n):
        nb = np.argsort(d2[i], kind="stable")[:min(K, n - 1)]
        a = dx[nb] - dx[i]
        b = dy[nb] - dy[i]
        ux = corr[nb, 0] - corr[i, 0]
        uy = corr[nb, 1] - corr[i, 1]
        mag = np.full(K, MISSING)
        dist = np.full(K, MISSING)
        mag[:len(nb)] = a * a + b * b
        dist[:len(nb)] = ux * ux + uy * uy
        o = np.argsort(mag, kind="stable")
        out[i, 4:4 + 2 * K:2] = 0.25 * np.sqrt(np.sqrt(mag[o]))
        out[i, 5:5 + 2 * K:2] = 0.25 * np.sqrt(np.sqrt(dist[o]))
    return out


def order(logits):
    """Descending order of one pair's logits, ties by index, NaN last
    (gcr_learned.cu, order_kernel): the permutation perm with
    sorted[k] = corr[perm[k]]."""
    z = np.asarray(logits, np.float32).astype(np.float64)
    z = np.where(np.isnan(z), -np.inf, z)
    return np.lexsort((np.arange(len(z)), -z))


def adam(m, v, P, g, lr, step, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (step counts from 1); returns (m, v, P)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    P = P - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return m, v, P


def forward(X, P, rounding=True):
    """(A1, A2, A3, z): the device forward (gcr_learned.cu, forward_kernel) in
    FP64. With rounding, the inputs of the first three layers are rounded to
    BF16 (the features, and A1, A2 as stored); A3 stays unrounded."""
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(P)
    r = bf16_round if rounding else (lambda v: np.asarray(v, np.float64))
    Xb = r(X)
    A1 = r(np.maximum(Xb @ W1 + b1, 0))
    A2 = r(np.maximum(A1 @ W2 + b2, 0))
    A3 = np.maximum(A2 @ W3 + b3, 0)
    z = A3 @ W4 + b4
    return A1, A2, A3, z


def grad_from(Xin, A1, A2, A3, z, P, y, w):
    """Weighted BCE with logits divided by sum(w), and its gradient, from the
    layer inputs of a forward pass (Xin: the first layer's input)."""
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(P)
    Xin, A1, A2, A3, z = (np.asarray(v, np.float64) for v in (Xin, A1, A2, A3, z))
    ws = np.sum(w)
    loss = np.sum(w * (np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z))))) / ws
    g4 = (1 / (1 + np.exp(-z)) - y) * w / ws
    G = np.zeros(OFF["count"])
    G[OFF["W4"]:OFF["b4"]] = A3.T @ g4
    G[OFF["b4"]] = g4.sum()
    dz3 = np.outer(g4, W4) * (A3 > 0)
    G[OFF["W3"]:OFF["b3"]] = (A2.T @ dz3).ravel()
    G[OFF["b3"]:OFF["W4"]] = dz3.sum(0)
    dz2 = (dz3 @ W3.T) * (A2 > 0)
    G[OFF["W2"]:OFF["b2"]] = (A1.T @ dz2).ravel()
    G[OFF["b2"]:OFF["W3"]] = dz2.sum(0)
    dz1 = (dz2 @ W2.T) * (A1 > 0)
    G[OFF["W1"]:OFF["b1"]] = (Xin.T @ dz1).ravel()
    G[OFF["b1"]:OFF["W2"]] = dz1.sum(0)
    return loss, G


def loss_and_grad(X, P, y, w, rounding=True):
    """Loss and gradient through forward(X, P, rounding); the BF16 roundings
    pass gradients straight through."""
    A1, A2, A3, z = forward(X, P, rounding)
    Xin = bf16_round(X) if rounding else np.asarray(X, np.float64)
    return grad_from(Xin, A1, A2, A3, z, P, y, w)
