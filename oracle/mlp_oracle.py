"""Test infrastructure: a NumPy restatement of the bit selector's MLP.

The reference has no learned component (it picks the fractional bit length by
the rule of Work/main.cpp:153-161 or by the manual sweep of Work/sub.cpp), so
this oracle is pinned by finite differences instead of reference vectors: the
CPU tests check its gradient against central differences in float64, and the
GPU tests check the library's CUDA forward, backward and Adam kernels against
it.  Nothing in the product imports this file.

Network: X -> (X - mu) / sd -> relu(W1 x + b1) -> relu(W2 h + b2) -> W3 h + b3.
Loss: masked mean squared error  L = sum M (Y - T)^2 / sum M.
Flat parameter layout: W1[H][I] b1[H] W2[H][H] b2[H] W3[O][H] b3[O].
"""
import numpy as np


def shapes(nin, hid, nout):
    return [("W1", (hid, nin)), ("b1", (hid,)), ("W2", (hid, hid)), ("b2", (hid,)), ("W3", (nout, hid)),
            ("b3", (nout,))]


def unpack(p, nin, hid, nout):
    out, o = {}, 0
    for name, shp in shapes(nin, hid, nout):
        n = int(np.prod(shp))
        out[name] = p[o:o + n].reshape(shp)
        o += n
    assert o == p.size
    return out


def forward(p, X, nin, hid, nout, mu=None, sd=None):
    w = unpack(p, nin, hid, nout)
    x = X if mu is None else (X - mu) / sd
    z1 = x @ w["W1"].T + w["b1"]
    a1 = np.maximum(z1, 0)
    z2 = a1 @ w["W2"].T + w["b2"]
    a2 = np.maximum(z2, 0)
    y = a2 @ w["W3"].T + w["b3"]
    return y, (x, a1, a2)


def loss_grad(p, X, T, M, nin, hid, nout, mu=None, sd=None):
    """Loss and flat gradient (same layout as p)."""
    w = unpack(p, nin, hid, nout)
    y, (x, a1, a2) = forward(p, X, nin, hid, nout, mu, sd)
    ms = M.sum()
    inv = 1.0 / ms if ms > 0 else 0.0
    d = y - T
    loss = float((M * d * d).sum() * inv)
    dy = 2.0 * M * d * inv
    g = {"W3": dy.T @ a2, "b3": dy.sum(0)}
    d2 = (dy @ w["W3"]) * (a2 > 0)
    g["W2"], g["b2"] = d2.T @ a1, d2.sum(0)
    d1 = (d2 @ w["W2"]) * (a1 > 0)
    g["W1"], g["b1"] = d1.T @ x, d1.sum(0)
    flat = np.concatenate([g[name].ravel() for name, _ in shapes(nin, hid, nout)])
    return loss, flat


def splitmix64_stream(seed):
    """The generator the library uses for initialisation and shuffling."""
    st = seed & 0xFFFFFFFFFFFFFFFF
    M64 = 0xFFFFFFFFFFFFFFFF
    while True:
        st = (st + 0x9E3779B97F4A7C15) & M64
        z = st
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
        yield z ^ (z >> 31)


def init_params(nin, hid, nout, seed):
    """He-uniform initialisation in the library's order (weights only, biases 0)."""
    gen = splitmix64_stream(seed)
    p = np.zeros(sum(int(np.prod(s)) for _, s in shapes(nin, hid, nout)), np.float64)
    o = 0
    for name, shp in shapes(nin, hid, nout):
        n = int(np.prod(shp))
        if name.startswith("W"):
            lim = np.sqrt(6.0 / shp[1])
            for i in range(n):
                u = (next(gen) >> 11) * (1.0 / 9007199254740992.0)
                p[o + i] = np.float32((2.0 * u - 1.0) * lim)
        o += n
    return p


def train(p, X, T, M, nin, hid, nout, epochs, batch, lr, seed, mu=None, sd=None):
    """Mini-batch Adam with the library's shuffle (Fisher-Yates on splitmix64)."""
    p = p.astype(np.float64).copy()
    m1, m2 = np.zeros_like(p), np.zeros_like(p)
    n = X.shape[0]
    batch = min(batch, n)
    gen = splitmix64_stream(seed)
    t = 0
    hist = []
    b1, b2, eps = 0.9, 0.999, 1e-8
    for _ in range(epochs):
        perm = list(range(n))
        for i in range(n - 1, 0, -1):
            j = next(gen) % (i + 1)
            perm[i], perm[j] = perm[j], perm[i]
        perm = np.array(perm)
        losses = []
        for off in range(0, n, batch):
            idx = perm[off:off + batch]
            loss, g = loss_grad(p, X[idx], T[idx], M[idx], nin, hid, nout, mu, sd)
            losses.append(loss)
            t += 1
            m1 = b1 * m1 + (1 - b1) * g
            m2 = b2 * m2 + (1 - b2) * g * g
            p -= lr * (m1 / (1 - b1 ** t)) / (np.sqrt(m2 / (1 - b2 ** t)) + eps)
        hist.append(np.mean(losses))
    return p, np.array(hist)
