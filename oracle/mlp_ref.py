"""float64 numpy restatement of the dispatcher network (forward, masked
mean-squared-error loss, backward) with the CUDA library's parameter layout.

TEST INFRASTRUCTURE ONLY: the oracle against which the library's hand-written
MLP kernels are tested (ndconv_mlp_forward / ndconv_mlp_gradient).  The network has no
counterpart in the reference crate; this file follows the library's own
definition: y = W3 relu(W2 relu(W1 x + b1) + b2) + b3 and
L = sum_{n,o} m[n,o] (y[n,o] - t[n,o])^2 / (2 sum(m)).

Flat parameter layout: W1[h][in], b1[h], W2[h][h], b2[h], W3[out][h], b3[out].
"""
import numpy as np


def sizes(n_in, n_h, n_out):
    return [("W1", (n_h, n_in)), ("b1", (n_h,)), ("W2", (n_h, n_h)), ("b2", (n_h,)),
            ("W3", (n_out, n_h)), ("b3", (n_out,))]


def unpack(params, n_in, n_h, n_out):
    out, off = {}, 0
    p = np.asarray(params, dtype=np.float64)
    for name, shp in sizes(n_in, n_h, n_out):
        cnt = int(np.prod(shp))
        out[name] = p[off:off + cnt].reshape(shp)
        off += cnt
    assert off == p.size, (off, p.size)
    return out


def pack(parts, n_in, n_h, n_out):
    return np.concatenate([np.asarray(parts[name], dtype=np.float64).ravel()
                           for name, _ in sizes(n_in, n_h, n_out)])


def forward(params, x, n_in, n_h, n_out):
    P = unpack(params, n_in, n_h, n_out)
    x = np.asarray(x, dtype=np.float64)
    a1 = np.maximum(x @ P["W1"].T + P["b1"], 0.0)
    a2 = np.maximum(a1 @ P["W2"].T + P["b2"], 0.0)
    return a2 @ P["W3"].T + P["b3"], (x, a1, a2)


def loss_and_grad(params, x, t, m, n_in, n_h, n_out):
    P = unpack(params, n_in, n_h, n_out)
    y, (a0, a1, a2) = forward(params, x, n_in, n_h, n_out)
    t = np.asarray(t, dtype=np.float64)
    m = np.asarray(m, dtype=np.float64)
    ms = max(m.sum(), 1.0)
    e = np.where(m != 0, y - t, 0.0)
    loss = 0.5 * float((m * e * e).sum()) / ms
    g3 = m * e / ms
    G = {"W3": g3.T @ a2, "b3": g3.sum(0)}
    g2 = (g3 @ P["W3"]) * (a2 > 0)
    G["W2"] = g2.T @ a1
    G["b2"] = g2.sum(0)
    g1 = (g2 @ P["W2"]) * (a1 > 0)
    G["W1"] = g1.T @ a0
    G["b1"] = g1.sum(0)
    return loss, pack(G, n_in, n_h, n_out)
