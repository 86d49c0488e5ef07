"""FP64 CPU restatement of the selector MLP (test infrastructure only): the
checker for the GPU forward/backward/Adam kernels of blis_gb300/csrc/gb_mlp.cu.

Layout of the parameter vector (same as the GPU): W1[64][16] b1[64]
W2[64][64] b2[64] W3[64][64] b3[64] W4[8][64] b4[8]; GELU(z) =
z * Phi(z) with the exact normal CDF; loss = sum mask*(out-y)^2 / norm.
"""
import numpy as np
from scipy.special import erf

NIN, NH, NOUT = 16, 64, 8
SHAPES = [("W1", (NH, NIN)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)),
          ("W3", (NH, NH)), ("b3", (NH,)), ("W4", (NOUT, NH)), ("b4", (NOUT,))]
NPARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p):
    out, o = {}, 0
    for name, shp in SHAPES:
        sz = int(np.prod(shp))
        out[name] = p[o:o + sz].reshape(shp)
        o += sz
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def init(seed=0):
    rng = np.random.default_rng(seed)
    d = {}
    for name, shp in SHAPES:
        if name.startswith("W"):
            d[name] = rng.normal(0.0, np.sqrt(2.0 / shp[1]), size=shp)
        else:
            d[name] = np.zeros(shp)
    return pack(d)


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def forward(p, x, keep=False):
    w = unpack(np.asarray(p, dtype=np.float64))
    x = np.asarray(x, dtype=np.float64)
    z1 = x @ w["W1"].T + w["b1"]
    a1 = gelu(z1)
    z2 = a1 @ w["W2"].T + w["b2"]
    a2 = gelu(z2)
    z3 = a2 @ w["W3"].T + w["b3"]
    a3 = gelu(z3)
    out = a3 @ w["W4"].T + w["b4"]
    if keep:
        return out, (x, z1, a1, z2, a2, z3, a3)
    return out


def loss_grad(p, x, y, mask, norm):
    w = unpack(np.asarray(p, dtype=np.float64))
    out, (x, z1, a1, z2, a2, z3, a3) = forward(p, x, keep=True)
    d = out - y
    loss = float((mask * d * d).sum() / norm)
    g4 = 2.0 * mask * d / norm
    gW4 = g4.T @ a3
    gb4 = g4.sum(0)
    g3 = (g4 @ w["W4"]) * gelu_grad(z3)
    gW3 = g3.T @ a2
    gb3 = g3.sum(0)
    g2 = (g3 @ w["W3"]) * gelu_grad(z2)
    gW2 = g2.T @ a1
    gb2 = g2.sum(0)
    g1 = (g2 @ w["W2"]) * gelu_grad(z1)
    gW1 = g1.T @ x
    gb1 = g1.sum(0)
    grad = pack({"W1": gW1, "b1": gb1, "W2": gW2, "b2": gb2, "W3": gW3, "b3": gb3, "W4": gW4, "b4": gb4})
    return loss, grad


def adam(p, g, m, v, lr, b1, b2, eps, wd, step):
    g = g + wd * p
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    p = p - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return p, m, v
