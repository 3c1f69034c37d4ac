"""CPU restatement (numpy, FP64) of the learned warm-start network of bes_gb300/csrc/mlp.cu.

TEST INFRASTRUCTURE ONLY: the tests use it as the checker of the GPU forward pass, gradients
and AdamW step.  The reference has no learned component; this network is this project's own
design, so the restatement follows the library's definition:

  features  x in [-1, 1]^3 (cell centroid scaled by the centroids' bounding box):
            [sin(pi 2^k x_a), cos(pi 2^k x_a)] for a = 0..2, k = 0..7 at columns 16a + 2k
            (+1), x itself at columns 48..50, zeros up to 64;
  condition c in R^3: the freestream Mach vector normalised by the training set's mean and
            standard deviation;
  hidden    for l = 0..3: z = h W_l^T + b_l; [gamma, beta] = c F_l^T + g_l (512 = 2 x 256);
            y = z (1 + gamma) + beta; h = silu(y)          (FiLM, width 256)
  output    o = h W_4^T + b_4 (5 values): the conserved variables relative to the
            freestream, divided by a per-variable scale;
  loss      sum over the batch and the 5 outputs of (o - t)^2 / (5 B).
Parameters are one flat FP32 vector in the order of `layout()`.
"""
from __future__ import annotations

import numpy as np

WIDTH = 256
K0 = 64
N_FOURIER = 8


def layout():
    """[(name, shape)] of the flat parameter vector."""
    out = []
    for l in range(4):
        k = K0 if l == 0 else WIDTH
        out += [(f"W{l}", (WIDTH, k)), (f"b{l}", (WIDTH,)), (f"F{l}", (2 * WIDTH, 3)),
                (f"g{l}", (2 * WIDTH,))]
    out += [("W4", (5, WIDTH)), ("b4", (5,))]
    return out


def n_params():
    return sum(int(np.prod(s)) for _, s in layout())


def unpack(flat):
    flat = np.asarray(flat, dtype=np.float64)
    p, off = {}, 0
    for name, shape in layout():
        n = int(np.prod(shape))
        p[name] = flat[off:off + n].reshape(shape)
        off += n
    return p


def pack(p):
    return np.concatenate([np.asarray(p[name], np.float64).ravel() for name, _ in layout()])


def encode(xn):
    """[n,3] scaled centroids -> [n,64] features."""
    xn = np.asarray(xn, dtype=np.float64)
    f = np.zeros((xn.shape[0], K0))
    for a in range(3):
        for k in range(N_FOURIER):
            w = np.pi * 2.0 ** k * xn[:, a]
            f[:, 16 * a + 2 * k] = np.sin(w)
            f[:, 16 * a + 2 * k + 1] = np.cos(w)
    f[:, 48:51] = xn
    return f


def bf16(x):
    """Round to bfloat16 (nearest even) through float32, as the GPU's __float2bfloat16."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def _id(x):
    return x


def _silu(y):
    return y / (1.0 + np.exp(-y))


def _dsilu(y):
    s = 1.0 / (1.0 + np.exp(-y))
    return s * (1.0 + y * (1.0 - s))


def forward(flat, X0, C, rounded=False):
    """Outputs [n,5] and the cache for backward.  rounded: round the GEMM operands (features,
    hidden weights, hidden activations) to bfloat16 where the GPU does."""
    r = bf16 if rounded else _id
    p = unpack(flat)
    h = r(np.asarray(X0, np.float64))
    C = np.asarray(C, np.float64)
    cache = []
    for l in range(4):
        z = h @ r(p[f"W{l}"]).T + p[f"b{l}"]
        gb = C @ p[f"F{l}"].T + p[f"g{l}"]
        gam, bet = gb[:, :WIDTH], gb[:, WIDTH:]
        y = z * (1.0 + gam) + bet
        cache.append((h, z, y, gam))
        h = r(_silu(y))
    o = h @ p["W4"].T + p["b4"]
    cache.append(h)
    return o, cache


def loss_and_grad(flat, X0, C, T, rounded=False):
    """Loss, its gradient (flat) and the outputs for one batch; rounded as in forward (and
    the GEMM operand dz rounded to bfloat16)."""
    r = bf16 if rounded else _id
    p = unpack(flat)
    C = np.asarray(C, np.float64)
    o, cache = forward(flat, X0, C, rounded)
    B = o.shape[0]
    d = o - np.asarray(T, np.float64)
    loss = float((d * d).sum() / (5.0 * B))
    dO = 2.0 * d / (5.0 * B)
    g = {}
    h4 = cache[4]
    g["W4"] = dO.T @ h4
    g["b4"] = dO.sum(axis=0)
    dh = dO @ p["W4"]
    for l in range(3, -1, -1):
        h, z, y, gam = cache[l]
        dy = dh * _dsilu(y)
        dz = dy * (1.0 + gam)
        dgb = np.concatenate([dy * z, dy], axis=1)
        g[f"F{l}"] = dgb.T @ C
        g[f"g{l}"] = dgb.sum(axis=0)
        g[f"W{l}"] = r(dz).T @ h
        g[f"b{l}"] = dz.sum(axis=0)
        dh = r(dz) @ r(p[f"W{l}"])
    return loss, pack(g), o


def adamw_step(flat, grad, m, v, t, lr, weight_decay, beta1=0.9, beta2=0.999, eps=1e-8):
    """One AdamW step (decoupled weight decay on the W matrices only); returns new (p, m, v)."""
    flat = np.asarray(flat, np.float64).copy()
    m = beta1 * np.asarray(m, np.float64) + (1 - beta1) * grad
    v = beta2 * np.asarray(v, np.float64) + (1 - beta2) * grad * grad
    mh = m / (1 - beta1 ** t)
    vh = v / (1 - beta2 ** t)
    decay = np.zeros_like(flat)
    off = 0
    for name, shape in layout():
        n = int(np.prod(shape))
        if name.startswith("W"):
            decay[off:off + n] = weight_decay
        off += n
    flat -= lr * (mh / (np.sqrt(vh) + eps) + decay * flat)
    return flat, m, v
