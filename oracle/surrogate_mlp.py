"""CPU FP64 restatement of the surrogate network -- test infrastructure only.

This is the oracle the tcgen05 training kernels' gradients are checked against (forward, loss and
backward in float64 numpy). The reference has no learned model, so the network's definition is the
library's own (black_simulation_gb300/csrc/bhk_surrogate.cu): inputs normalised to [-1, 1]^5,
Fourier features [sin, cos](2 pi B u), 4 x (H, SiLU) with H = 256 or 64, a head of 8 outputs (padded
to 16), loss =
cross-entropy over 3 logits + squared errors of r_disk / 30 and ln g (disk rays) and of the escape
unit vector (escaped rays), batch means.

With `emulate_bf16=True` the values the GPU stores in BF16 are rounded the same way (features,
weights, pre-activations z, activations, dY, dZ) and the activation is evaluated as the GPU does it
(BF16 half-argument, BF16 tanh, one BF16 multiply-add); everything else stays float64, so the
difference from the GPU is its FP32 accumulation order and the hardware tanh approximations.
"""
from __future__ import annotations

import numpy as np

N_IN, N_FREQ, N_FEAT, N_HID, N_OUT, N_OUT_PAD = 5, 32, 64, 256, 8, 16
IMAGE_SCALE = 12.0


def layers(width=N_HID):
    """(fan_out, fan_in) per layer for hidden width `width`."""
    return ((width, N_FEAT), (width, width), (width, width), (width, width), (N_OUT_PAD, width))


LAYERS = layers()


def width_of(p):
    """The hidden width whose parameter count is the length of p."""
    for w in (64, 256):
        if sum(fo * fi + fo for fo, fi in layers(w)) == len(p):
            return w
    raise ValueError("parameter vector matches no hidden width")


def unpack(p):
    res, o = [], 0
    for fo, fi in layers(width_of(p)):
        W = p[o:o + fo * fi].reshape(fo, fi)
        o += fo * fi
        b = p[o:o + fo]
        o += fo
        res.append((W, b))
    return res


def num_params(width=N_HID):
    return sum(fo * fi + fo for fo, fi in layers(width))


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def normalise(x):
    x = np.asarray(x, dtype=np.float32)
    u = np.empty_like(x)
    u[:, 0] = x[:, 0] * np.float32(2.0 / 0.998) - np.float32(1.0)
    u[:, 1] = (x[:, 1] - np.float32(0.0872664626)) * np.float32(2.0 / 1.4660765717) - np.float32(1.0)
    u[:, 2] = (x[:, 2] - np.float32(1.3010299957)) * np.float32(2.0 / 1.6989700043) - np.float32(1.0)
    u[:, 3] = x[:, 3] * np.float32(1.0 / IMAGE_SCALE)
    u[:, 4] = x[:, 4] * np.float32(1.0 / IMAGE_SCALE)
    return u.astype(np.float64)


def features(x, B):
    u = normalise(x)
    p = u @ np.asarray(B, dtype=np.float64).T
    return np.concatenate([np.sin(2 * np.pi * p), np.cos(2 * np.pi * p)], axis=1)


def sigmoid(z):
    return 0.5 + 0.5 * np.tanh(0.5 * z)


def silu_bf16(z):
    """The GPU's activation: with h = bf16(z / 2), t = tanh(h) in BF16, silu = bf16(h t + h)."""
    h = bf16(0.5 * np.asarray(z, dtype=np.float64))
    t = bf16(np.tanh(h))
    return bf16(h * t + h)


def forward(p, B, x, emulate_bf16=False):
    """Returns (Y [n x 16], cache) with cache = (F, [z_l], [a_l], weights used)."""
    rnd = bf16 if emulate_bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    layers = [(rnd(W), np.asarray(b, dtype=np.float64)) for W, b in unpack(np.asarray(p, dtype=np.float64))]
    F = rnd(features(x, B))
    h, zs, acts = F, [], []
    for W, b in layers[:4]:
        z = h @ W.T + b
        a = silu_bf16(z) if emulate_bf16 else z * sigmoid(z)
        zs.append(rnd(z))
        acts.append(a)
        h = a
    W5, b5 = layers[4]
    Y = h @ W5.T + b5
    return Y, (F, zs, acts, layers)


def loss_terms(Y, cls, tgt, weights=(1.0, 1.0, 1.0, 1.0)):
    """(terms[4], dY [n x 16] of their weighted sum) for class labels 1..3 (others ignored)."""
    n = Y.shape[0]
    c = np.asarray(cls, dtype=np.int64) - 1
    tgt = np.asarray(tgt, dtype=np.float64)
    L = Y[:, :3]
    m = L.max(axis=1, keepdims=True)
    e = np.exp(L - m)
    P = e / e.sum(axis=1, keepdims=True)
    d = np.zeros_like(Y)
    terms = np.zeros(4)
    valid = (c >= 0) & (c < 3)
    idx = np.nonzero(valid)[0]
    terms[0] = -np.log(np.maximum(P[idx, c[idx]], 1e-30)).sum() / n
    onehot = np.zeros((n, 3))
    onehot[idx, c[idx]] = 1.0
    d[:, :3] = np.where(valid[:, None], P - onehot, 0.0) / n
    disk = c == 1
    esc = c == 2
    er = np.where(disk, Y[:, 3] - tgt[:, 3], 0.0)
    eg = np.where(disk, Y[:, 4] - tgt[:, 4], 0.0)
    terms[1] = (er ** 2).sum() / n
    terms[2] = (eg ** 2).sum() / n
    d[:, 3] = 2 * er / n
    d[:, 4] = 2 * eg / n
    ev = np.where(esc[:, None], Y[:, 5:8] - tgt[:, 5:8], 0.0)
    terms[3] = (ev ** 2).sum() / n
    d[:, 5:8] = 2 * ev / n
    w = np.asarray(weights, dtype=np.float64)
    d[:, :3] *= w[0]
    d[:, 3] *= w[1]
    d[:, 4] *= w[2]
    d[:, 5:8] *= w[3]
    return terms, d


def gradients(p, B, x, cls, tgt, emulate_bf16=False, weights=(1.0, 1.0, 1.0, 1.0)):
    """(flat gradient of the weighted sum of the loss terms, terms[4])."""
    rnd = bf16 if emulate_bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    Y, (F, zs, acts, layers) = forward(p, B, x, emulate_bf16)
    terms, d = loss_terms(Y, cls, tgt, weights)
    grads = []
    dY = rnd(d)
    W5, _ = layers[4]
    grads.append((dY.T @ acts[3], d.sum(axis=0)))
    dA = dY @ W5
    for l in range(3, -1, -1):
        z = zs[l]
        s = sigmoid(z)
        dz = dA * s * (1.0 + z * (1.0 - s))
        dzr = rnd(dz)
        h = F if l == 0 else acts[l - 1]
        grads.append((dzr.T @ h, dz.sum(axis=0)))
        if l > 0:
            dA = dzr @ layers[l][0]
    grads = grads[::-1]
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return flat, terms


def loss(p, B, x, cls, tgt):
    Y, _ = forward(p, B, x)
    return loss_terms(Y, cls, tgt)[0].sum()
