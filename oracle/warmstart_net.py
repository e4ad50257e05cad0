"""CPU oracle of the learned warm start network (numpy, float64).

TEST INFRASTRUCTURE ONLY: the oracle of ofblend_gb300's network kernels
(csrc/flof_net.cu, csrc/flof_model.cu).  The network has no counterpart in
the reference, so this is a from-scratch restatement of the same
architecture, used for the forward pass and, by finite differences, for the
gradients of the GPU training kernels.

Layout: a tensor over a cubic 4D grid of extent R with C channels is an
array of shape (R, R, R, R, C) indexed [t, z, y, x, c].  Weights of a 3^4
convolution are W[tap, ci, co] with tap = ox + 3 (oy + 3 (oz + 3 ot)), the
offsets along x, y, z, t in 0..2 (padding 1); a 1^4 convolution has one tap.
The parameter vector holds, layer by layer, the weights then the biases.
"""
from __future__ import annotations

import numpy as np

INPUT_SCALE = -200.0
# (cin, cout, kernel, stride, relu, in_div, out_div) of E1, D1, E2, D2, B, U2, U1, O
LAYERS = [(2, 16, 3, 1, 1, 1, 1), (16, 32, 3, 2, 1, 1, 2), (32, 32, 3, 1, 1, 2, 2),
          (32, 64, 3, 2, 1, 2, 4), (64, 64, 3, 1, 1, 4, 4), (96, 32, 3, 1, 1, 2, 2),
          (48, 16, 3, 1, 1, 1, 1), (16, 4, 1, 1, 0, 1, 1)]


def split_params(p: np.ndarray):
    out, off = [], 0
    for cin, cout, ks, _, _, _, _ in LAYERS:
        taps = 81 if ks == 3 else 1
        w = p[off:off + taps * cin * cout].reshape(taps, cin, cout)
        off += taps * cin * cout
        b = p[off:off + cout]
        off += cout
        out.append((w, b))
    assert off == p.size
    return out


def num_params() -> int:
    return sum((81 if ks == 3 else 1) * ci * co + co for ci, co, ks, _, _, _, _ in LAYERS)


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round float32 values to the nearest bfloat16 (ties to even)."""
    u = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def conv(x: np.ndarray, w: np.ndarray, b: np.ndarray, ks: int, stride: int) -> np.ndarray:
    R = x.shape[0]
    Ro = R // stride
    cout = w.shape[2]
    out = np.zeros((Ro, Ro, Ro, Ro, cout), np.float64)
    if ks == 1:
        out += x[::stride, ::stride, ::stride, ::stride] @ w[0]
    else:
        xp = np.pad(x, ((1, 1),) * 4 + ((0, 0),))
        for tap in range(81):
            ox, oy, oz, ot = tap % 3, (tap // 3) % 3, (tap // 9) % 3, tap // 27
            sl = xp[ot:ot + stride * Ro:stride, oz:oz + stride * Ro:stride,
                    oy:oy + stride * Ro:stride, ox:ox + stride * Ro:stride]
            out += sl @ w[tap]
    return out + b


def upcat(lo: np.ndarray, skip: np.ndarray) -> np.ndarray:
    up = lo.repeat(2, 0).repeat(2, 1).repeat(2, 2).repeat(2, 3)
    return np.concatenate([up, skip], axis=-1)


def forward(params: np.ndarray, i0: np.ndarray, i1: np.ndarray) -> np.ndarray:
    """Velocity (R, R, R, R, 4) for coarse inputs i0, i1 of shape (R, R, R, R)."""
    L = split_params(np.asarray(params, np.float64))
    x = np.stack([i0, i1], axis=-1).astype(np.float64) * INPUT_SCALE
    relu = lambda a: np.maximum(a, 0.0)

    def c(l, a):
        ci, co, ks, st, rl, _, _ = LAYERS[l]
        y = conv(a, L[l][0], L[l][1], ks, st)
        return relu(y) if rl else y

    a0 = c(0, x)
    a1 = c(1, a0)
    a2 = c(2, a1)
    a3 = c(3, a2)
    a4 = c(4, a3)
    a5 = c(5, upcat(a4, a2))
    a6 = c(6, upcat(a5, a0))
    return c(7, a6)


def loss(params, i0, i1, target) -> float:
    pred = forward(params, i0, i1)
    return float(np.mean((pred - np.asarray(target, np.float64)) ** 2))


def fd_grad(params, i0, i1, target, idx, rel=1e-3) -> np.ndarray:
    """Central finite differences of the loss for the parameters idx."""
    p = np.asarray(params, np.float64).copy()
    g = np.empty(len(idx))
    for k, i in enumerate(idx):
        h = rel * max(abs(p[i]), 1e-2)
        old = p[i]
        p[i] = old + h
        lp = loss(p, i0, i1, target)
        p[i] = old - h
        lm = loss(p, i0, i1, target)
        p[i] = old
        g[k] = (lp - lm) / (2 * h)
    return g
