"""CPU oracle of the learned warm start network (numpy, float64).

TEST INFRASTRUCTURE ONLY: the oracle of ofblend_gb300's network kernels
(csrc/flof_conv_tc.cu, csrc/flof_net.cu, csrc/flof_model.cu).  The network has no counterpart in
the reference, so this is a from-scratch restatement of the same
architecture, used for the forward pass and for the gradients of the GPU training
kernels: by finite differences of the loss, and by an analytic backward
pass (loss_and_grad) that is itself checked against finite differences.

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


def _conv_backward(x, w, ks, stride, dy):
    """Gradients (dx, dw, db) of conv(x, w, b, ks, stride) for output gradient dy."""
    Ro = dy.shape[0]
    dw = np.zeros_like(w)
    db = dy.reshape(-1, dy.shape[-1]).sum(axis=0)
    if ks == 1:
        xs = x[::stride, ::stride, ::stride, ::stride]
        dw[0] = xs.reshape(-1, xs.shape[-1]).T @ dy.reshape(-1, dy.shape[-1])
        dx = np.zeros_like(x)
        dx[::stride, ::stride, ::stride, ::stride] += dy @ w[0].T
        return dx, dw, db
    xp = np.pad(x, ((1, 1),) * 4 + ((0, 0),))
    dxp = np.zeros_like(xp)
    dy2 = dy.reshape(-1, dy.shape[-1])
    for tap in range(81):
        ox, oy, oz, ot = tap % 3, (tap // 3) % 3, (tap // 9) % 3, tap // 27
        idx = (slice(ot, ot + stride * Ro, stride), slice(oz, oz + stride * Ro, stride),
               slice(oy, oy + stride * Ro, stride), slice(ox, ox + stride * Ro, stride))
        sl = xp[idx]
        dw[tap] = sl.reshape(-1, sl.shape[-1]).T @ dy2
        dxp[idx] += dy @ w[tap].T
    return dxp[1:-1, 1:-1, 1:-1, 1:-1], dw, db


def loss_and_grad(params, i0, i1, target):
    """Loss and its analytic gradient (same layout as the parameter vector),
    by backpropagation through forward()'s graph, in float64."""
    L = split_params(np.asarray(params, np.float64))
    x = np.stack([i0, i1], axis=-1).astype(np.float64) * INPUT_SCALE

    def c(l, a):
        ci, co, ks, st, rl, _, _ = LAYERS[l]
        y = conv(a, L[l][0], L[l][1], ks, st)
        return np.maximum(y, 0.0) if rl else y

    a0 = c(0, x)
    a1 = c(1, a0)
    a2 = c(2, a1)
    a3 = c(3, a2)
    a4 = c(4, a3)
    c5 = upcat(a4, a2)
    a5 = c(5, c5)
    c6 = upcat(a5, a0)
    a6 = c(6, c6)
    out = c(7, a6)
    t = np.asarray(target, np.float64)
    n = out.size
    loss = float(np.mean((out - t) ** 2))
    grads = [None] * 8

    def back(l, inp, y, dy):
        if LAYERS[l][4]:
            dy = dy * (y > 0)
        dx, dw, db = _conv_backward(inp, L[l][0], LAYERS[l][2], LAYERS[l][3], dy)
        grads[l] = (dw, db)
        return dx

    def upcat_back(d, c1):
        dlo = d[..., :c1]
        R = d.shape[0]
        dlo = dlo.reshape(R // 2, 2, R // 2, 2, R // 2, 2, R // 2, 2, c1).sum(axis=(1, 3, 5, 7))
        return dlo, d[..., c1:]

    d6 = back(7, a6, out, 2.0 * (out - t) / n)
    dc6 = back(6, c6, a6, d6)
    d5, d0 = upcat_back(dc6, 32)
    dc5 = back(5, c5, a5, d5)
    d4, d2 = upcat_back(dc5, 64)
    d3 = back(4, a3, a4, d4)
    d2 = d2 + back(3, a2, a3, d3)
    d1 = back(2, a1, a2, d2)
    d0 = d0 + back(1, a0, a1, d1)
    back(0, x, a0, d0)
    g = np.concatenate([np.concatenate([dw.ravel(), db]) for dw, db in grads])
    return loss, g
