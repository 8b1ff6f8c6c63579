"""CPU oracle of the super-resolution network's kernels (numpy).

TEST INFRASTRUCTURE ONLY: tests/ use it to check the BF16 tensor-core
kernels of include/lh_srnet.h (forward convolution with its epilogue, data and
weight gradients, loss, AdamW) and the gradient of the whole network.  The
product never imports it.  The learned warm start has no counterpart in the
reference, so there is nothing of the reference to pin; these functions are
the plain definitions of the operations, evaluated in float64 on the same
bf16-rounded operands the kernels read.

Layouts match the kernels: activations [Y][Z][X][C], weights [27][Cout][Cin]
with tap = (dy+1)*9 + (dz+1)*3 + (dx+1); x and z periodic, y zero-padded.
"""
from __future__ import annotations

import numpy as np

BIAS, RELU, GATE, RES = 8, 1, 4, 2


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64).astype(np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def bf16_bits(a: np.ndarray) -> np.ndarray:
    """bfloat16 bit patterns (uint16) of float32 values (rounded as bf16_round)."""
    return (bf16_round(a).view(np.uint32) >> 16).astype(np.uint16)


def from_bf16_bits(b: np.ndarray) -> np.ndarray:
    return (b.astype(np.uint32) << 16).view(np.float32)


def shifted(a: np.ndarray, oy: int, oz: int, ox: int) -> np.ndarray:
    """s[y, z, x] = a[y + oy, (z + oz) mod Z, (x + ox) mod X], zero outside y."""
    Y = a.shape[0]
    s = np.roll(np.roll(a, -oz, axis=1), -ox, axis=2)
    out = np.zeros_like(s)
    lo, hi = max(0, -oy), min(Y, Y - oy)
    if hi > lo:
        out[lo:hi] = s[lo + oy:hi + oy]
    return out


def taps():
    for t in range(27):
        yield t, t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1


def conv_fwd(x, w, bias=None, res=None, gate=None, flags=0):
    """Forward convolution with the kernel's epilogue, in float64."""
    x = np.asarray(x, np.float64)
    w = np.asarray(w, np.float64)
    out = np.zeros(x.shape[:3] + (w.shape[1],))
    for t, oy, oz, ox in taps():
        out += shifted(x, oy, oz, ox) @ w[t].T
    if flags & BIAS:
        out += bias
    if flags & RELU:
        out = np.maximum(out, 0.0)
    if flags & GATE:
        out = np.where(np.asarray(gate) > 0, out, 0.0)
    if flags & RES:
        out += res
    return out


def conv_dgrad(dout, w):
    """Data gradient of conv_fwd (without epilogue)."""
    dout = np.asarray(dout, np.float64)
    w = np.asarray(w, np.float64)
    dx = np.zeros(dout.shape[:3] + (w.shape[2],))
    for t, oy, oz, ox in taps():
        dx += shifted(dout @ w[t], -oy, -oz, -ox)
    return dx


def conv_wgrad(x, dout):
    """Weight and bias gradients of conv_fwd: dw [27][Cout][Cin], db [Cout]."""
    x = np.asarray(x, np.float64)
    dout = np.asarray(dout, np.float64)
    co, ci = dout.shape[-1], x.shape[-1]
    dw = np.zeros((27, co, ci))
    D = dout.reshape(-1, co)
    for t, oy, oz, ox in taps():
        dw[t] = D.T @ shifted(x, oy, oz, ox).reshape(-1, ci)
    return dw, D.sum(axis=0)


def flip_weights(w):
    """wt[tap][ci][co] = w[26 - tap][co][ci]."""
    return np.ascontiguousarray(np.transpose(w[::-1], (0, 2, 1)))


def mse(corr, base, target):
    """Loss and its gradient with respect to corr (16 channels, 0..2 used)."""
    nvox = base.shape[0]
    d = base.astype(np.float64) + corr[:, :3].astype(np.float64) - target.astype(np.float64)
    g = np.zeros(corr.shape)
    g[:, :3] = 2.0 * d / (3.0 * nvox)
    return float(np.sum(d * d) / (3.0 * nvox)), g


def adam(p, g, m, v, lr, b1, b2, eps, wd, step):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh, vh = m / (1 - b1 ** step), v / (1 - b2 ** step)
    p = p * (1 - lr * wd) - lr * mh / (np.sqrt(vh) + eps)
    return p, m, v


def network_loss_and_grads(params, x, base, target, nblocks=4, round_bf16=True):
    """The whole network in float64 with activations rounded to bf16 where
    the kernels store them (round_bf16=False: no rounding, for finite
    differences): returns the loss and the gradients of every parameter (same
    structure as params: list of (w, b))."""
    r = bf16_round if round_bf16 else (lambda a: np.asarray(a, np.float64))
    h = r(conv_fwd(x, params[0][0], params[0][1], flags=BIAS))
    hs = [h]
    for b in range(nblocks):
        w1, b1 = params[1 + 2 * b]
        w2, b2 = params[2 + 2 * b]
        t = r(conv_fwd(h, w1, b1, flags=BIAS | RELU))
        h = r(conv_fwd(t, w2, b2, res=h, flags=BIAS | RES))
        hs.append(t)
        hs.append(h)
    wt, bt = params[-1]
    corr = conv_fwd(h, wt, bt, flags=BIAS)
    corr = corr.astype(np.float32) if round_bf16 else corr
    Y, Z, X = x.shape[:3]
    loss, dcorr = mse(corr.reshape(-1, corr.shape[-1]), base.reshape(-1, 3), target.reshape(-1, 3))
    dcorr = r(dcorr.reshape(Y, Z, X, -1).astype(np.float32 if round_bf16 else np.float64))
    grads = [None] * len(params)
    grads[-1] = conv_wgrad(h, dcorr)
    dh = r(conv_dgrad(dcorr, wt))
    for b in reversed(range(nblocks)):
        w1, _ = params[1 + 2 * b]
        w2, _ = params[2 + 2 * b]
        t, h_in = hs[1 + 2 * b], hs[2 * b]
        grads[2 + 2 * b] = conv_wgrad(t, dh)
        dpre = r(np.where(t > 0, conv_dgrad(dh, w2), 0.0))
        grads[1 + 2 * b] = conv_wgrad(h_in, dpre)
        dh = r(conv_dgrad(dpre, w1) + dh)
    grads[0] = conv_wgrad(x, dh)
    return loss, grads
