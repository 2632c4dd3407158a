"""CPU restatement of the learned surrogate (test infrastructure only).

The surrogate has no counterpart in the reference; this file states its
definition for the parity tests of the CUDA kernels in
wrach_gb300/csrc/surrogate.cu:

  features   for each particle taking part in the solve (the first
             `capacity` of its cell), the 12 nearest taking-part particles in
             the 3x3 cells around its cell (the candidates of its Jacobi
             iterations) by binary32 squared distance, ties by index, each as
             (dx, dy, dvx, dvy) relative to the particle; then its velocity;
             zero padding to 64; rounded to BF16.
  network    64 -> 64 -> 64 -> 2, GELU (tanh form) after the hidden layers, BF16
             weights and activations, accumulation in float64 here (FP32 on
             the GPU).
  gradients  of L = 0.5 * mean over rows of |y - t|^2, with the BF16
             roundings the tensor-core operands get on the GPU (dy, dz2, dz1).
"""
import math

import numpy as np

IN, HID, OUT_PAD, K = 64, 64, 8, 12
N_PARAMS = IN * HID + HID + HID * HID + HID + HID * OUT_PAD + OUT_PAD


def bf16(a):
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32).copy()
    nan = np.isnan(a)
    out[nan] = a[nan]
    return out


def bf16_bits(a):
    return bf16(a).view(np.uint32) >> 16


def unpack(p):
    p = np.asarray(p, np.float64)
    o = 0
    w1 = p[o:o + IN * HID].reshape(IN, HID); o += IN * HID
    b1 = p[o:o + HID]; o += HID
    w2 = p[o:o + HID * HID].reshape(HID, HID); o += HID * HID
    b2 = p[o:o + HID]; o += HID
    w3 = p[o:o + HID * OUT_PAD].reshape(HID, OUT_PAD); o += HID * OUT_PAD
    b3 = p[o:o + OUT_PAD]
    return w1, b1, w2, b2, w3, b3


def pack(w1, b1, w2, b2, w3, b3):
    return np.concatenate([w1.ravel(), b1, w2.ravel(), b2, w3.ravel(), b3]).astype(np.float32)


# GELU in its tanh form (Hendrycks & Gimpel, 2016), as the CUDA kernels
# compute it (there with the hardware tanh, relative error about 2^-11)
_C, _A = math.sqrt(2.0 / math.pi), 0.044715


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(_C * (z + _A * z ** 3)))


def gelu_grad(z):
    t = np.tanh(_C * (z + _A * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * _C * (1.0 + 3.0 * _A * z * z)


def _q(a, on):
    """BF16 rounding as the tensor-core operands get it (identity if off)."""
    a = np.asarray(a, np.float64)
    return bf16(a.astype(np.float32)).astype(np.float64) if on else a


def _weights(p, rb=True):
    w1, b1, w2, b2, w3, b3 = unpack(p)
    return _q(w1, rb), b1, _q(w2, rb), b2, _q(w3, rb), b3


def forward(p, x, round_bf16=True):
    """Network outputs (n, 2) and the intermediate values.  With
    round_bf16=False the same function without any BF16 rounding (smooth, for
    finite-difference checks)."""
    rb = round_bf16
    w1, b1, w2, b2, w3, b3 = _weights(p, rb)
    x = _q(x, rb)
    z1 = x @ w1 + b1
    h1 = _q(gelu(z1), rb)
    z2 = h1 @ w2 + b2
    h2 = _q(gelu(z2), rb)
    y = h2 @ w3 + b3
    return y[:, :2], (x, z1, h1, z2, h2)


def loss(p, x, t, round_bf16=True):
    y, _ = forward(p, x, round_bf16)
    e = y - np.asarray(t, np.float64)
    return 0.5 * np.sum(e * e) / x.shape[0]


def gradients(p, x, t, round_bf16=True):
    """(gradient in parameter order, loss) of 0.5 * mean |y - t|^2."""
    rb = round_bf16
    w1, b1, w2, b2, w3, b3 = _weights(p, rb)
    y, (xb, z1, h1, z2, h2) = forward(p, x, rb)
    n = x.shape[0]
    e = y - np.asarray(t, np.float64)
    loss = 0.5 * np.sum(e * e) / n
    dy = np.zeros((n, OUT_PAD))
    dy[:, :2] = e / n
    dyq = _q(dy, rb)
    dz2 = (dyq @ w3.T) * gelu_grad(z2)
    dz2q = _q(dz2, rb)
    dz1 = (dz2q @ w2.T) * gelu_grad(z1)
    dz1q = _q(dz1, rb)
    g_w3 = h2.T @ dyq
    g_b3 = dy.sum(0)
    g_w2 = h1.T @ dz2q
    g_b2 = dz2.sum(0)
    g_w1 = xb.T @ dz1q
    g_b1 = dz1.sum(0)
    return pack(g_w1, g_b1, g_w2, g_b2, g_w3, g_b3).astype(np.float64), loss


def features(world_gx, world_gy, capacity, table, pos, vel):
    """BF16 features (n, 64) of a binned frame (reference-layout table)."""
    pos = np.asarray(pos, np.float32)
    vel = np.asarray(vel, np.float32)
    n = pos.shape[0]
    out = np.zeros((n, IN), np.float32)
    start = np.asarray(table, np.int64)[1:]
    for c in range(world_gx * world_gy):
        s, e = start[c], start[c + 1]
        cy, cx = divmod(c, world_gx)
        cand = []
        for ny in range(max(cy - 1, 0), min(cy + 1, world_gy - 1) + 1):
            for nx in range(max(cx - 1, 0), min(cx + 1, world_gx - 1) + 1):
                nc = ny * world_gx + nx
                js, je = start[nc], start[nc + 1]
                cand.extend(range(js, min(je, js + capacity)))
        cand = np.asarray(cand, np.int64)
        for i in range(s, min(e, s + capacity)):
            j = cand[cand != i]
            dx = (pos[j, 0] - pos[i, 0]).astype(np.float32)
            dy = (pos[j, 1] - pos[i, 1]).astype(np.float32)
            d = (dx * dx + dy * dy).astype(np.float32)
            order = np.lexsort((j, d))[:K]
            for k, o in enumerate(order):
                jj = j[o]
                out[i, 4 * k:4 * k + 4] = [pos[jj, 0] - pos[i, 0], pos[jj, 1] - pos[i, 1],
                                           vel[jj, 0] - vel[i, 0], vel[jj, 1] - vel[i, 1]]
            out[i, 4 * K:4 * K + 2] = vel[i]
    return bf16(out)
