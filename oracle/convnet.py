"""CPU oracle of the learned preconditioner's network (test infrastructure:
only the tests load it, as the checker of csrc/precond_net.cu).

The network has no reference counterpart (the reference's SCF has no
preconditioner, chebyr_m.f90).  This is a NumPy restatement of what the
device kernels compute: three 'same' 3^3 convolutions over channels-last
[batch, z, y, x, 16] fields (zeros outside the box), SiLU after the first
two, weights [27 taps][16 ci][16 co] with tap = (dz+1)*9 + (dy+1)*3 + (dx+1),
and the interior mean-square loss of the two output channels.

`forward` / `loss_grad` with bf16=True round every stored quantity where the
device stores it as BF16 (inputs, weights, hidden activations, the
backpropagated gradients), so that the device results differ from these only
by FP32 summation order (and a rare BF16 rounding that lands on the other
side of a tie); with bf16=False they are plain FP64, for finite-difference
checks of the backward formulas.
"""
from __future__ import annotations

import numpy as np

CH = 16
TAPS = 27
WL = TAPS * CH * CH
PL = WL + CH
CIN = (3, 16, 16)
COUT = (16, 16, 2)


def bf16(a):
    """Round to BF16 (nearest, ties to even) and back to float64."""
    a32 = np.ascontiguousarray(a, np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32).astype(np.float64)


def bf16_bits(a):
    a32 = np.ascontiguousarray(a, np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def from_bits(b):
    return (np.asarray(b, np.uint32) << 16).view(np.float32).astype(np.float64)


def layer_params(p, l):
    blk = np.asarray(p, np.float64)[l * PL:(l + 1) * PL]
    return blk[:WL].reshape(TAPS, CH, CH), blk[WL:]


def silu(x):
    return x / (1.0 + np.exp(-x))


def silu_grad(x):
    s = 1.0 / (1.0 + np.exp(-x))
    return s * (1.0 + x * (1.0 - s))


def conv(x, W):
    """'same' 3^3 convolution: out[v, co] = sum_tap,ci x[v + off(tap), ci] W[tap, ci, co]."""
    b, nz, ny, nx, _ = x.shape
    xp = np.zeros((b, nz + 2, ny + 2, nx + 2, CH))
    xp[:, 1:-1, 1:-1, 1:-1] = x
    out = np.zeros((b, nz, ny, nx, CH))
    for tap in range(TAPS):
        dz, dy, dx = tap // 9, (tap // 3) % 3, tap % 3
        out += xp[:, dz:dz + nz, dy:dy + ny, dx:dx + nx] @ W[tap]
    return out


def conv_t(d, W):
    """Adjoint of `conv` in its input: dx[v, ci] = sum_tap,co d[v - off(tap), co] W[tap, ci, co]."""
    b, nz, ny, nx, _ = d.shape
    dp = np.zeros((b, nz + 2, ny + 2, nx + 2, CH))
    dp[:, 1:-1, 1:-1, 1:-1] = d
    out = np.zeros((b, nz, ny, nx, CH))
    for tap in range(TAPS):
        dz, dy, dx = tap // 9, (tap // 3) % 3, tap % 3
        out += dp[:, 2 - dz:2 - dz + nz, 2 - dy:2 - dy + ny, 2 - dx:2 - dx + nx] @ W[tap].T
    return out


def conv_wgrad(x, d):
    """dW[tap, ci, co] = sum_v x[v + off(tap), ci] d[v, co]."""
    b, nz, ny, nx, _ = x.shape
    xp = np.zeros((b, nz + 2, ny + 2, nx + 2, CH))
    xp[:, 1:-1, 1:-1, 1:-1] = x
    dW = np.zeros((TAPS, CH, CH))
    dm = d.reshape(-1, CH)
    for tap in range(TAPS):
        dz, dy, dx = tap // 9, (tap // 3) % 3, tap % 3
        dW[tap] = xp[:, dz:dz + nz, dy:dy + ny, dx:dx + nx].reshape(-1, CH).T @ dm
    return dW


def forward(params, x, bf16_round=True):
    """x float [batch, nz, ny, nx, 16] (the BF16 input values).  Returns the
    output [.., 16] and the intermediates (pre-activations, activations)."""
    rnd = bf16 if bf16_round else (lambda a: np.asarray(a, np.float64))
    acts = [rnd(x)]
    pres = []
    h = acts[0]
    for l in range(3):
        W, b = layer_params(params, l)
        z = conv(h, rnd(W)) + b
        pres.append(z)
        if l < 2:
            h = rnd(silu(z))
            acts.append(h)
        else:
            h = z
    return h, pres, acts


def interior_mask(P, margin):
    m = np.zeros((P, P, P), bool)
    m[margin:P - margin, margin:P - margin, margin:P - margin] = True
    return m


def loss_grad(params, x, tgt, margin, bf16_round=True):
    """Loss of a batch of P^3 patches and its gradient (layout of params)."""
    rnd = bf16 if bf16_round else (lambda a: np.asarray(a, np.float64))
    out, pres, acts = forward(params, x, bf16_round)
    b, P = x.shape[0], x.shape[1]
    mask = interior_mask(P, margin)[None, :, :, :, None]
    count = 2.0 * b * float((P - 2 * margin) ** 3)
    diff = (out[..., :2] - tgt) * mask
    loss = float((diff ** 2).sum() / count)
    d = np.zeros_like(out)
    d[..., :2] = rnd(2.0 * diff / count)
    grad = np.zeros(3 * PL)
    for l in (2, 1, 0):
        W, _ = layer_params(params, l)
        dW = conv_wgrad(acts[l], d)
        db = d.reshape(-1, CH).sum(axis=0)
        cin, cout = CIN[l], COUT[l]
        dW[:, cin:, :] = 0.0
        dW[:, :, cout:] = 0.0
        db[cout:] = 0.0
        grad[l * PL:l * PL + WL] = dW.reshape(-1)
        grad[l * PL + WL:(l + 1) * PL] = db
        if l > 0:
            d = rnd(conv_t(d, rnd(W)) * silu_grad(pres[l - 1]))
    return loss, grad
