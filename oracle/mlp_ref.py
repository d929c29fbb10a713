"""CPU restatement of the surrogate network's forward pass, MSE loss and gradient.

TEST INFRASTRUCTURE ONLY: the GPU tests compare the library's BF16 tensor-core kernels
against this numpy version. BF16 rounding (round to nearest even) is applied at the same
points as the kernels (network input, hidden activations, weights, the loss gradient that
feeds the GEMMs); everything else is FP64 here versus FP32 accumulation on the GPU.
"""
from __future__ import annotations

import math

import numpy as np


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


_erf = np.vectorize(math.erf)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_d(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2 * math.pi)


def unpack(params, widths):
    out, o = [], 0
    for a, b in zip(widths[:-1], widths[1:]):
        W = params[o:o + a * b].reshape(a, b); o += a * b
        bb = params[o:o + b]; o += b
        out.append((W.astype(np.float64), bb.astype(np.float64)))
    return out


def forward(params, widths, x, norm):
    in_mu, in_sd, out_mu, out_sd = norm
    layers = unpack(params, widths)
    h = bf16((x - in_mu) / in_sd).astype(np.float64)
    hs, zs = [h], []
    for l, (W, b) in enumerate(layers):
        z = h @ bf16(W).astype(np.float64) + b
        zs.append(z)
        if l < len(layers) - 1:
            h = bf16(gelu(z)).astype(np.float64)
            hs.append(h)
    y = zs[-1] * out_sd + out_mu
    return y, hs, zs


def loss_grad(params, widths, x, t, norm):
    in_mu, in_sd, out_mu, out_sd = norm
    layers = unpack(params, widths)
    y, hs, zs = forward(params, widths, x, norm)
    tn = (t - out_mu) / out_sd
    d = zs[-1] - tn
    n = d.size
    loss = float((d * d).sum() / n)
    dz = 2 * d / n
    grads = []
    for l in range(len(layers) - 1, -1, -1):
        W, b = layers[l]
        dzb = bf16(dz).astype(np.float64)
        gW = hs[l].T @ dzb
        gb = dz.sum(0)
        grads.append((gW, gb))
        if l > 0:
            dh = dzb @ bf16(W).astype(np.float64).T
            dz = dh * gelu_d(zs[l - 1])
    grads.reverse()
    g = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, g
