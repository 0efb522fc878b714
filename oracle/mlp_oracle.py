"""CPU oracle of the surrogate MLP (test infrastructure only).

FP64 restatement of the network the GPU trains (omg_audio_gb300/csrc/mlp.cu,
api_mlp.cpp): layers n_in -> hidden (GELU, tanh form) -> ... -> n_out, mean
squared error over all outputs. With `bf16=True` it rounds what the GPU keeps
in BF16 (inputs, weights, hidden activations, the output gradient fed to the
GEMMs) to BF16 and does everything else in FP64, so the GPU's gradients differ
from it only by FP32 accumulation order; with `bf16=False` it is the plain
FP64 network. No reference counterpart: the reference has no surrogate.
"""
from __future__ import annotations

import numpy as np

K0 = 0.7978845608028654
K1 = 0.044715


def bf16(a):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    x = np.ascontiguousarray(a, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def bf16_bits(a):
    x = np.ascontiguousarray(a, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(K0 * (z + K1 * z ** 3)))


def gelu_grad(z):
    t = np.tanh(K0 * (z + K1 * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * K0 * (1.0 + 3.0 * K1 * z * z)


def forward(layers, x, bf=True):
    """layers: [(W [out x in], b [out])]; returns output and the saved (Z, A)."""
    r = bf16 if bf else (lambda a: np.asarray(a, np.float64))
    a = r(x)
    saved = []
    for i, (W, b) in enumerate(layers):
        z = a @ r(W).T + np.asarray(b, np.float64)
        saved.append((a, z))
        if i + 1 < len(layers):
            a = r(gelu(z).astype(np.float32)) if bf else gelu(z)
        else:
            a = z
    return a, saved


def loss_and_grads(layers, x, y, bf=True):
    r = bf16 if bf else (lambda a: np.asarray(a, np.float64))
    out, saved = forward(layers, x, bf)
    n = out.size
    err = out - np.asarray(y, np.float64)
    loss = float(np.mean(err * err))
    dz = 2.0 * err / n
    grads = [None] * len(layers)
    for i in range(len(layers) - 1, -1, -1):
        W, b = layers[i]
        a_in, z = saved[i]
        dzh = r(dz.astype(np.float32)) if bf else dz
        gW = dzh.T @ a_in
        gb = dz.sum(axis=0)
        grads[i] = (gW, gb)
        if i == 0:
            break
        dx = dzh @ r(W)
        dz = dx * gelu_grad(saved[i - 1][1])
    return loss, grads
