"""CPU oracle of the learned closure network (test infrastructure only: the
GPU tests use it as the checker; nothing in the product imports it).

FP64 numpy restatement of the network in include/psph.h: 6 -> 64 -> 64 -> 64
-> 1, SiLU hidden layers, softplus output, with the same BF16 rounding as the
GPU path (weights W1..W3, the standardised inputs and the first two hidden
activations; round to nearest even), and the training loss
mean((softplus(z) - y)^2) with straight-through gradients through the
roundings. The GPU's backward pass runs on the tensor cores, whose operands
are BF16: the deltas of layers 3 and 2 are rounded where they enter a
product (the deltas of the layer below, and the W3 / W2 gradients), as here.
The features follow the same definitions as the closure kernel.
"""
from __future__ import annotations

import numpy as np

NIN, NH = 6, 64
OW1 = 0
OB1 = OW1 + NH * NIN
OW2 = OB1 + NH
OB2 = OW2 + NH * NH
OW3 = OB2 + NH
OB3 = OW3 + NH * NH
OW4 = OB3 + NH
OB4 = OW4 + NH
NPARAMS = OB4 + 1


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    return {
        "W1": p[OW1:OB1].reshape(NH, NIN), "b1": p[OB1:OW2],
        "W2": p[OW2:OB2].reshape(NH, NH), "b2": p[OB2:OW3],
        "W3": p[OW3:OB3].reshape(NH, NH), "b3": p[OB3:OW4],
        "w4": p[OW4:OB4], "b4": p[OB4],
    }


def sigmoid(z):
    return 1.0 / (1.0 + np.exp(-z))


def silu(z):
    return z * sigmoid(z)


def dsilu(z):
    s = sigmoid(z)
    return s * (1.0 + z * (1.0 - s))


def softplus(z):
    return np.where(z > 20.0, z, np.log1p(np.exp(np.minimum(z, 20.0))))


def standardize(x, norm):
    x = np.asarray(x, np.float32)
    norm = np.asarray(norm, np.float32)
    return ((x - norm[:NIN]) * norm[NIN:2 * NIN]).astype(np.float32)


def forward(params, norm, x, quantize=True):
    """quantize=False drops the BF16 roundings (exact FP64 network, used to
    check the backward pass by finite differences)."""
    q = bf16 if quantize else (lambda a: np.asarray(a, np.float64))
    w = unpack(params)
    u = q(standardize(x, norm))
    z1 = u @ q(w["W1"]).T + w["b1"]
    a1 = q(silu(z1))
    z2 = a1 @ q(w["W2"]).T + w["b2"]
    a2 = q(silu(z2))
    z3 = a2 @ q(w["W3"]).T + w["b3"]
    a3 = silu(z3)
    z4 = a3 @ w["w4"] + w["b4"]
    return {"u": u, "z1": z1, "a1": a1, "z2": z2, "a2": a2, "z3": z3, "a3": a3, "z4": z4, "c": softplus(z4)}


def loss_grad(params, norm, x, y, quantize=True):
    q = bf16 if quantize else (lambda a: np.asarray(a, np.float64))
    w = unpack(params)
    f = forward(params, norm, x, quantize)
    y = np.asarray(y, np.float64)
    B = len(y)
    e = f["c"] - y
    loss = float(np.mean(e * e))
    g4 = 2.0 * e * sigmoid(f["z4"]) / B
    d3 = g4[:, None] * w["w4"][None, :] * dsilu(f["z3"])
    d2 = (q(d3) @ q(w["W3"])) * dsilu(f["z2"])
    d1 = (q(d2) @ q(w["W2"])) * dsilu(f["z1"])
    grad = np.zeros(NPARAMS)
    grad[OW1:OB1] = (d1.T @ f["u"]).ravel()
    grad[OB1:OW2] = d1.sum(0)
    grad[OW2:OB2] = (q(d2).T @ f["a1"]).ravel()
    grad[OB2:OW3] = d2.sum(0)
    grad[OW3:OB3] = (q(d3).T @ f["a2"]).ravel()
    grad[OB3:OW4] = d3.sum(0)
    grad[OW4:OB4] = g4 @ f["a3"]
    grad[OB4] = g4.sum()
    return loss, grad


def features(strain_rate, vort, density, rho0, h, dx, nnb, cs):
    """Raw closure features from per-particle fields (strain_rate (n, 9), the
    reference's fluid StrainRate; vort = |vorticity|; cs = sound speed Cs);
    same definitions as the closure kernel: rates in units of Cs / h."""
    S = np.asarray(strain_rate, np.float64).reshape(-1, 9)
    temp = (S[:, 0] ** 2 + 2 * S[:, 1] * S[:, 3] + 2 * S[:, 2] * S[:, 6] + S[:, 4] ** 2 + 2 * S[:, 5] * S[:, 7]
            + S[:, 8] ** 2)
    shear = np.sqrt(0.5 * temp)
    det = (S[:, 0] * (S[:, 4] * S[:, 8] - S[:, 5] * S[:, 7]) - S[:, 1] * (S[:, 3] * S[:, 8] - S[:, 5] * S[:, 6])
           + S[:, 2] * (S[:, 3] * S[:, 7] - S[:, 4] * S[:, 6]))
    with np.errstate(divide="ignore", invalid="ignore"):
        r3 = np.where(temp > 0, det / (temp * np.sqrt(temp)), 0.0)
    ts = np.asarray(h, np.float64) / np.asarray(cs, np.float64)
    f = np.stack([np.log(np.maximum(shear * ts, 1e-12)), r3, np.log(np.maximum(vort * ts, 1e-12)),
                  np.asarray(density) / rho0, np.asarray(h) / dx + 0 * shear, np.asarray(nnb, np.float64)], axis=1)
    return f, shear
