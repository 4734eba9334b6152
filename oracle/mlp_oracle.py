"""CPU reference of the learned proposer's MLP -- TEST INFRASTRUCTURE.

numpy restatement of the forward pass, loss and backward pass that the CUDA
kernels (geos-chem_gb300/csrc/kpp_mlp.cu) implement: 56 -> 128 -> 128 -> 5,
exact-erf GELU, weights rounded to bf16, activations/accumulation in float64
here (the GPU accumulates in fp32, so agreement is to fp32 rounding).
Loss: mean squared error on output 0 + w_ce * mean softmax cross-entropy on
outputs 1..4.  Used only to check the GPU gradients.
"""
import numpy as np
from math import erf, sqrt, pi

_erf = np.vectorize(erf)


def bf16(a):
    """Round float32 values to bf16 (round to nearest even), returned as float64."""
    a = np.asarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    u = ((u + rounding) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / sqrt(2.0)))


def gelu_grad(z):
    cdf = 0.5 * (1.0 + _erf(z / sqrt(2.0)))
    pdf = np.exp(-0.5 * z * z) / sqrt(2.0 * pi)
    return cdf + z * pdf


def forward(x, p):
    W1, W2, W3 = bf16(p["w1"]), bf16(p["w2"]), bf16(p["w3"])
    z1 = x @ W1.T + p["b1"]
    h1 = gelu(z1)
    z2 = h1 @ W2.T + p["b2"]
    h2 = gelu(z2)
    out = h2 @ W3.T + p["b3"]
    return dict(z1=z1, h1=h1, z2=z2, h2=h2, out=out, W1=W1, W2=W2, W3=W3)


def loss_and_grads(x, y_h, y_bin, p, w_ce=0.5):
    x = np.asarray(x, np.float64)
    M = x.shape[0]
    f = forward(x, p)
    out = f["out"]
    e = out[:, 0] - y_h
    logits = out[:, 1:]
    mx = logits.max(axis=1, keepdims=True)
    ex = np.exp(logits - mx)
    s = ex.sum(axis=1, keepdims=True)
    q = ex / s
    ce = -(logits[np.arange(M), y_bin] - mx[:, 0] - np.log(s[:, 0]))
    loss = np.mean(e * e) + w_ce * np.mean(ce)
    dout = np.zeros_like(out)
    dout[:, 0] = 2.0 * e / M
    onehot = np.zeros_like(q)
    onehot[np.arange(M), y_bin] = 1.0
    dout[:, 1:] = w_ce * (q - onehot) / M
    g = {}
    g["w3"] = dout.T @ f["h2"]
    g["b3"] = dout.sum(0)
    dh2 = dout @ f["W3"]
    dz2 = dh2 * gelu_grad(f["z2"])
    g["w2"] = dz2.T @ f["h1"]
    g["b2"] = dz2.sum(0)
    dh1 = dz2 @ f["W2"]
    dz1 = dh1 * gelu_grad(f["z1"])
    g["w1"] = dz1.T @ x
    g["b1"] = dz1.sum(0)
    return loss, g, f
