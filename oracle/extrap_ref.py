"""CPU restatement of the learned extrapolator's forward and backward passes (test infrastructure).

Mirrors em_lab_gb300/extrap.py + csrc/learn.cu operation for operation: BF16 rounding (round to
nearest even) of the input, the im2col columns, the weight copies, every activation and every
backward GEMM operand at exactly the points where the device kernels round; sums in FP64. With
exact=True no rounding is applied, for finite-difference checks of the backward formulas. Only the
tests import this module; the product never does.
"""
from __future__ import annotations

import numpy as np

from em_lab_gb300 import extrap as X


def bf16(a):
    """float32 -> nearest BF16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).reshape(a.shape)


def _r(a, exact):
    return np.asarray(a, np.float64) if exact else bf16(np.asarray(a, np.float32)).astype(np.float64)


def im2col(x, Lin, C, k, stride, pad, Lout):
    B = x.shape[0]
    cols = np.zeros((B, Lout, k, C), x.dtype)
    for l in range(Lout):
        for j in range(k):
            p = l * stride - pad + j
            if 0 <= p < Lin:
                cols[:, l, j, :] = x[:, p, :]
    return cols.reshape(B * Lout, k * C)


def col2im(dcols, B, Lin, C, k, stride, pad, Lout):
    d = dcols.reshape(B, Lout, k, C)
    dx = np.zeros((B, Lin, C), dcols.dtype)
    for l in range(Lout):
        for j in range(k):
            p = l * stride - pad + j
            if 0 <= p < Lin:
                dx[:, p, :] += d[:, l, j, :]
    return dx


def forward(params, x, zt, exact=False):
    """x (B, T_IN, 2), zt (B, AUX): every intermediate the backward pass needs, and y."""
    B = x.shape[0]
    W = {n: _r(params[n][0], exact) for n in params}
    b = {n: np.asarray(params[n][1], np.float64) for n in params}
    c1, c2 = X.CONV
    cache = {"W": W}
    x0 = _r(x, exact)
    cols1 = im2col(x0, c1[6], c1[1], c1[3], c1[4], c1[5], c1[7])
    z1 = cols1 @ W["conv1"].T + b["conv1"]
    a1 = _r(np.maximum(z1, 0.0), exact).reshape(B, c1[7], c1[2])
    cols2 = im2col(a1, c2[6], c2[1], c2[3], c2[4], c2[5], c2[7])
    z2 = cols2 @ W["conv2"].T + b["conv2"]
    enc = _r(np.maximum(z2, 0.0), exact).reshape(B, X.ENC)
    h = np.concatenate([enc, _r(zt, exact)], axis=1)
    cache.update(cols1=cols1, z1=z1, cols2=cols2, z2=z2, h0=h)
    zs, hs = {}, {"fc1": h}
    for k, (name, _, _, relu) in enumerate(X.HEAD):
        z = hs[name] @ W[name].T + b[name]
        zs[name] = z
        if k + 1 < len(X.HEAD):
            hs[X.HEAD[k + 1][0]] = _r(np.maximum(z, 0.0) if relu else z, exact)
    cache.update(z=zs, h=hs)
    return zs["out"], cache


def backward(params, cache, t, n, exact=False):
    """Gradients {name: (dW, db)} of the MSE over the first n rows (OUT outputs each)."""
    y = cache["z"]["out"]
    B = y.shape[0]
    W = cache["W"]
    dy = np.zeros_like(y)
    dy[:n] = 2.0 * (y[:n] - np.asarray(t[:n], np.float64)) / (n * X.OUT)
    grads = {}
    up = dy
    for name, _, _, relu in reversed(X.HEAD):
        dz = up * (cache["z"][name] > 0.0) if relu else up
        dzr = _r(dz, exact)
        grads[name] = (dzr.T @ cache["h"][name], dz.sum(axis=0))
        up = dzr @ W[name]
    c1, c2 = X.CONV
    dz2 = (up[:, :X.ENC].reshape(B * c2[7], c2[2])) * (cache["z2"] > 0.0)
    dz2r = _r(dz2, exact)
    grads["conv2"] = (dz2r.T @ cache["cols2"], dz2.sum(axis=0))
    dcols2 = dz2r @ W["conv2"]
    da1 = col2im(dcols2, B, c2[6], c2[1], c2[3], c2[4], c2[5], c2[7]).reshape(B * c1[7], c1[2])
    dz1 = da1 * (cache["z1"] > 0.0)
    dz1r = _r(dz1, exact)
    grads["conv1"] = (dz1r.T @ cache["cols1"], dz1.sum(axis=0))
    return grads


def loss(params, x, zt, t, n, exact=True):
    y, _ = forward(params, x, zt, exact)
    return float(np.sum((y[:n] - t[:n]) ** 2) / (n * X.OUT))
