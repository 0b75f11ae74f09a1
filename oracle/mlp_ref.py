"""numpy restatement of the sizing MLP (8 -> 32 -> 32 -> 2, ReLU, MSE on
standardised targets) -- TEST INFRASTRUCTURE: the CPU check of the CUDA
forward / backward kernels in gpu_spgemm_gb300/csrc/mlp.cu."""
from __future__ import annotations

import numpy as np

NF, NH, NO = 8, 32, 2
OFF_W1 = 0
OFF_B1 = OFF_W1 + NH * NF
OFF_W2 = OFF_B1 + NH
OFF_B2 = OFF_W2 + NH * NH
OFF_W3 = OFF_B2 + NH
OFF_B3 = OFF_W3 + NO * NH
NPARAM = OFF_B3 + NO


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[OFF_W1:OFF_B1].reshape(NH, NF), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(NH, NH),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3].reshape(NO, NH), p[OFF_B3:NPARAM])


def forward(p, norm, X):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    norm = np.asarray(norm, np.float64)
    xin = (np.asarray(X, np.float64) - norm[:NF]) * norm[NF:2 * NF]
    h1 = np.maximum(xin @ W1.T + b1, 0)
    h2 = np.maximum(h1 @ W2.T + b2, 0)
    out = h2 @ W3.T + b3
    return xin, h1, h2, out


def gradient(p, norm, X, Y):
    """Gradient of mean((out - y_std)^2) over all outputs; returns (grad, loss)."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    norm = np.asarray(norm, np.float64)
    xin, h1, h2, out = forward(p, norm, X)
    y = (np.asarray(Y, np.float64) - norm[2 * NF:2 * NF + NO]) / norm[2 * NF + NO:]
    d = out - y
    nb = X.shape[0]
    loss = float((d * d).sum() / (nb * NO))
    dout = 2.0 * d / (nb * NO)
    g = np.zeros(NPARAM)
    g[OFF_W3:OFF_B3] = (dout.T @ h2).ravel()
    g[OFF_B3:] = dout.sum(0)
    dh2 = (dout @ W3) * (h2 > 0)
    g[OFF_W2:OFF_B2] = (dh2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = dh2.sum(0)
    dh1 = (dh2 @ W2) * (h1 > 0)
    g[OFF_W1:OFF_B1] = (dh1.T @ xin).ravel()
    g[OFF_B1:OFF_W2] = dh1.sum(0)
    return g, loss
