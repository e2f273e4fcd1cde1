"""CPU (numpy, FP64) oracle of the closure network: forward pass, MSE loss and
gradients, for checking the GPU's BF16 tensor-core kernels.

TEST INFRASTRUCTURE ONLY. The network has no counterpart in GENESIS 1.3 v4; this
restates the GPU network's definition (genesis-1.3-version4_gb300/csrc/
g4gpu_learned.cpp): layers nin -> width -> width -> width -> nout, widths padded to
multiples of 16, ReLU after every hidden layer, parameters stored per layer as
W [n_out][n_in] then b [n_out]. With bf16=True the operands that the GPU rounds to
BF16 (inputs, weights, activations and output gradients entering a GEMM) are rounded
the same way, so that the remaining difference is summation order.
"""
import numpy as np


def round_bf16(a):
    """Round-to-nearest-even to bfloat16, returned as float64."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def pad16(n):
    return (n + 15) // 16 * 16


def unpack(params, nin, width, nout):
    dims = [pad16(nin), pad16(width), pad16(width), pad16(width), pad16(nout)]
    layers, o = [], 0
    for l in range(4):
        k, n = dims[l], dims[l + 1]
        W = params[o:o + n * k].reshape(n, k).astype(np.float64)
        o += n * k
        b = params[o:o + n].astype(np.float64)
        o += n
        layers.append((W, b))
    return layers, dims


def forward_backward(params, X, T, nin, width, nout, bf16=True):
    """Returns (Y [n][nout], loss, grads flat like params). X and T are normalised."""
    rnd = round_bf16 if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    layers, dims = unpack(params, nin, width, nout)
    n = X.shape[0]
    A0 = np.zeros((n, dims[0]))
    A0[:, :nin] = X
    acts = [A0]
    for l, (W, b) in enumerate(layers):
        Z = rnd(acts[l]) @ rnd(W).T + b
        acts.append(np.maximum(Z, 0) if l < 3 else Z)
    Y = acts[4][:, :nout]
    diff = Y - T
    loss = float(np.mean(diff ** 2))
    dZ = np.zeros_like(acts[4])
    dZ[:, :nout] = 2.0 * diff / (n * nout)
    grads = [None] * 4
    for l in range(3, -1, -1):
        W, b = layers[l]
        grads[l] = (rnd(dZ).T @ rnd(acts[l]), dZ.sum(axis=0))
        if l > 0:
            dZ = (rnd(dZ) @ rnd(W)) * (acts[l] > 0)
    flat = np.concatenate([np.concatenate([dW.ravel(), db]) for dW, db in grads])
    return Y, loss, flat
