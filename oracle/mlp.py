"""FP64 numpy oracle of the learned-guess network -- TEST INFRASTRUCTURE ONLY.

Same architecture and parameter layout as the CUDA network (petrbf_gb300/csrc/mlp.cu):
layers 256 -> 256 -> 256 -> 256 -> 16, ReLU after the hidden layers, per layer
W[out][in] row-major then b[out]; the forward pass uses the weights rounded to BF16
(round to nearest even), the biases in FP32; the loss is the masked mean-squared error.
Gradients are taken with respect to the FP32 master weights through the BF16 rounding
(straight-through), as the CUDA backward does.

bf16_operands (the CUDA network's tensor-core GEMMs): every GEMM operand is rounded to BF16
as the network rounds it -- the features and hidden activations entering a layer, and the
output gradient dZ entering dW = dZ^T H and dH = dZ W -- while the products are summed in
FP64 here (FP32 on the GPU), the ReLU masks, biases and bias gradients stay unrounded.
"""
import numpy as np

LAYERS = [(256, 256), (256, 256), (256, 256), (256, 16)]


def bf16(a):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    u = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w, round_weights=True):
    out, o = [], 0
    for fin, fout in LAYERS:
        W = np.asarray(w[o:o + fin * fout], np.float64).reshape(fout, fin)
        o += fin * fout
        b = np.asarray(w[o:o + fout], np.float64)
        o += fout
        out.append((bf16(w[o - fout - fin * fout:o - fout]).reshape(fout, fin) if round_weights else W, b))
    return out


def _op(a, on):
    """A GEMM operand: rounded to BF16 (through FP32) when the GPU rounds it."""
    return bf16(np.asarray(a, np.float32)) if on else np.asarray(a, np.float64)


def forward(w, X, round_weights=True, bf16_operands=True):
    acts, h = [], np.asarray(X, np.float64)
    layers = unpack(w, round_weights)
    for k, (W, b) in enumerate(layers):
        z = _op(h, bf16_operands) @ W.T + b
        h = np.maximum(z, 0.0) if k < len(layers) - 1 else z
        acts.append(h)
    return acts


def loss_grad(w, X, T, M, round_weights=True, bf16_operands=True):
    X, T, M = (np.asarray(a, np.float64) for a in (X, T, M))
    layers = unpack(w, round_weights)
    acts = forward(w, X, round_weights, bf16_operands)
    cnt = M.sum()
    d = (acts[-1] - T) * M
    loss = (d * d).sum() / cnt
    dz = 2.0 * d / cnt
    grads = [None] * len(layers)
    for k in range(len(layers) - 1, -1, -1):
        hin = _op(acts[k - 1] if k > 0 else X, bf16_operands)
        W, _ = layers[k]
        dzo = _op(dz, bf16_operands)
        grads[k] = (dzo.T @ hin, dz.sum(axis=0))
        if k > 0:
            dz = (dzo @ W) * (acts[k - 1] > 0)
    flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    return loss, flat
