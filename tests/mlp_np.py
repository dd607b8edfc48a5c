"""CPU restatement of the surrogate network the GPU kernels compute (a test oracle).

Parameters per layer: W [in][out], b [out].  Hidden layers apply the exact GELU
z Phi(z) = z (1 + erf(z / sqrt 2)) / 2, the output layer is linear, the loss is the mean squared
error over every output.  With bf16=True, values are rounded to BF16 (round to nearest even) where
the kernels store BF16: the inputs, the weights, the hidden activations, the output gradient, the
activation gradients and the pre-activation gradients; sums are exact (float64 here, FP32 there).
"""
import numpy as np
from scipy.special import erf


def round_bf16(x):
    x = np.asarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def split(params, widths):
    out = []
    off = 0
    for a, b in zip(widths[:-1], widths[1:]):
        W = params[off:off + a * b].reshape(a, b)
        off += a * b
        bias = params[off:off + b]
        off += b
        out.append((np.asarray(W, dtype=np.float64), np.asarray(bias, dtype=np.float64)))
    return out


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def loss_and_grads(params, widths, x, y, bf16=True):
    r = round_bf16 if bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    layers = split(params, widths)
    acts = [r(x)]
    zs = []
    for i, (W, b) in enumerate(layers):
        z = acts[-1] @ r(W) + b
        zs.append(z)
        if i + 1 < len(layers):
            acts.append(r(gelu(z)))
    out = zs[-1]
    n = out.size
    diff = out - y
    loss = float(np.sum(diff * diff) / n)
    grads = []
    dz = r(2.0 * diff / n)
    for i in range(len(layers) - 1, -1, -1):
        W, b = layers[i]
        gW = acts[i].T @ dz
        gb = dz.sum(axis=0)
        grads.append((gW, gb))
        if i == 0:
            break
        da = r(dz @ r(W).T)
        dz = r(da * gelu_grad(zs[i - 1]))
    grads.reverse()
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat


def predict(params, widths, x, bf16=True):
    r = round_bf16 if bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    layers = split(params, widths)
    a = r(x)
    for i, (W, b) in enumerate(layers):
        z = a @ r(W) + b
        a = r(gelu(z)) if i + 1 < len(layers) else z
    return a
