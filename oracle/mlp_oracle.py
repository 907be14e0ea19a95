"""FP64 restatement of the warm-start MLP's forward and backward passes
(test infrastructure: the checker for the GPU training kernels).

It mirrors the roundings the GPU path applies -- BF16 inputs, weights and
hidden activations, BF16 gradients as GEMM operands, everything else carried
in FP64 -- so that the remaining difference to the GPU gradients is FP32
accumulation order.
"""
import numpy as np
from scipy.special import erf

DIMS = (16, 256, 256, 256, 16)


def bf16(x):
    """Round to bfloat16 (round to nearest even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params, dims=DIMS):
    out, off = [], 0
    for l in range(len(dims) - 1):
        k, n = dims[l], dims[l + 1]
        W = params[off:off + k * n].reshape(k, n).astype(np.float64)
        off += k * n
        b = params[off:off + n].astype(np.float64)
        off += n
        out.append((W, b))
    return out


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)


def loss_and_grads(params, X, T, nout, emulate_bf16=True, dims=DIMS):
    """X: standardised features [M,16]; T: standardised targets [M,nout].
    Returns (sum of squared errors, flat gradient like the GPU's layout)."""
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, np.float64))
    layers = unpack(params, dims)
    M = X.shape[0]
    h = r(X)
    hs, zs = [h], []
    for l, (W, b) in enumerate(layers):
        z = h @ r(W) + b
        if l < len(layers) - 1:
            zs.append(z)
            h = r(gelu(z))
            hs.append(h)
        else:
            y = z
    d = np.zeros_like(y)
    d[:, :nout] = y[:, :nout] - T
    loss = float(np.sum(d * d))
    dZ = 2.0 * d / (M * nout)
    grads = []
    for l in range(len(layers) - 1, -1, -1):
        W, b = layers[l]
        gW = hs[l].T @ r(dZ)
        gb = dZ.sum(0)
        grads.append((gW, gb))
        if l > 0:
            dH = r(dZ) @ r(W).T
            dZ = dH * gelu_grad(zs[l - 1])
    grads.reverse()
    return loss, np.concatenate([np.concatenate([g.ravel(), b]) for g, b in grads])


def init_params(seed, dims=DIMS):
    rng = np.random.default_rng(seed)
    parts = []
    for l in range(len(dims) - 1):
        k, n = dims[l], dims[l + 1]
        bound = np.sqrt(6.0 / k)
        parts.append(rng.uniform(-bound, bound, k * n))
        parts.append(rng.uniform(-0.1, 0.1, n))
    return np.concatenate(parts).astype(np.float32)
