"""FP64 numpy restatement of the learned-start MLP (TEST INFRASTRUCTURE ONLY).

The network maps potential parameters to starting-state coefficients: tanh hidden
layers, linear output, mean-squared-error loss averaged over every output element.
The GPU kernels multiply with BF16 copies of the FP32 master weights; this oracle
rounds the weights the same way (round to nearest even) and does the rest in FP64,
so gradients agree to FP32 accumulation accuracy.  No reference counterpart: the
Rust crate has no learned component.
"""
import numpy as np


def bf16(a):
    """Round FP32 values to the nearest BF16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params, widths):
    """Flat parameters (per layer: W out x in row-major, then b) -> [(W, b)]."""
    out, off = [], 0
    for i, o in zip(widths[:-1], widths[1:]):
        w = params[off:off + i * o].reshape(o, i)
        off += i * o
        b = params[off:off + o]
        off += o
        out.append((w, b))
    return out


def forward(params, widths, x):
    acts = [np.asarray(x, dtype=np.float64)]
    layers = unpack(params, widths)
    for li, (w, b) in enumerate(layers):
        z = acts[-1] @ bf16(w).T + b.astype(np.float64)
        acts.append(np.tanh(z) if li + 1 < len(layers) else z)
    return acts


def loss_and_gradients(params, widths, x, t):
    acts = forward(params, widths, x)
    layers = unpack(params, widths)
    y = acts[-1]
    d = y - np.asarray(t, dtype=np.float64)
    loss = float(np.mean(d * d))
    dz = 2.0 * d / d.size
    grads = []
    for li in range(len(layers) - 1, -1, -1):
        w, _ = layers[li]
        if li + 1 < len(layers):
            dz = dz * (1.0 - acts[li + 1] ** 2)
        gw = dz.T @ acts[li]
        gb = dz.sum(axis=0)
        grads.append((gw, gb))
        dz = dz @ bf16(w)
    grads.reverse()
    flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    return loss, flat
