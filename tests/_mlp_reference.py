"""CPU reference of the device MLP (forward, loss, gradients) with the device's rounding points:
GEMM operands rounded to bfloat16 (round to nearest even), products accumulated exactly,
activations and gradients kept in FP32 between products."""
import numpy as np


def bf16(x):
    x32 = np.ascontiguousarray(x, dtype=np.float32)
    b = x32.view(np.uint32).astype(np.uint64)
    r = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(flat, n_in, n_hidden, n_layers, n_out):
    """Layer list [(W [out x in], b [out])] from the flat parameter order of mithra_mlp_weights."""
    out, w = [], 0
    dims = [n_in] + [n_hidden] * n_layers + [n_out]
    for l in range(n_layers + 1):
        i, o = dims[l], dims[l + 1]
        W = flat[w:w + o * i].reshape(o, i).astype(np.float64)
        w += o * i
        b = flat[w:w + o].astype(np.float64)
        w += o
        out.append((W, b))
    return out


def loss_and_grads(layers, X, Y, exact=False):
    """exact=True: no rounding at all (float64 throughout), for finite-difference checks."""
    rb = (lambda x: np.asarray(x, dtype=np.float64)) if exact else bf16
    f32 = (lambda x: x) if exact else (lambda x: x.astype(np.float32).astype(np.float64))
    B, n_out = Y.shape
    h = rb(X)
    ins, acts = [h], []
    z = None
    for l, (W, b) in enumerate(layers):
        z = f32(ins[-1] @ rb(W).T + b)
        if l < len(layers) - 1:
            a = np.maximum(z, 0.0)
            acts.append(a)
            ins.append(rb(a))
    loss = float(np.mean((z - Y) ** 2))
    dz = rb(2.0 * (z - Y) / (B * n_out))
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        W, _ = layers[l]
        gW = dz.T @ ins[l]
        gb = dz.sum(axis=0)
        grads[l] = (gW, gb)
        if l > 0:
            dh = f32(dz @ rb(W))
            dz = rb(dh * (acts[l - 1] > 0))
    flat = np.concatenate([np.concatenate([g.ravel(), gb]) for g, gb in grads])
    return loss, flat
