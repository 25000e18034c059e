"""Float64 CPU oracle for the surrogate MLP's kernels (test infrastructure
only).

Mirrors the computation of the surrogate kernels: inputs are syndrome bits,
hidden layers are ReLU, the output layer gives logits, the loss is the mean
soft-target cross-entropy.  With ``bf16=True`` the values the kernels round
to bfloat16 (weights, stored activations, output gradient and hidden
gradients) are rounded here at the same points, so the remaining difference
is float32 accumulation order; with ``bf16=False`` it is the exact float64
network the kernels approximate.
"""
import numpy as np


def round_bf16(x):
    """Round-to-nearest-even to bfloat16, returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = (u + 0x7FFF + lsb) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def layout(n_in, hidden, n_layers, n_out):
    """(w_off, dout, din, b_off) per layer, the parameter vector layout of
    tqec_mlp (layer 0's din is n_in rounded up to 64)."""
    in_pad = (n_in + 63) // 64 * 64
    out = []
    off = 0
    for l in range(n_layers):
        din = in_pad if l == 0 else hidden
        dout = n_out if l == n_layers - 1 else hidden
        w_off = off
        off += din * dout
        b_off = off
        off += dout
        off = (off + 7) // 8 * 8
        out.append((w_off, dout, din, b_off))
    return out, off


def unpack(packed, n_bits, in_pad):
    bits = np.unpackbits(np.atleast_2d(packed), axis=1, count=n_bits, bitorder="little").astype(np.float64)
    x = np.zeros((bits.shape[0], in_pad))
    x[:, :n_bits] = bits
    return x


def forward_backward(params, packed, targets, n_in, hidden, n_layers, n_out, bf16=True):
    """Returns (loss, grads) for the flat parameter vector."""
    lay, n = layout(n_in, hidden, n_layers, n_out)
    rb = round_bf16 if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    W = [params[o:o + dout * din].reshape(dout, din).astype(np.float64) for o, dout, din, _ in lay]
    B = [params[b:b + dout].astype(np.float64) for _, dout, _, b in lay]
    Wq = [rb(w) for w in W]
    x = unpack(packed, n_in, lay[0][2])
    acts = [x]
    h = x
    for l in range(n_layers - 1):
        h = rb(np.maximum(h @ Wq[l].T + B[l], 0.0))
        acts.append(h)
    logits = h @ Wq[-1].T + B[-1]
    m = logits.max(axis=1, keepdims=True)
    lse = np.log(np.exp(logits - m).sum(axis=1, keepdims=True)) + m
    logp = logits - lse
    t = np.asarray(targets, dtype=np.float64)
    rows = logits.shape[0]
    loss = float(-(t * logp).sum() / rows)
    dy = rb((np.exp(logp) - t) / rows)
    g = np.zeros(n)
    for l in range(n_layers - 1, -1, -1):
        w_off, dout, din, b_off = lay[l]
        g[w_off:w_off + dout * din] = (dy.T @ acts[l]).ravel()
        g[b_off:b_off + dout] = dy.sum(axis=0)
        if l > 0:
            dy = rb((dy @ Wq[l]) * (acts[l] > 0))
    return loss, g
