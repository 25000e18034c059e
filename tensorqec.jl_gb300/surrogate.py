"""The learned surrogate with exact fallback.

A ReLU MLP (float32 master weights, bf16 GEMM operands, float32
accumulation; trained by the native library's own kernels) maps syndrome
bits to the logical class.  Its labels are the exact contraction's class
probabilities.  At decode time the rows whose softmax confidence is below a
calibrated threshold go to the exact contraction, which also serves as the
reference the surrogate's decisions are measured against.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import native
from .error_model import pack_syndromes, random_error_pattern, syndrome_extraction


class MLPConfig(C.Structure):
    _fields_ = [("n_in", C.c_int32), ("hidden", C.c_int32), ("n_layers", C.c_int32), ("n_out", C.c_int32),
                ("seed", C.c_uint64), ("device", C.c_int32)]


def _lib():
    L = native.lib()
    if not getattr(L, "_tqec_mlp_bound", False):
        vp, i64 = C.c_void_p, C.c_int64
        sig = {"tqec_mlp_create": [vp, vp], "tqec_mlp_destroy": [vp], "tqec_mlp_param_count": [vp, vp],
               "tqec_mlp_get_params": [vp, vp, i64], "tqec_mlp_set_params": [vp, vp, i64],
               "tqec_mlp_gradients": [vp, vp, vp, i64, vp, vp],
               "tqec_mlp_train_step": [vp, vp, vp, i64, C.c_float, vp, vp],
               "tqec_mlp_train_step_rows": [vp, vp, vp, i64, vp, i64, C.c_float, vp, vp],
               "tqec_mlp_infer": [vp, vp, i64, vp, vp, vp],
               "tqec_gated_decode": [vp, vp, C.c_float, vp, i64, vp, vp, vp],
               "tqec_gated_last_fallback": [vp, vp],
               "tqec_mlp_save": [vp, C.c_char_p], "tqec_mlp_load": [vp, C.c_char_p],
               "tqec_mlp_set_gemm": [vp, C.c_int], "tqec_mlp_forward_logits": [vp, vp, i64, vp]}
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = C.c_int
        L._tqec_mlp_bound = True
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Surrogate:
    """Owner of a native ``tqec_mlp``."""

    def __init__(self, n_in, n_out, hidden=512, n_layers=4, seed=1, device=0):
        self.cfg = dict(n_in=n_in, n_out=n_out, hidden=hidden, n_layers=n_layers)
        h = C.c_void_p()
        native.check(_lib().tqec_mlp_create(C.byref(MLPConfig(n_in, hidden, n_layers, n_out, seed, device)),
                                            C.byref(h)))
        self._h = h
        n = C.c_int64()
        native.check(_lib().tqec_mlp_param_count(self._h, C.byref(n)))
        self.n_params = n.value
        self.threshold = None

    def close(self):
        if getattr(self, "_h", None):
            _lib().tqec_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def params(self):
        out = np.empty(self.n_params, dtype=np.float32)
        native.check(_lib().tqec_mlp_get_params(self._h, _p(out), self.n_params))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        native.check(_lib().tqec_mlp_set_params(self._h, _p(p), p.size))

    def gradients(self, packed, targets):
        packed = np.ascontiguousarray(packed, dtype=np.uint8)
        targets = np.ascontiguousarray(targets, dtype=np.float32)
        g = np.empty(self.n_params, dtype=np.float32)
        loss = C.c_float()
        native.check(_lib().tqec_mlp_gradients(self._h, _p(packed), _p(targets), packed.shape[0], _p(g),
                                                C.byref(loss)))
        return g, loss.value

    def train_step(self, packed, targets, lr):
        packed = np.ascontiguousarray(packed, dtype=np.uint8)
        targets = np.ascontiguousarray(targets, dtype=np.float32)
        loss = C.c_float()
        native.check(_lib().tqec_mlp_train_step(self._h, _p(packed), _p(targets), packed.shape[0], lr,
                                                C.byref(loss), None))
        return loss.value

    def train_step_rows(self, syn_ptr, tgt_ptr, n_set, rows_ptr, n, lr, with_loss=False, stream=None):
        """One Adam step on rows[0..n) of a device-resident training set
        (raw device pointers); returns the loss only when asked (that call
        synchronises)."""
        loss = C.c_float()
        native.check(_lib().tqec_mlp_train_step_rows(self._h, C.c_void_p(syn_ptr), C.c_void_p(tgt_ptr), n_set,
                                                     C.c_void_p(rows_ptr), n, lr,
                                                     C.byref(loss) if with_loss else None,
                                                     C.c_void_p(stream) if stream else None))
        return loss.value if with_loss else None

    def infer(self, packed):
        packed = np.ascontiguousarray(packed, dtype=np.uint8)
        n = packed.shape[0]
        cls = np.empty(n, dtype=np.int32)
        conf = np.empty(n, dtype=np.float32)
        native.check(_lib().tqec_mlp_infer(self._h, _p(packed), n, _p(cls), _p(conf), None))
        return cls, conf

    def use_tensor_cores(self, on=True):
        """How the layers run: False (0) SIMT GEMMs; 1 or 2 tcgen05 GEMMs layer
        by layer (one block per SM with a 4-stage ring, or two with a 2-stage
        ring); True (3, the default) inference by the fused tcgen05 forward
        kernel where the shape allows, training as 2."""
        mode = 3 if on is True else (0 if on is False else int(on))
        native.check(_lib().tqec_mlp_set_gemm(self._h, mode))

    def logits(self, packed):
        packed = np.ascontiguousarray(packed, dtype=np.uint8)
        out = np.empty((packed.shape[0], self.cfg["n_out"]), dtype=np.float32)
        native.check(_lib().tqec_mlp_forward_logits(self._h, _p(packed), packed.shape[0], _p(out)))
        return out

    def save(self, path):
        native.check(_lib().tqec_mlp_save(self._h, path.encode()))

    def load(self, path):
        native.check(_lib().tqec_mlp_load(self._h, path.encode()))


def soft_labels(logp):
    """Class probabilities from log-marginals (rows normalised)."""
    m = np.max(logp, axis=1, keepdims=True)
    m = np.where(np.isfinite(m), m, 0.0)
    p = np.exp(logp - m)
    s = p.sum(axis=1, keepdims=True)
    return (p / np.where(s > 0, s, 1.0)).astype(np.float32)


def sample_bits(ct, n, rng):
    ep = random_error_pattern(ct.em, rng, nsamples=n)
    s = syndrome_extraction(ep, ct.tanner)
    return np.concatenate([s.sx, s.sz], axis=1)


def _draw_labelled(ct, sampler, rng, seed, offset, m, nbytes, label_precision=native.TQEC_F32):
    """m syndromes (GPU sampler at counter `offset`, or the host sampler) and
    their exact class probabilities (contracted in `label_precision`), as
    host arrays."""
    sub = 1 << 20
    packed = np.empty((m, nbytes), dtype=np.uint8)
    targets = np.empty((m, ct.n_classes), dtype=np.float32)
    for i in range(0, m, sub):
        k = min(sub, m - i)
        if sampler is not None:
            packed[i:i + k], _ = sampler.sample(seed, k, offset=offset + i)
        else:
            packed[i:i + k] = pack_syndromes(sample_bits(ct, k, rng))
        targets[i:i + k] = soft_labels(ct.program.contract_packed(packed[i:i + k], label_precision))
    return packed, targets


def train_surrogate(ct, n_train=1 << 24, batch=16384, epochs=4, lr=3e-3, hidden=512, n_layers=4, seed=1,
                    rng=None, log=None, gpu_sampler=True, chunk=0, device_resident=None, label_precision="f32"):
    """Trains a surrogate for a compiled CSS decoder on n_train sampled
    syndromes labelled by the exact contraction's class probabilities:
    label_precision "f32" (the renormalised float32 contraction, every class
    probability within the program's rounding bound of float64: 4.8e-5
    relative at d=7) or "f64" (the float64 contraction, about 4x slower to
    label).  Syndromes come from the GPU sampler (Philox, seeded by `seed`)
    or, with gpu_sampler=False, from the host sampler.  With chunk > 0 the
    syndromes are drawn and labelled `chunk` at a time and each chunk gets
    its `epochs` passes before the next is drawn (fresh data in bounded
    memory); chunk=0 draws them all first.  The learning rate follows one
    cosine schedule over all steps.

    device_resident (default: when torch sees a GPU): the training set lives
    in device memory, each epoch's shuffle is a device permutation, and a
    step gathers its batch on the device without a host round trip (the loss
    is read back every 200 steps and over the last 50).  Otherwise every step
    copies its batch from host memory.  Returns (surrogate, stats)."""
    rng = np.random.default_rng(seed) if rng is None else rng
    chunk = n_train if chunk <= 0 else min(chunk, n_train)
    n_train -= n_train % batch
    chunk -= chunk % batch
    if n_train <= 0 or chunk <= 0:
        raise ValueError("n_train and chunk must hold at least one batch")
    torch = None
    if device_resident is None or device_resident:
        try:
            import torch
            if not torch.cuda.is_available():
                torch = None
        except ImportError:
            torch = None
        if device_resident and torch is None:
            raise RuntimeError("device_resident training needs torch with a CUDA device")
    nbytes = (ct.n_syndrome + 7) // 8
    sampler = native.Sampler(ct.tanner, ct.lx, ct.lz, ct.em, ct.decoder.device) if gpu_sampler else None
    sur = Surrogate(ct.n_syndrome, ct.n_classes, hidden, n_layers, seed, ct.decoder.device)
    total_steps = epochs * (n_train // batch)
    losses = []
    t_label = t_train = 0.0
    s = 0
    gen = None
    if torch is not None:
        dev = torch.device("cuda", ct.decoder.device)
        gen = torch.Generator(device=dev)
        gen.manual_seed(int(seed) & 0x7FFFFFFFFFFFFFFF)
    try:
        for c0 in range(0, n_train, chunk):
            m = min(chunk, n_train - c0)
            t0 = time.time()
            packed, targets = _draw_labelled(ct, sampler, rng, seed, c0, m, nbytes,
                                             {"f32": native.TQEC_F32, "f64": native.TQEC_F64}[label_precision])
            if torch is not None:
                d_syn = torch.from_numpy(packed).to(dev)
                d_tgt = torch.from_numpy(targets).to(dev)
                del packed, targets
            t1 = time.time()
            t_label += t1 - t0
            nb = m // batch
            for _ in range(epochs):
                if torch is not None:
                    perm = torch.randperm(m, generator=gen, device=dev, dtype=torch.int64).to(torch.int32)
                    stream = torch.cuda.current_stream(dev).cuda_stream
                else:
                    perm = rng.permutation(m)
                for j in range(nb):
                    cur_lr = lr * 0.5 * (1 + np.cos(np.pi * s / total_steps))
                    want = s % 200 == 0 or s >= total_steps - 50
                    if torch is not None:
                        loss = sur.train_step_rows(d_syn.data_ptr(), d_tgt.data_ptr(), m,
                                                   perm.data_ptr() + 4 * j * batch, batch, cur_lr,
                                                   with_loss=want, stream=stream)
                    else:
                        idx = perm[j * batch:(j + 1) * batch]
                        loss = sur.train_step(packed[idx], targets[idx], cur_lr)
                    if want:
                        losses.append(loss)
                        if log and s % 200 == 0:
                            log(f"step {s}/{total_steps} loss {loss:.5f}")
                    s += 1
            if torch is not None:
                torch.cuda.synchronize(dev)
            t_train += time.time() - t1
    finally:
        if sampler is not None:
            sampler.close()
    stats = {"label_seconds": t_label, "train_seconds": t_train, "steps": s, "batch": batch,
             "label_precision": label_precision,
             "n_train": n_train, "epochs": epochs, "chunk": chunk, "device_resident": torch is not None,
             "final_loss": float(np.mean(losses[-50:])) if losses else None}
    return sur, stats


def calibrate(sur, ct, n_val=1 << 20, target_mismatch=1e-4, rng=None, seed=2):
    """Smallest confidence threshold whose accepted rows disagree with the
    exact decoder on at most target_mismatch of all rows (measured on n_val
    fresh syndromes).  Returns (threshold, stats)."""
    rng = np.random.default_rng(seed) if rng is None else rng
    bits = sample_bits(ct, n_val, rng)
    packed = pack_syndromes(bits)
    exact = ct.program.decode_packed(packed)
    cls, conf = sur.infer(packed)
    wrong = cls != exact
    order = np.argsort(-conf, kind="stable")
    cum_wrong = np.cumsum(wrong[order])
    allowed = target_mismatch * n_val
    ok = np.flatnonzero(cum_wrong <= allowed)
    k = int(ok[-1]) + 1 if ok.size else 0   # accept the k most confident rows
    thr = float(conf[order[k - 1]]) if k > 0 else 2.0
    # ties at the threshold: accept only rows strictly above when needed
    acc = conf >= thr
    if (wrong & acc).sum() > allowed:
        thr = float(np.nextafter(np.float32(thr), np.float32(2.0)))
        acc = conf >= thr
    stats = {"threshold": thr, "accept_fraction": float(acc.mean()),
             "mismatch_accepted": float((wrong & acc).mean()), "raw_accuracy_vs_exact": float((~wrong).mean()),
             "n_val": n_val}
    sur.threshold = thr
    return thr, stats


class GatedDecoder:
    """Surrogate first, exact contraction for rows below the threshold."""

    def __init__(self, ct, sur, threshold=None):
        self.ct = ct
        self.sur = sur
        self.threshold = sur.threshold if threshold is None else threshold

    def decode_packed(self, packed, classes=None):
        packed = np.ascontiguousarray(packed, dtype=np.uint8)
        n = packed.shape[0]
        if classes is None:
            classes = np.empty(n, dtype=np.int32)
        nf = C.c_int64()
        native.check(_lib().tqec_gated_decode(self.sur.handle, self.ct.program._h, self.threshold, _p(packed), n,
                                              _p(classes), C.byref(nf), None))
        self.last_fallback = nf.value
        return classes

    def decode_ptrs(self, syn_ptr, n, cls_ptr, stream=None, wait=True):
        """Device (or host) buffers.  wait=False with a stream: the call
        returns without a host synchronisation; after synchronising the
        stream, ``fallback_count()`` gives the rows sent to the contraction."""
        nf = C.c_int64()
        sync = wait or not stream
        native.check(_lib().tqec_gated_decode(self.sur.handle, self.ct.program._h, self.threshold,
                                              C.c_void_p(syn_ptr), n, C.c_void_p(cls_ptr),
                                              C.byref(nf) if sync else None,
                                              C.c_void_p(stream) if stream else None))
        if sync:
            self.last_fallback = nf.value
            return nf.value
        return None

    def fallback_count(self):
        """Rows the last decode sent to the exact contraction (synchronise
        the stream of an asynchronous decode first)."""
        nf = C.c_int64()
        native.check(_lib().tqec_gated_last_fallback(self.sur.handle, C.byref(nf)))
        self.last_fallback = nf.value
        return nf.value

    def decode_batch(self, bits):
        return self.decode_packed(pack_syndromes(bits))
