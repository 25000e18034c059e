"""Error models, syndromes and decoding results
(TensorQEC's src/decoding/error_model.jl and interfaces.jl).

Sampling uses numpy's PCG64 stream (``random_error_pattern``) or the GPU
Philox sampler of the native library; neither reproduces Julia's RNG, so a
seed here names a different sample than the same seed in Julia.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class IndependentFlipError:
    """error_model.jl:13-15: bit i flips with probability p[i]."""
    p: np.ndarray

    def __post_init__(self):
        self.p = np.asarray(self.p, dtype=np.float64)


@dataclass
class IndependentDepolarizingError:
    """error_model.jl:41-45: per-qubit X, Y, Z probabilities."""
    px: np.ndarray
    py: np.ndarray
    pz: np.ndarray

    def __post_init__(self):
        self.px = np.asarray(self.px, dtype=np.float64)
        self.py = np.asarray(self.py, dtype=np.float64)
        self.pz = np.asarray(self.pz, dtype=np.float64)


def iid_error(*args):
    """iid_error(p, n) -> IndependentFlipError (error_model.jl:28);
    iid_error(px, py, pz, n) -> IndependentDepolarizingError (:61);
    iid_error(p, tanner::CSSTannerGraph) -> depolarizing with px=py=pz=p
    (:62, note: each Pauli gets p, as in the reference)."""
    if len(args) == 2:
        p, n = args
        if hasattr(n, "stgx"):
            return iid_error(p, p, p, n.nq)
        if hasattr(n, "s2q"):
            n = n.nq
        return IndependentFlipError(np.full(n, float(p)))
    px, py, pz, n = args
    return IndependentDepolarizingError(np.full(n, float(px)), np.full(n, float(py)), np.full(n, float(pz)))


def depolarizing(p: float, n: int) -> IndependentDepolarizingError:
    """Code-capacity depolarising noise of total rate p (X, Y, Z each p/3)."""
    return iid_error(p / 3, p / 3, p / 3, n)


@dataclass
class CSSErrorPattern:
    """error_model.jl:81-84 (uint8 0/1 vectors)."""
    xerror: np.ndarray
    zerror: np.ndarray


@dataclass
class SimpleSyndrome:
    s: np.ndarray


@dataclass
class CSSSyndrome:
    """error_model.jl:138-141: sx = X-check bits, sz = Z-check bits."""
    sx: np.ndarray
    sz: np.ndarray

    def bits(self) -> np.ndarray:
        """[sx..., sz...] (the update_syndrome! order, tndecoder.jl:148-158);
        a batch of syndromes (2-D sx, sz) gives one row per syndrome."""
        return np.concatenate([np.asarray(self.sx, np.uint8), np.asarray(self.sz, np.uint8)], axis=-1) & 1

    def __eq__(self, other):
        return (np.array_equal(np.asarray(self.sx) & 1, np.asarray(other.sx) & 1)
                and np.array_equal(np.asarray(self.sz) & 1, np.asarray(other.sz) & 1))


@dataclass
class DecodingResult:
    """interfaces.jl:116-119."""
    success_tag: bool
    error_pattern: object


def random_error_pattern(em, rng=None, nsamples=None):
    """error_model.jl:69-71 and :97-117.  One uniform per qubit: Y if
    r < py, X if r < px + py, Z if r < px + py + pz.  With ``nsamples`` the
    result is batched: arrays of shape (nsamples, n)."""
    rng = np.random.default_rng() if rng is None else rng
    if isinstance(em, IndependentFlipError):
        shape = (em.p.size,) if nsamples is None else (nsamples, em.p.size)
        return (rng.random(shape) < em.p).astype(np.uint8)
    n = em.px.size
    shape = (n,) if nsamples is None else (nsamples, n)
    r = rng.random(shape)
    y = r < em.py
    x = ~y & (r < em.px + em.py)
    z = ~y & ~x & (r < em.px + em.py + em.pz)
    ex = (x | y).astype(np.uint8)
    ez = (z | y).astype(np.uint8)
    return CSSErrorPattern(ex, ez)


def syndrome_extraction(error, tanner):
    """error_model.jl:131-146.  For a CSS graph: sx = Hx ez, sz = Hz ex.
    Batched inputs (2-D error arrays) give 2-D syndrome arrays."""
    if isinstance(error, CSSErrorPattern):
        ez = np.asarray(error.zerror).astype(np.int64)
        ex = np.asarray(error.xerror).astype(np.int64)
        sx = (ez @ tanner.stgx.H.T.astype(np.int64)) % 2
        sz = (ex @ tanner.stgz.H.T.astype(np.int64)) % 2
        return CSSSyndrome(sx.astype(np.uint8), sz.astype(np.uint8))
    H = tanner.H if hasattr(tanner, "H") else tanner
    e = np.asarray(error).astype(np.int64)
    return SimpleSyndrome(((e @ np.asarray(H).T.astype(np.int64)) % 2).astype(np.uint8))


def check_logical_error(e1, e2, lx, lz=None):
    """error_model.jl:161-181.  For CSS patterns: a logical error when
    lx.(ez1 - ez2) or lz.(ex1 - ex2) is odd.  Accepts batched patterns and
    then returns a bool array."""
    if isinstance(e1, CSSErrorPattern):
        dz = (np.asarray(e1.zerror).astype(np.int64) + np.asarray(e2.zerror)) % 2
        dx = (np.asarray(e1.xerror).astype(np.int64) + np.asarray(e2.xerror)) % 2
        a = (dz @ np.asarray(lx).T.astype(np.int64)) % 2
        b = (dx @ np.asarray(lz).T.astype(np.int64)) % 2
        return np.any(a, axis=-1) | np.any(b, axis=-1)
    d = (np.asarray(e1).astype(np.int64) + np.asarray(e2)) % 2
    return np.any((d @ np.asarray(lx).T.astype(np.int64)) % 2, axis=-1)


def pack_syndromes(bits: np.ndarray) -> np.ndarray:
    """Bit-packs syndrome rows (n, nbits) into (n, ceil(nbits/8)) bytes,
    bit j at byte j//8, bit j%8 (the native library's row format)."""
    bits = np.atleast_2d(np.asarray(bits, dtype=np.uint8) & 1)
    return np.packbits(bits, axis=1, bitorder="little")


def unpack_syndromes(packed: np.ndarray, nbits: int) -> np.ndarray:
    return np.unpackbits(np.atleast_2d(packed), axis=1, count=nbits, bitorder="little")
