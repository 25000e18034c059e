"""ctypes wrapper of the oracle's C contractor (test infrastructure only).

``CContractor(graph, steps)`` evaluates TensorQEC's per-syndrome contraction
(src/decoding/tndecoder.jl:148-165) in float64 along the given tree, with
one-hot syndrome leaves rewritten for every syndrome and nothing folded
across syndromes; rows are spread over OpenMP threads.
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        L.oracle_create.restype = C.c_void_p
        L.oracle_create.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                    C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p]
        L.oracle_contract.restype = C.c_int
        L.oracle_contract.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int]
        L.oracle_destroy.argtypes = [C.c_void_p]
        L.oracle_max_threads.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class CContractor:
    def __init__(self, ixs, tensors, iy, syndrome_positions, steps):
        ix_off = np.zeros(len(ixs) + 1, dtype=np.int32)
        ix_off[1:] = np.cumsum([len(x) for x in ixs])
        labels = np.array([v for x in ixs for v in x], dtype=np.int32)
        d_off = np.zeros(len(tensors) + 1, dtype=np.int64)
        d_off[1:] = np.cumsum([np.asarray(t).size for t in tensors])
        data = np.concatenate([np.asarray(t, dtype=np.float64).ravel(order="F") for t in tensors])
        iy = np.asarray(iy, dtype=np.int32)
        syn = np.asarray(syndrome_positions, dtype=np.int32)
        st = np.ascontiguousarray(steps, dtype=np.int32).reshape(-1)
        self._keep = (ix_off, labels, d_off, data, iy, syn, st)
        self.n_classes = 1 << len(iy)
        self.h = lib().oracle_create(len(ixs), _p(ix_off), _p(labels), _p(d_off), _p(data), len(iy), _p(iy),
                                     len(syn), _p(syn), len(st) // 2, _p(st))
        if not self.h:
            raise ValueError("oracle_create rejected the network/tree")

    def contract(self, packed, threads=0):
        packed = np.ascontiguousarray(packed, dtype=np.uint8)
        n = packed.shape[0]
        marg = np.empty((n, self.n_classes), dtype=np.float64)
        cls = np.empty(n, dtype=np.int32)
        lib().oracle_contract(self.h, _p(packed), n, _p(marg), _p(cls), threads)
        return marg, cls

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_destroy(self.h)
            self.h = None


def max_threads():
    return lib().oracle_max_threads()


def host_cores():
    """Cores this process may run on.  OMP_NUM_THREADS (which torchrun sets
    to 1 for every rank) does not limit it."""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1
