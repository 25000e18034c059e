"""ctypes binding of ``libtqec_gb300.so`` (declared in include/tqec_gb300.h).

The library is the product: when it is missing the package raises instead
of falling back to any other implementation.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtqec_gb300.so")

TQEC_OK = 0
TQEC_F64 = 0
TQEC_F32 = 1
TQEC_F32X2 = 2
TQEC_F32_BF16 = 3
TQEC_FLAG_PLAIN = 1
TQEC_FLAG_NORECHECK = 2
TQEC_FLAG_MAP = 4
TQEC_FLAG_SPLIT_ARENA = 8
TQEC_FLAG_NO_TENSOR_CORES = 16
TQEC_FLAG_RECHECK_F64 = 32
TQEC_FLAG_SHARED_ITEMS = 64

ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "out of device memory",
          -4: "unsupported network", -5: "timeout", -6: "I/O error"}


class TqecError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Network(C.Structure):
    _fields_ = [("n_tensors", C.c_int32), ("ix_offsets", C.c_void_p), ("ix_labels", C.c_void_p),
                ("data_offsets", C.c_void_p), ("data", C.c_void_p), ("n_out", C.c_int32),
                ("out_labels", C.c_void_p), ("n_syndrome", C.c_int32), ("syndrome_tensors", C.c_void_p)]


class Tree(C.Structure):
    _fields_ = [("n_steps", C.c_int32), ("steps", C.c_void_p)]


class Options(C.Structure):
    _fields_ = [("precision", C.c_int32), ("flags", C.c_uint32), ("device", C.c_int32),
                ("group", C.c_int32), ("threads", C.c_int32), ("margin", C.c_double),
                ("big_elems", C.c_int32), ("reserved", C.c_int32)]


class ProgramInfo(C.Structure):
    _fields_ = [("n_syndrome", C.c_int32), ("syndrome_bytes", C.c_int32), ("n_classes", C.c_int32),
                ("n_steps", C.c_int32), ("n_tree_steps", C.c_int32), ("width", C.c_int32),
                ("arena_elems", C.c_int64), ("flops_per_syndrome", C.c_double), ("flops_tree", C.c_double),
                ("err_bound_f32", C.c_double), ("err_bound_f64", C.c_double),
                ("group_f32", C.c_int32), ("threads_f32", C.c_int32), ("smem_f32", C.c_int32),
                ("group_f64", C.c_int32), ("threads_f64", C.c_int32), ("smem_f64", C.c_int32),
                ("resident_f32", C.c_int32), ("resident_f64", C.c_int32), ("tables_smem_f32", C.c_int32),
                ("tables_smem_f64", C.c_int32), ("arena_small", C.c_int64), ("split_f32", C.c_int32),
                ("split_f64", C.c_int32), ("tensor_steps", C.c_int32), ("tensor_f32", C.c_int32),
                ("recheck_precision", C.c_int32), ("cluster_blocks", C.c_int32), ("err_bound_f32x2", C.c_double),
                ("shared_items_f32", C.c_int32), ("shared_items_f64", C.c_int32),
                ("cluster_tuned_steps", C.c_int32), ("info_pad", C.c_int32)]


class PlanView(C.Structure):
    _fields_ = [("n_steps", C.c_int32), ("steps", C.c_void_p), ("n_perm", C.c_int64),
                ("perm", C.c_void_p), ("n_consts", C.c_int64), ("consts", C.c_void_p),
                ("arena_elems", C.c_int64), ("width", C.c_int32), ("n_classes", C.c_int32),
                ("n_syndrome", C.c_int32), ("flops_per_syndrome", C.c_double), ("flops_tree", C.c_double),
                ("err_terms", C.c_double), ("map_mode", C.c_int32), ("n_vars", C.c_int32),
                ("n_vartab", C.c_int64), ("vartab", C.c_void_p), ("n_report", C.c_int32), ("report", C.c_void_p),
                ("fixed", C.c_void_p)]


class OrderOptions(C.Structure):
    _fields_ = [("trials", C.c_int32), ("sweeps", C.c_int32), ("target_width", C.c_int32),
                ("width_penalty", C.c_double), ("seed", C.c_uint64), ("tensor_discount", C.c_double)]


STEP_DTYPE = np.dtype([("a_kind", "<i4"), ("b_kind", "<i4"), ("a_ref", "<i4"), ("b_ref", "<i4"),
                       ("a_prod", "<i4"), ("b_prod", "<i4"), ("a_sel", "i1", (4,)), ("b_sel", "i1", (4,)),
                       ("lh", "<i4"), ("lfa", "<i4"), ("lfb", "<i4"), ("lk", "<i4"),
                       ("out_off", "<i4"), ("perm_off", "<i4"), ("flags", "<i4"), ("var_off", "<i4")])
assert STEP_DTYPE.itemsize == 64

_lib = None


def lib():
    """Loads the native library (built by build_native.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with build_native.build() "
                          "(the decoder has no non-native implementation)")
    L = C.CDLL(LIB_PATH)
    vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
    sig = {
        "tqec_program_create": [vp, vp, vp, vp],
        "tqec_program_destroy": [vp],
        "tqec_program_info": [vp, vp],
        "tqec_decode_batch": [vp, vp, i64, vp, vp, vp, vp],
        "tqec_contract_batch": [vp, vp, i64, i32, vp, vp],
        "tqec_last_recheck_count": [vp, vp],
        "tqec_program_autotune": [vp, i64],
        "tqec_program_set_cluster": [vp, i32, i32, i32, i32],
        "tqec_program_trim": [vp],
        "tqec_program_save": [vp, C.c_char_p],
        "tqec_program_load": [C.c_char_p, i32, vp],
        "tqec_plan_inspect": [vp, vp, vp, vp],
        "tqec_multi_create": [vp, i32, vp],
        "tqec_multi_destroy": [vp],
        "tqec_multi_set_work": [vp, i32, vp, vp, vp],
        "tqec_multi_reset": [vp, vp],
        "tqec_multi_launch": [vp, vp],
        "tqec_multi_info": [vp, vp, vp, vp],
        "tqec_plan_inspect_flags": [vp, vp, C.c_uint32, vp, vp],
        "tqec_map_decode_batch": [vp, vp, i64, vp, vp, vp],
        "tqec_plan_release": [vp],
        "tqec_optimize_order": [vp, vp, vp, vp, vp],
        "tqec_last_error": [vp, C.c_size_t],
        "tqec_patterns_create": [i32, i32, i32, i32, vp, vp, i32, vp, i32, vp, vp, vp, i32, vp],
        "tqec_patterns_destroy": [vp],
        "tqec_patterns_decode": [vp, vp, vp, i64, vp, vp, vp, vp],
        "tqec_sampler_create": [i32, i32, i32, vp, vp, i32, vp, vp, vp, vp, vp, i32, vp],
        "tqec_sampler_destroy": [vp],
        "tqec_sample": [vp, C.c_uint64, C.c_uint64, i64, vp, vp, vp],
        "tqec_monte_carlo": [vp, vp, vp, C.c_float, C.c_uint64, i64, i64, vp, vp],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_int
    L.tqec_version.restype = C.c_char_p
    L.tqec_version.argtypes = []
    _lib = L
    return L


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    lib().tqec_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def check(code):
    if code != TQEC_OK:
        raise TqecError(code, last_error())
    return code


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class NetworkArrays:
    """Keeps the flattened network arrays alive while the struct is used."""

    def __init__(self, graph):
        (self.ix_off, self.labels, self.d_off, self.data, self.iy,
         self.synd) = graph.flat()
        self.struct = Network(len(graph.ixs), _ptr(self.ix_off), _ptr(self.labels), _ptr(self.d_off),
                              _ptr(self.data), len(self.iy), _ptr(self.iy), len(self.synd), _ptr(self.synd))


def optimize_order(graph, trials=32, sweeps=60, target_width=0, width_penalty=1.0, seed=1, tensor_discount=0.0):
    """Contraction order for a FactorGraph: an (n_tensors - 1, 2) int32 array
    of node ids (tqec_tree convention), log2 of its multiply-adds and its
    width.  tensor_discount > 1 counts the multiply-adds of GEMM-shaped steps
    that many times less."""
    na = NetworkArrays(graph)
    steps = np.zeros((max(graph.n_tensors - 1, 0), 2), dtype=np.int32)
    lm = C.c_double(0)
    w = C.c_int32(0)
    o = OrderOptions(trials, sweeps, target_width, width_penalty, seed, tensor_discount)
    check(lib().tqec_optimize_order(C.byref(na.struct), C.byref(o), _ptr(steps), C.byref(lm), C.byref(w)))
    return steps, lm.value, w.value


def inspect_plan(graph, steps, flags=0):
    """The compiled program as numpy arrays (no GPU needed)."""
    na = NetworkArrays(graph)
    steps = np.ascontiguousarray(steps, dtype=np.int32)
    tree = Tree(steps.shape[0], _ptr(steps))
    view = PlanView()
    h = C.c_void_p()
    check(lib().tqec_plan_inspect_flags(C.byref(na.struct), C.byref(tree), flags, C.byref(view), C.byref(h)))
    try:
        st = np.frombuffer(C.string_at(view.steps, 64 * view.n_steps), dtype=STEP_DTYPE).copy()
        perm = (np.frombuffer(C.string_at(view.perm, 4 * view.n_perm), dtype=np.int32).copy()
                if view.n_perm else np.zeros(0, np.int32))
        consts = (np.frombuffer(C.string_at(view.consts, 8 * view.n_consts), dtype=np.float64).copy()
                  if view.n_consts else np.zeros(0))
        out = {"steps": st, "perm": perm, "consts": consts, "arena_elems": view.arena_elems,
               "width": view.width, "n_classes": view.n_classes, "n_syndrome": view.n_syndrome,
               "flops_per_syndrome": view.flops_per_syndrome, "flops_tree": view.flops_tree,
               "err_terms": view.err_terms, "map_mode": bool(view.map_mode)}
        if view.map_mode:
            out["n_vars"] = view.n_vars
            out["vartab"] = np.frombuffer(C.string_at(view.vartab, 4 * view.n_vartab), dtype=np.int32).copy()
            out["report"] = np.frombuffer(C.string_at(view.report, 4 * view.n_report), dtype=np.int32).copy()
            out["fixed"] = np.frombuffer(C.string_at(view.fixed, view.n_vars), dtype=np.int8).copy()
        return out
    finally:
        lib().tqec_plan_release(h)


class Program:
    """Owner of a ``tqec_program`` (a compiled network on one GPU)."""

    def __init__(self, graph, steps, precision=TQEC_F32, flags=0, device=0, group=0, threads=0, margin=-1.0,
                 big_elems=0):
        L = lib()
        na = NetworkArrays(graph)
        steps = np.ascontiguousarray(steps, dtype=np.int32)
        tree = Tree(steps.shape[0], _ptr(steps))
        opts = Options(precision, flags, device, group, threads, margin, big_elems, 0)
        h = C.c_void_p()
        check(L.tqec_program_create(C.byref(na.struct), C.byref(tree), C.byref(opts), C.byref(h)))
        self._h = h
        self.precision = precision
        self.flags = flags
        info = ProgramInfo()
        check(L.tqec_program_info(self._h, C.byref(info)))
        self.info = {f: getattr(info, f) for f, _ in ProgramInfo._fields_}

    def close(self):
        if getattr(self, "_h", None):
            lib().tqec_program_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_classes(self):
        return self.info["n_classes"]

    @property
    def syndrome_bytes(self):
        return self.info["syndrome_bytes"]

    def decode_packed(self, packed, classes=None, logp=None, err=None, stream=None):
        """Host numpy arrays in and out (copies inside the call)."""
        packed = np.ascontiguousarray(packed, dtype=np.uint8)
        n = packed.shape[0]
        if classes is None:
            classes = np.empty(n, dtype=np.int32)
        check(lib().tqec_decode_batch(self._h, _ptr(packed), n, _ptr(classes), _ptr(logp), _ptr(err), stream))
        return classes

    def decode_ptrs(self, syn_ptr, n, cls_ptr, logp_ptr=None, err_ptr=None, stream=None):
        """Raw (device or host) pointers, e.g. from torch tensors."""
        check(lib().tqec_decode_batch(self._h, C.c_void_p(syn_ptr), n, C.c_void_p(cls_ptr),
                                      C.c_void_p(logp_ptr) if logp_ptr else None,
                                      C.c_void_p(err_ptr) if err_ptr else None,
                                      C.c_void_p(stream) if stream else None))

    def contract_packed(self, packed, precision, logp=None):
        packed = np.ascontiguousarray(packed, dtype=np.uint8)
        n = packed.shape[0]
        if logp is None:
            logp = np.empty((n, self.n_classes), dtype=np.float64)
        check(lib().tqec_contract_batch(self._h, _ptr(packed), n, precision, _ptr(logp), None))
        return logp

    def contract_ptrs(self, syn_ptr, n, precision, logp_ptr, stream=None):
        check(lib().tqec_contract_batch(self._h, C.c_void_p(syn_ptr), n, precision, C.c_void_p(logp_ptr),
                                        C.c_void_p(stream) if stream else None))

    def map_decode_packed(self, packed, n_report):
        """TQEC_FLAG_MAP programs: (values of the reported variables as an
        (n, n_report) 0/1 array, log-probability of the configuration)."""
        packed = np.ascontiguousarray(packed, dtype=np.uint8)
        n = packed.shape[0]
        rb = (n_report + 7) // 8
        asg = np.empty((n, rb), dtype=np.uint8)
        logp = np.empty(n, dtype=np.float64)
        check(lib().tqec_map_decode_batch(self._h, _ptr(packed), n, _ptr(asg), _ptr(logp), None))
        return np.unpackbits(asg, axis=1, count=n_report, bitorder="little"), logp

    def last_recheck_count(self):
        c = C.c_int64(0)
        check(lib().tqec_last_recheck_count(self._h, C.byref(c)))
        return c.value

    def set_cluster(self, precision, blocks, threads=512, small_in_smem=-1):
        """Single-syndrome launches of `precision` on clusters of `blocks`
        blocks (0: one block per syndrome); small_in_smem 1 / 0 / -1: the
        small intermediates in the first block's shared memory / all in
        global memory / the first where it fits."""
        check(lib().tqec_program_set_cluster(self._h, precision, blocks, threads, small_in_smem))
        self._refresh_info()

    def trim(self):
        """Frees the cached intermediate arenas (allocated again on use)."""
        check(lib().tqec_program_trim(self._h))

    def autotune(self, n_probe=4096):
        check(lib().tqec_program_autotune(self._h, n_probe))
        self._refresh_info()

    def _refresh_info(self):
        info = ProgramInfo()
        check(lib().tqec_program_info(self._h, C.byref(info)))
        self.info = {f: getattr(info, f) for f, _ in ProgramInfo._fields_}

    def save(self, path):
        """Writes the network, tree, options and launch shapes to `path`."""
        check(lib().tqec_program_save(self._h, os.fsencode(path)))

    @classmethod
    def load(cls, path, device=-1):
        """A program compiled again from a file of ``save`` on `device`
        (-1: the device it was saved from), with the saved launch shapes when
        the device matches."""
        h = C.c_void_p()
        check(lib().tqec_program_load(os.fsencode(path), device, C.byref(h)))
        self = cls.__new__(cls)
        self._h = h
        self._refresh_info()
        # the options follow the 16-byte file header (magic, version, byte-order mark)
        with open(path, "rb") as f:
            f.seek(16)
            self.precision, self.flags = (int(v) for v in np.frombuffer(f.read(8), dtype="<i4"))
        return self


class PatternDecoder:
    """Owner of a ``tqec_patterns`` (batched error_pattern for a CSS code)."""

    def __init__(self, tanner, lx, lz, device=0):
        from . import gf2

        rx, cx = gf2.right_inverse(tanner.stgx.H)
        rz, cz = gf2.right_inverse(tanner.stgz.H)
        self._keep = [np.ascontiguousarray(a, dtype=np.uint8) for a in (rx, rz, cx, cz, lx, lz)]
        rx, rz, cx, cz, lxa, lza = self._keep
        self.nq = tanner.nq
        h = C.c_void_p()
        check(lib().tqec_patterns_create(tanner.nq, tanner.stgx.ns, tanner.stgz.ns, lx.shape[0], _ptr(rx),
                                         _ptr(rz), cx.shape[0], _ptr(cx) if cx.size else None, cz.shape[0],
                                         _ptr(cz) if cz.size else None, _ptr(lxa), _ptr(lza), device,
                                         C.byref(h)))
        self._h = h

    def decode(self, packed, classes):
        packed = np.ascontiguousarray(packed, dtype=np.uint8)
        classes = np.ascontiguousarray(classes, dtype=np.int32)
        n = packed.shape[0]
        qb = (self.nq + 7) // 8
        ex = np.empty((n, qb), dtype=np.uint8)
        ez = np.empty((n, qb), dtype=np.uint8)
        ok = np.empty(n, dtype=np.uint8)
        check(lib().tqec_patterns_decode(self._h, _ptr(packed), _ptr(classes), n, _ptr(ex), _ptr(ez), _ptr(ok),
                                         None))
        unpack = lambda a: np.unpackbits(a, axis=1, count=self.nq, bitorder="little")  # noqa: E731
        return unpack(ex), unpack(ez), ok

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                lib().tqec_patterns_destroy(self._h)
                self._h = None
        except Exception:
            pass


class Sampler:
    """Owner of a ``tqec_sampler``: seeded code-capacity sampling on the GPU
    and the Monte-Carlo logical-error count."""

    def __init__(self, tanner, lx, lz, em, device=0):
        arrs = [np.ascontiguousarray(a, dtype=np.uint8) for a in (tanner.stgx.H, tanner.stgz.H, lx, lz)]
        ps = [np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), (tanner.nq,)))
              for v in (em.px, em.py, em.pz)]
        self._keep = arrs + ps
        hx, hz, lxa, lza = arrs
        self.ns = tanner.ns
        self.syn_bytes = (tanner.ns + 7) // 8
        h = C.c_void_p()
        check(lib().tqec_sampler_create(tanner.nq, tanner.stgx.ns, tanner.stgz.ns, _ptr(hx), _ptr(hz), lx.shape[0],
                                        _ptr(lxa), _ptr(lza), _ptr(ps[0]), _ptr(ps[1]), _ptr(ps[2]), device,
                                        C.byref(h)))
        self._h = h

    def sample(self, seed, n, offset=0):
        """(packed syndromes (n, syn_bytes), true classes (n,))."""
        syn = np.empty((n, self.syn_bytes), dtype=np.uint8)
        cls = np.empty(n, dtype=np.int32)
        check(lib().tqec_sample(self._h, seed, offset, n, _ptr(syn), _ptr(cls), None))
        return syn, cls

    def monte_carlo(self, program, seed, n_total, batch=1 << 16, mlp=None, threshold=0.0):
        """(logical errors, fallback rows) over n_total sampled syndromes."""
        ne = C.c_int64()
        nf = C.c_int64()
        check(lib().tqec_monte_carlo(self._h, program._h, mlp, threshold, seed, n_total, batch, C.byref(ne),
                                     C.byref(nf)))
        return ne.value, nf.value

    def close(self):
        if getattr(self, "_h", None):
            lib().tqec_sampler_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MultiDecoder:
    """Owner of a ``tqec_multi``: several programs decoded by one persistent
    launch per batch (float32 + double-float or float64 recheck), capturable
    in a CUDA graph.

    ``set_work(batch_end_rows, syn_ptrs, cls_ptrs)``: batch_end_rows is an
    (n_batches, n_programs) array of cumulative end rows; the pointers are
    device buffers of each program's packed syndromes and int32 classes."""

    def __init__(self, programs):
        self.programs = list(programs)
        arr = (C.c_void_p * len(self.programs))(*[p._h for p in self.programs])
        h = C.c_void_p()
        check(lib().tqec_multi_create(arr, len(self.programs), C.byref(h)))
        self._h = h

    def set_work(self, batch_end_rows, syn_ptrs, cls_ptrs):
        rows = np.ascontiguousarray(batch_end_rows, dtype=np.int64)
        n = len(self.programs)
        assert rows.ndim == 2 and rows.shape[1] == n
        syn = (C.c_void_p * n)(*syn_ptrs)
        cls = (C.c_void_p * n)(*cls_ptrs)
        check(lib().tqec_multi_set_work(self._h, rows.shape[0], _ptr(rows), syn, cls))

    def reset(self, stream=None):
        check(lib().tqec_multi_reset(self._h, C.c_void_p(stream) if stream else None))

    def launch(self, stream=None):
        check(lib().tqec_multi_launch(self._h, C.c_void_p(stream) if stream else None))

    def info(self):
        n = len(self.programs)
        g = np.zeros(n, dtype=np.int32)
        sm = np.zeros(n, dtype=np.int32)
        grid = C.c_int32()
        check(lib().tqec_multi_info(self._h, _ptr(g), _ptr(sm), C.byref(grid)))
        return {"groups": g.tolist(), "arena_in_smem": sm.tolist(), "grid": grid.value}

    def close(self):
        if getattr(self, "_h", None):
            lib().tqec_multi_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
