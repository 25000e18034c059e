"""tqec_decode_batch_noalloc: the float64 batch decode that allocates no
device memory, for callers that cannot allocate while they decode (a
real-time decoding loop that must not stall or fail on an allocation, or a
process whose device memory another allocator already holds in full).

Called through the C ABI with device buffers and checked against the
existing entry point on two calls in a row.  Tolerance: classes identical,
float64 log-marginals within 1e-10 relative (the same kernel arithmetic).
This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]


def _entry(pkg):
    f = pkg.native.lib().tqec_decode_batch_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def _syndromes(pkg, t, em, n, seed):
    rng = np.random.default_rng(seed)
    ep = pkg.random_error_pattern(em, rng, nsamples=n)
    s = pkg.syndrome_extraction(ep, t)
    return np.concatenate([s.sx, s.sz], axis=1)


@pytest.mark.parametrize("d,precision", [(5, "f64"), (7, "f32")])
def test_noalloc_matches_decode_batch_twice(pkg, d, precision):
    torch = pytest.importorskip("torch")
    noalloc = _entry(pkg)
    t = pkg.tanner_graph(pkg.SurfaceCode(d, d))
    em = pkg.depolarizing(0.08, t.nq)
    ct = pkg.compile(pkg.TNMMAP(precision=precision), t, em)
    nc = ct.n_classes
    for call, seed in enumerate((11, 12)):
        n = 3000 if d == 5 else 700
        bits = _syndromes(pkg, t, em, n, seed)
        packed = pkg.pack_syndromes(bits)
        want_lp = ct.class_logprobs(bits, precision="f64")
        want_cls = ct.program.decode_packed(packed) if precision == "f64" else np.argmax(want_lp, axis=1)
        d_syn = torch.from_numpy(packed).cuda()
        d_cls = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        d_lp = torch.full((n, nc), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = noalloc(ct.program._h, C.c_void_p(d_syn.data_ptr()), n, C.c_void_p(d_cls.data_ptr()),
                     C.c_void_p(d_lp.data_ptr()), None)
        assert rc == 0, pkg.native.last_error()
        got_cls = d_cls.cpu().numpy()
        got_lp = d_lp.cpu().numpy()
        np.testing.assert_array_equal(got_cls, want_cls, err_msg=f"call {call}")
        scale = np.exp(want_lp.max(axis=1, keepdims=True))
        err = np.abs(np.exp(got_lp) - np.exp(want_lp)) / scale
        assert err.max() <= 1e-10, f"call {call}: {err.max():.3e}"
    ct.close()


def test_noalloc_rejects_host_pointers_and_oversized_programs(pkg):
    torch = pytest.importorskip("torch")
    noalloc = _entry(pkg)
    t = pkg.tanner_graph(pkg.SurfaceCode(5, 5))
    ct = pkg.compile(pkg.TNMMAP(precision="f64"), t, pkg.depolarizing(0.05, t.nq))
    packed = pkg.pack_syndromes(np.zeros((4, t.ns), np.uint8))
    cls = np.zeros(4, np.int32)
    rc = noalloc(ct.program._h, packed.ctypes.data_as(C.c_void_p), 4, cls.ctypes.data_as(C.c_void_p), None, None)
    assert rc == pkg.native.TqecError(-1, "").code
    assert "device pointers" in pkg.native.last_error()
    ct.close()
    # a most-probable-configuration (TNMAP) program is refused before any launch
    mp = pkg.compile(pkg.TNMAP(), t, pkg.depolarizing(0.05, t.nq))
    d_syn = torch.zeros((4, mp.program.syndrome_bytes), dtype=torch.uint8, device="cuda")
    d_cls = torch.zeros(4, dtype=torch.int32, device="cuda")
    rc = noalloc(mp.program._h, C.c_void_p(d_syn.data_ptr()), 4, C.c_void_p(d_cls.data_ptr()), None, None)
    assert rc == -1
    assert "tqec_map_decode_batch" in pkg.native.last_error()
    mp.close()
    # toric 5x5: a float64 working set far above the 32 MiB scratch
    tb = pkg.tanner_graph(pkg.ToricCode(5, 5))
    big = pkg.compile(pkg.TNMMAP(precision="f64", optimizer=pkg.TreeSA(restarts=1, sweeps=300)), tb,
                      pkg.depolarizing(0.05, tb.nq))
    assert big.program.info["arena_elems"] * 8 > (32 << 20)
    d_syn = torch.zeros((4, big.program.syndrome_bytes), dtype=torch.uint8, device="cuda")
    d_cls = torch.zeros(4, dtype=torch.int32, device="cuda")
    rc = noalloc(big.program._h, C.c_void_p(d_syn.data_ptr()), 4, C.c_void_p(d_cls.data_ptr()), None, None)
    assert rc == -4
    assert "exceeds the 33554432-byte scratch" in pkg.native.last_error()
    big.close()
