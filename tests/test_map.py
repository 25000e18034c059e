"""TNMAP (most probable configuration) against enumeration.

The reference's TNMAP (src/decoding/tndecoder.jl:9-57) returns a maximiser
of the product of the prior tensors over all error configurations that
reproduce the syndrome.  The CPU tests run the compiled max-product program
(planner output: steps, tables, variable tables) through the numpy emulator
and its back-tracking; the GPU tests run the CUDA kernel.  Both are checked
against the oracle's enumeration (oracle/tnmmap_oracle.py), the known answer
of test/decoding/tndecoder.jl:68-87 (px = 0.26 on qubits 2 and 3 makes
TNMAP decode X1 into a logical error) and the correlated-prior problem of
test/decoding/general_decoding.jl:30-46 (restated on the d=3 surface code).
"""
import numpy as np
import pytest

from conftest import gpu_available
from plan_emulator import map_backtrack, run_plan

gpu = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]


def _general(pkg, d=3, em=None):
    from tensorqec_gb300 import network
    t = pkg.tanner_graph(pkg.SurfaceCode(d, d))
    if em is None:
        em = pkg.iid_error(0.05, 0.06, 0.1, t.nq)
    general, ixs, ts = network.reduce2general(t, em)
    return t, general, ixs, ts


def _syndromes(pkg, t, em, n, seed):
    rng = np.random.default_rng(seed)
    ep = pkg.random_error_pattern(em, rng, nsamples=n)
    syn = pkg.syndrome_extraction(ep, t)
    return np.concatenate([syn.sx, syn.sz], axis=1).astype(np.uint8), ep


def _check_optimal(oracle, general, ixs, ts, bits, cfg, logp=None, rtol=1e-12):
    ref = oracle.most_probable_configs(general.H, ixs, ts, bits)
    got = oracle.config_log_probability(ixs, ts, cfg)
    for r in range(bits.shape[0]):
        best = ref[r][0]
        np.testing.assert_array_equal((cfg[r].astype(np.int64) @ general.H.T.astype(np.int64)) % 2, bits[r])
        assert abs(got[r] - best) <= rtol * abs(best) + 1e-12, (r, got[r], best)
        if logp is not None:
            assert abs(logp[r] - best) <= max(rtol, 1e-12) * abs(best) + 1e-9, (r, logp[r], best)


def _map_plan(pkg, general, ixs, ts):
    from tensorqec_gb300 import decoder, native, network
    graph = network.tnmap_graph(general, ixs, ts)
    steps = decoder.optimize_code(graph, decoder.TreeSA(restarts=1))
    return native.inspect_plan(graph, steps, native.TQEC_FLAG_MAP)


def test_map_plan_emulated_matches_enumeration(pkg, oracle):
    em = pkg.iid_error(0.05, 0.06, 0.1, 9)
    t, general, ixs, ts = _general(pkg, 3, em)
    plan = _map_plan(pkg, general, ixs, ts)
    assert plan["map_mode"] and plan["n_classes"] == 1
    bits, _ = _syndromes(pkg, t, em, 40, 3)
    val, arena = run_plan(plan, bits, return_arena=True)
    cfg = map_backtrack(plan, bits, arena)
    _check_optimal(oracle, general, ixs, ts, bits, cfg, np.log(val[:, 0]), rtol=1e-12)


def test_map_plan_emulated_reference_kat(pkg, oracle):
    """tndecoder.jl:68-87: X1 on the d=3 surface code; with px = 0.26 on
    qubits 2 and 3 the most probable error is X2 X3, a logical error."""
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    lx, lz = pkg.logical_operator(t)
    ex = np.zeros(9, np.uint8)
    ex[0] = 1
    sz = (t.stgz.H.astype(np.int64) @ ex) % 2
    bits = np.concatenate([np.zeros(t.stgx.ns, np.uint8), sz.astype(np.uint8)])[None, :]
    for heavy, logical in ((False, False), (True, True)):
        px = np.full(9, 0.1)
        if heavy:
            px[1] = px[2] = 0.26
        em = pkg.IndependentDepolarizingError(px, np.zeros(9), np.zeros(9))
        _, general, ixs, ts = _general(pkg, 3, em)
        plan = _map_plan(pkg, general, ixs, ts)
        val, arena = run_plan(plan, bits, return_arena=True)
        cfg = map_backtrack(plan, bits, arena)[0]
        e1 = pkg.CSSErrorPattern(cfg[:9], cfg[9:])
        e0 = pkg.CSSErrorPattern(ex, np.zeros(9, np.uint8))
        assert pkg.check_logical_error(e1, e0, lx, lz) == logical


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")
def test_gpu_map_matches_enumeration(pkg, oracle, precision):
    em = pkg.iid_error(0.05, 0.06, 0.1, 9)
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    ct = pkg.compile(pkg.TNMAP(precision=precision), t, em)
    bits, _ = _syndromes(pkg, t, em, 300, 11)
    (ex, ez), logp = ct.decode_batch(bits, return_logp=True)
    cfg = np.concatenate([ex, ez], axis=1)
    _, general, ixs, ts = _general(pkg, 3, em)
    _check_optimal(oracle, general, ixs, ts, bits, cfg, logp, rtol=1e-12 if precision == "f64" else 2e-5)
    # one-at-a-time decode agrees with the batch
    res = ct.decode(pkg.CSSSyndrome(bits[0, :t.stgx.ns], bits[0, t.stgx.ns:]))
    assert np.array_equal(res.error_pattern.xerror, ex[0]) and np.array_equal(res.error_pattern.zerror, ez[0])
    ct.close()


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")
def test_gpu_map_reference_kat(pkg):
    """tndecoder.jl:68-87 on the GPU."""
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    lx, lz = pkg.logical_operator(t)
    ex = np.zeros(9, np.uint8)
    ex[0] = 1
    sz = ((t.stgz.H.astype(np.int64) @ ex) % 2).astype(np.uint8)
    syn = pkg.CSSSyndrome(np.zeros(t.stgx.ns, np.uint8), sz)
    for heavy in (False, True):
        px = np.full(9, 0.1)
        if heavy:
            px[1] = px[2] = 0.26
        ct = pkg.compile(pkg.TNMAP(), t, pkg.IndependentDepolarizingError(px, np.zeros(9), np.zeros(9)))
        res = ct.decode(syn)
        assert res.success_tag
        ep = res.error_pattern
        assert pkg.syndrome_extraction(ep, t) == syn
        assert pkg.check_logical_error(ep, pkg.CSSErrorPattern(ex, np.zeros(9, np.uint8)), lx, lz) == heavy
        ct.close()


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")
def test_gpu_map_classical_and_correlated(pkg, oracle):
    """compile(TNMAP(), tanner.stgz) (tndecoder.jl:31-43, interfaces.jl:4-14)
    and a general problem with a correlated rank-4 prior
    (general_decoding.jl:30-46: qubits 4 and 7 share one tensor that allows
    only I on both or Y on qubit 7)."""
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    stgz = t.stgz
    ct = pkg.compile(pkg.TNMAP(), stgz, pkg.iid_error(0.05, 9))
    rng = np.random.default_rng(123)
    e = (rng.random((200, 9)) < 0.05).astype(np.uint8)
    s = ((e.astype(np.int64) @ stgz.H.T.astype(np.int64)) % 2).astype(np.uint8)
    cfg, logp = ct.decode_batch(s, return_logp=True)
    ixs = [[i + 1] for i in range(9)]
    ts = [np.array([0.95, 0.05])] * 9
    _check_optimal(oracle, stgz, ixs, ts, s, cfg, logp)
    r = ct.decode(pkg.SimpleSyndrome(s[0]))
    assert np.array_equal((stgz.H.astype(np.int64) @ r.error_pattern) % 2, s[0])
    ct.close()

    nq = 9
    a = np.zeros((2, 2, 2, 2))
    a[0, 0, 0, 0] = 0.99
    a[0, 0, 1, 1] = 0.01
    single = np.array([1 - 0.05 - 0.03 - 0.01, 0.05, 0.01, 0.03])  # [1-p, px, pz, py]
    ixs = [[i, i + nq] for i in (1, 2, 3, 5, 6, 8, 9)] + [[4, 4 + nq, 7, 7 + nq]]
    ts = [single] * 7 + [a]
    ct = pkg.compile(pkg.TNMAP(), t, (ixs, ts))
    em = pkg.iid_error(0.05, 0.03, 0.01, nq)
    bits, _ = _syndromes(pkg, t, em, 100, 9)
    (ex, ez), logp = ct.decode_batch(bits, return_logp=True)
    from tensorqec_gb300 import network
    general, gixs, gts = network.reduce2general(t, (ixs, ts))
    cfg = np.concatenate([ex, ez], axis=1)
    ok = np.isfinite(logp)
    ref = oracle.most_probable_configs(general.H, gixs, gts, bits)
    for r in range(bits.shape[0]):
        if not np.isfinite(ref[r][0]):
            assert not ok[r]
            continue
        _check_optimal(oracle, general, gixs, gts, bits[r:r + 1], cfg[r:r + 1], logp[r:r + 1])
        assert cfg[r, 3] == 0 and cfg[r, 3 + nq] == 0 and cfg[r, 6] == cfg[r, 6 + nq]
    ct.close()


@pytest.mark.gpu
@pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")
def test_gpu_map_d5_self_consistent(pkg, oracle):
    """d=5: beyond enumeration, so the decoded configuration must reproduce
    the syndrome, carry exactly the reported maximum, and f32 must find the
    same maximum as f64."""
    t = pkg.tanner_graph(pkg.SurfaceCode(5, 5))
    em = pkg.depolarizing(0.08, t.nq)
    bits, _ = _syndromes(pkg, t, em, 2000, 21)
    c64 = pkg.compile(pkg.TNMAP(precision="f64"), t, em)
    c32 = pkg.compile(pkg.TNMAP(precision="f32"), t, em)
    (ex, ez), lp64 = c64.decode_batch(bits, return_logp=True)
    (fx, fz), lp32 = c32.decode_batch(bits, return_logp=True)
    from tensorqec_gb300 import network
    general, ixs, ts = network.reduce2general(t, em)
    H = general.H.astype(np.int64)
    for cx, cz, lp, tol in ((ex, ez, lp64, 1e-12), (fx, fz, lp32, 2e-5)):
        cfg = np.concatenate([cx, cz], axis=1).astype(np.int64)
        np.testing.assert_array_equal((cfg @ H.T) % 2, bits)
        own = oracle.config_log_probability(ixs, ts, cfg)
        np.testing.assert_allclose(own, lp64, rtol=tol)
        np.testing.assert_allclose(lp, lp64, rtol=tol)
    c64.close()
    c32.close()
