"""GPU parity: the CUDA contraction against the oracle.

Tolerances (tests/parity.py): float64 class log-probabilities within 1e-10
relative, class by class (|logp - log p_ref| <= 1e-10 |log p_ref|, -inf
exactly on the oracle's zero classes); float32 and double-float class
log-probabilities within twice the program's stated rounding bound, class by
class; decisions equal to the oracle's argmax except where the oracle's top
two classes are within 1e-9 relative of each other (a tie that summation
order decides).
"""
import json
import os

import numpy as np
import pytest

from conftest import gpu_available
from parity import assert_class_logprobs, assert_class_logprobs_within

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TIE = 1e-9


def assert_decisions(cls, want_mar):
    want_mar = np.asarray(want_mar)
    best = want_mar.argmax(axis=1)
    srt = np.sort(want_mar, axis=1)
    top, second = srt[:, -1], srt[:, -2]
    tie = (top - second) <= TIE * np.maximum(top, 1e-300)
    bad = (cls != best) & ~tie
    assert not bad.any(), f"{bad.sum()} decision mismatches outside ties, rows {np.flatnonzero(bad)[:10]}"
    # when the classes differ on a tie, the chosen class must be one of the tied maxima
    ok = want_mar[np.arange(len(cls)), cls] >= top * (1 - 1e-9)
    assert ok.all()


def assert_marginals(logp, want_mar, rtol):
    """rtol 1e-10: the float64 per-class bound; a larger rtol is a reduced
    precision's rounding bound, held class by class as a log-space error.
    Either way the error relative to the row's largest class stays within
    rtol too."""
    want_mar = np.asarray(want_mar)
    if rtol <= 1e-10:
        assert_class_logprobs(logp, want_mar, rtol)
    else:
        assert_class_logprobs_within(logp, want_mar, rtol)
    got = np.exp(logp)
    scale = want_mar.max(axis=1, keepdims=True)
    err = np.abs(got - want_mar) / np.maximum(scale, 1e-300)
    assert err.max() <= rtol, f"max relative error {err.max():.3e} > {rtol:.1e}"


def css_case(pkg, oracle, kind, d, p, n, seed):
    code = {"surface": lambda: pkg.SurfaceCode(d, d), "toric": lambda: pkg.ToricCode(d, d),
            "488": lambda: pkg.Color488(d), "666": lambda: pkg.Color666(d)}[kind]()
    t = pkg.tanner_graph(code)
    em = pkg.depolarizing(p, t.nq)
    rng = np.random.default_rng(seed)
    ep = pkg.random_error_pattern(em, rng, nsamples=n)
    syn = pkg.syndrome_extraction(ep, t)
    bits = np.concatenate([syn.sx, syn.sz], axis=1)
    if kind == "surface":
        st, nq = oracle.surface_code_stabilizers(d, d)
    elif kind == "toric":
        st, nq = oracle.toric_code_stabilizers(d, d)
    else:
        st, nq = oracle.color_code_stabilizers(kind, d)
    dec = oracle.OracleDecoder(oracle.css_tanner(st, nq), em.px, em.py, em.pz)
    return t, em, bits, dec


@pytest.fixture(scope="module")
def d3(pkg, oracle):
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    em = pkg.depolarizing(0.05, t.nq)
    st, nq = oracle.surface_code_stabilizers(3, 3)
    ot = oracle.css_tanner(st, nq)
    lx, lz = oracle.logical_operator(ot)
    brute = oracle.brute_force_marginals(ot, em.px, em.py, em.pz, lx, lz)
    bits = ((np.arange(256)[:, None] >> np.arange(8)[None, :]) & 1).astype(np.uint8)
    return t, em, bits, brute


@pytest.mark.parametrize("precision,plain", [("f64", True), ("f64", False), ("f32", False)])
def test_d3_every_syndrome_vs_enumeration(pkg, d3, precision, plain):
    t, em, bits, brute = d3
    ct = pkg.compile(pkg.TNMMAP(precision=precision, plain=plain), t, em)
    cls, logp = ct.decode_batch(bits, return_logp=True)
    assert_decisions(cls, brute)
    if precision == "f64":
        assert_marginals(logp, brute, 1e-10)
    else:
        lp64 = ct.class_logprobs(bits, precision="f64")
        lp32 = ct.class_logprobs(bits, precision="f32")
        assert_marginals(lp64, brute, 1e-10)
        bound = ct.program.info["err_bound_f32"]
        assert_marginals(lp32, brute, 2 * bound)
    ct.close()


def test_zero_syndrome_kat_on_gpu(pkg):
    """test/decoding/tndecoder.jl:101-110 on the device."""
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    ct = pkg.compile(pkg.TNMMAP(precision="f64", plain=True), t, pkg.iid_error(0.1, 0.0, 0.0, 9))
    lp = ct.class_logprobs(np.zeros((1, 8), dtype=np.uint8))
    np.testing.assert_allclose(np.exp(lp[0]), [0.3972875040000002, 0.0, 0.004284496000000001, 0.0],
                               atol=1e-10)
    ct.close()


def test_decision_kat_x1_on_gpu(pkg):
    """tndecoder.jl:60-73: X1 with px=0.1 decodes with no logical error and
    the rebuilt pattern reproduces the syndrome."""
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    em = pkg.iid_error(0.1, 0.0, 0.0, 9)
    ct = pkg.compile(pkg.TNMMAP(precision="f64"), t, em)
    ex = np.array([1, 0, 0, 0, 0, 0, 0, 0, 0], dtype=np.uint8)
    truth = pkg.CSSErrorPattern(ex, np.zeros(9, np.uint8))
    syn = pkg.syndrome_extraction(truth, t)
    res = pkg.decode(ct, syn)
    assert res.success_tag
    assert not pkg.check_logical_error(res.error_pattern, truth, ct.lx, ct.lz)
    assert pkg.syndrome_extraction(res.error_pattern, t) == syn
    ct.close()


@pytest.mark.parametrize("kind,d,p,n", [("surface", 5, 0.08, 400), ("surface", 7, 0.05, 48),
                                        ("toric", 3, 0.05, 128), ("488", 5, 0.05, 128),
                                        ("666", 5, 0.08, 128)])
def test_css_codes_vs_oracle(pkg, oracle, kind, d, p, n):
    t, em, bits, dec = css_case(pkg, oracle, kind, d, p, n, seed=100 + d)
    want = dec.marginals(bits)
    for precision in ("f64", "f32"):
        ct = pkg.compile(pkg.TNMMAP(precision=precision), t, em)
        cls, logp = ct.decode_batch(bits, return_logp=True)
        assert_decisions(cls, want)
        lp = ct.class_logprobs(bits)
        tol = 1e-10 if precision == "f64" else 2 * ct.program.info["err_bound_f32"]
        assert_marginals(lp, want, tol)
        ct.close()


def test_dem_every_syndrome_vs_oracle(pkg, oracle):
    text = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_kat.json")))["dem_small"]["text"]
    dem = pkg.parse_dem_string(text)
    bits = ((np.arange(64)[:, None] >> np.arange(6)[None, :]) & 1).astype(np.uint8)
    want = oracle.OracleDEMDecoder(oracle.parse_dem_string(text)).marginals(bits)
    for precision in ("f64", "f32"):
        ct = pkg.compile(pkg.TNMMAP(precision=precision, factorize=True), dem)
        cls, logp = ct.decode_batch(bits, return_logp=True)
        assert_decisions(cls, want)
        tol = 1e-10 if precision == "f64" else 2 * ct.program.info["err_bound_f32"]
        assert_marginals(ct.class_logprobs(bits), want, tol)
        for r in range(0, 64, 7):
            res = ct.decode(pkg.SimpleSyndrome(bits[r]))
            if res.success_tag:
                s = pkg.syndrome_extraction(res.error_pattern, ct.tanner).s
                assert np.array_equal(s, bits[r])
        ct.close()


def test_f32_recheck_decisions_equal_f64_at_scale(pkg):
    """65,536 d=5 syndromes: float32 + recheck decides exactly like float64
    wherever float64's margin exceeds the float64 bound."""
    t = pkg.tanner_graph(pkg.SurfaceCode(5, 5))
    em = pkg.depolarizing(0.11, t.nq)
    rng = np.random.default_rng(5)
    ep = pkg.random_error_pattern(em, rng, nsamples=65536)
    syn = pkg.syndrome_extraction(ep, t)
    bits = np.concatenate([syn.sx, syn.sz], axis=1)
    ct = pkg.compile(pkg.TNMMAP(precision="f32"), t, em)
    cls32 = ct.decode_batch(bits)
    lp64 = ct.class_logprobs(bits, precision="f64")
    cls64 = np.argmax(lp64, axis=1)
    srt = np.sort(lp64, axis=1)
    tie = (srt[:, -1] - srt[:, -2]) <= 1e-9
    assert not ((cls32 != cls64) & ~tie).any()
    n_re = ct.program.last_recheck_count()
    assert 0 <= n_re < 65536 // 10
    ct.close()


def test_empty_batch_and_device_pointers(pkg):
    torch = pytest.importorskip("torch")
    t = pkg.tanner_graph(pkg.SurfaceCode(5, 5))
    em = pkg.depolarizing(0.05, t.nq)
    ct = pkg.compile(pkg.TNMMAP(precision="f32"), t, em)
    assert ct.decode_batch(np.zeros((0, t.ns), np.uint8)).shape == (0,)
    rng = np.random.default_rng(9)
    ep = pkg.random_error_pattern(em, rng, nsamples=1000)
    syn = pkg.syndrome_extraction(ep, t)
    bits = np.concatenate([syn.sx, syn.sz], axis=1)
    want = ct.decode_batch(bits)
    d_syn = torch.from_numpy(pkg.pack_syndromes(bits)).cuda()
    d_cls = torch.empty(1000, dtype=torch.int32, device="cuda")
    d_lp = torch.empty((1000, 4), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    ct.program.decode_ptrs(d_syn.data_ptr(), 1000, d_cls.data_ptr(), d_lp.data_ptr(), None, stream)
    torch.cuda.synchronize()
    assert np.array_equal(d_cls.cpu().numpy(), want)
    ct.close()


@pytest.mark.parametrize("kind,d", [("surface", 3), ("surface", 7), ("toric", 4), ("666", 5)])
def test_gpu_error_patterns(pkg, oracle, kind, d):
    """error_pattern (tndecoder.jl:167-174) on the GPU: each rebuilt pattern
    reproduces its syndrome and carries the decoded class."""
    code = {"surface": lambda: pkg.SurfaceCode(d, d), "toric": lambda: pkg.ToricCode(d, d),
            "666": lambda: pkg.Color666(d)}[kind]()
    t = pkg.tanner_graph(code)
    em = pkg.depolarizing(0.08, t.nq)
    ct = pkg.compile(pkg.TNMMAP(precision="f32"), t, em)
    rng = np.random.default_rng(31)
    ep = pkg.random_error_pattern(em, rng, nsamples=2000)
    syn = pkg.syndrome_extraction(ep, t)
    bits = np.concatenate([syn.sx, syn.sz], axis=1)
    forced = rng.integers(0, ct.n_classes, size=2000).astype(np.int32)
    for classes in (None, forced):
        cls, ex, ez, ok = ct.decode_patterns(bits, classes)
        assert ok.all()
        assert np.array_equal((ez.astype(np.int64) @ t.stgx.H.T) % 2, syn.sx)
        assert np.array_equal((ex.astype(np.int64) @ t.stgz.H.T) % 2, syn.sz)
        k = ct.lx.shape[0]
        a = (ez.astype(np.int64) @ ct.lx.T) % 2
        b = (ex.astype(np.int64) @ ct.lz.T) % 2
        got = (a * (1 << np.arange(k))).sum(1) + (b * (1 << (k + np.arange(k)))).sum(1)
        assert np.array_equal(got, cls)
    # the single-syndrome decode path agrees with the batched one
    res = ct.decode(pkg.CSSSyndrome(syn.sx[0], syn.sz[0]))
    assert res.success_tag and pkg.syndrome_extraction(res.error_pattern, t) == pkg.CSSSyndrome(syn.sx[0], syn.sz[0])
    ct.close()


@pytest.mark.parametrize("group,threads", [(1, 256), (2, 128), (2, 512), (1, 1024)])
def test_split_arena_shapes_vs_plain_f64(pkg, group, threads):
    """Launch shapes that keep each syndrome's small intermediates in shared
    memory and its large ones in global memory give the float64 result
    (float32 within its bound) and the same decisions."""
    t = pkg.tanner_graph(pkg.SurfaceCode(7, 7))
    em = pkg.depolarizing(0.05, t.nq)
    rng = np.random.default_rng(77)
    ep = pkg.random_error_pattern(em, rng, nsamples=300)
    s = pkg.syndrome_extraction(ep, t)
    bits = np.concatenate([s.sx, s.sz], axis=1)
    ref = pkg.compile(pkg.TNMMAP(precision="f64", plain=True), t, em)
    want = ref.class_logprobs(bits)
    ref.close()
    for precision in ("f64", "f32"):
        ct = pkg.compile(pkg.TNMMAP(precision=precision, group=group, threads=threads, split_arena=True), t, em)
        info = ct.program.info
        assert info["arena_small"] > 0 and info[f"split_{precision}"] == 1
        lp = ct.class_logprobs(bits)
        if precision == "f64":
            assert_class_logprobs(lp, np.exp(want))
        else:
            assert_class_logprobs_within(lp, np.exp(want), 2 * info["err_bound_f32"])
        assert_decisions(ct.decode_batch(bits), np.exp(want))
        ct.close()


@pytest.mark.parametrize("threads", [128, 256, 512])
def test_shared_item_shapes_vs_plain_f64(pkg, threads):
    """One-syndrome blocks whose lanes share the four-output items of steps
    that would leave threads idle (each lane a run of the contracted range,
    partial sums combined by shuffles): float64 and double-float per class
    within 1e-10 of the plain float64 contraction, float32 within its bound,
    the same decisions."""
    t = pkg.tanner_graph(pkg.SurfaceCode(7, 7))
    em = pkg.depolarizing(0.06, t.nq)
    ep = pkg.random_error_pattern(em, np.random.default_rng(78), nsamples=300)
    s = pkg.syndrome_extraction(ep, t)
    bits = np.concatenate([s.sx, s.sz], axis=1)
    ref = pkg.compile(pkg.TNMMAP(precision="f64", plain=True), t, em)
    want = np.exp(ref.class_logprobs(bits))
    ref.close()
    for precision in ("f64", "f32"):
        ct = pkg.compile(pkg.TNMMAP(precision=precision, group=1, threads=threads, shared_items=True), t, em)
        info = ct.program.info
        assert info[f"shared_items_{precision}"] == 1
        lp = ct.class_logprobs(bits)
        if precision == "f64":
            assert_class_logprobs(lp, want)
        else:
            assert_class_logprobs_within(lp, want, 2 * info["err_bound_f32"])
            assert_class_logprobs(ct.class_logprobs(bits, precision="f32x2"), want)
        assert_decisions(ct.decode_batch(bits), want)
        ct.close()


def test_tensor_core_steps_vs_float64(pkg):
    """GEMM-shaped steps of a circuit-level model (rotated Z-memory d=5, 2
    rounds) run on the tensor cores in float32 launches (tf32 high/low
    split); the result stays within the float32 program's bound of the
    float64 contraction (float64 runs them on the SIMT path) and decides the
    same classes outside exact ties."""
    from tensorqec_gb300 import circuit, dem as demmod

    dm = circuit.detector_error_model(circuit.memory_z_circuit(5, 2, 0.001))
    rng = np.random.default_rng(8)
    _, det, _ = demmod.sample_dem(dm, 256, rng)
    ct32 = pkg.compile(pkg.TNMMAP(precision="f32", optimizer=pkg.TreeSA(trials=16, sweeps=1000, restarts=2)), dm)
    info = ct32.program.info
    assert info["tensor_steps"] > 0 and info["tensor_f32"] == 1
    lp32 = ct32.class_logprobs(det)
    lp64 = ct32.class_logprobs(det, precision="f64")
    top = np.max(lp64, axis=1, keepdims=True)
    assert np.max(np.abs(np.exp(lp32 - top) - np.exp(lp64 - top))) <= 2 * info["err_bound_f32"]
    cls = ct32.decode_batch(det)
    srt = np.sort(lp64, axis=1)
    tie = (srt[:, -1] - srt[:, -2]) <= 1e-9
    assert not ((cls != np.argmax(lp64, axis=1)) & ~tie).any()
    ct32.close()


def test_tensor_cores_switch_and_autotune(pkg):
    """The same circuit-level program with its GEMM-shaped steps on the SIMT
    path (TQEC_FLAG_NO_TENSOR_CORES) and after an autotune that may pick
    either path: both stay within the float32 bound of float64."""
    from tensorqec_gb300 import circuit, dem as demmod

    dm = circuit.detector_error_model(circuit.memory_z_circuit(5, 2, 0.001))
    _, det, _ = demmod.sample_dem(dm, 512, np.random.default_rng(9))
    opt = pkg.TreeSA(trials=16, sweeps=1000, restarts=2, seed=3)
    ct_tc = pkg.compile(pkg.TNMMAP(precision="f32", optimizer=opt), dm)
    ct_si = pkg.compile(pkg.TNMMAP(precision="f32", optimizer=opt, tensor_cores=False), dm)
    assert ct_tc.program.info["tensor_steps"] > 0
    assert ct_si.program.info["tensor_steps"] == 0 and ct_si.program.info["tensor_f32"] == 0
    lp64 = ct_tc.class_logprobs(det, precision="f64")
    top = np.max(lp64, axis=1, keepdims=True)
    for ct in (ct_si, ct_tc):
        ct.program.autotune(512)
        lp32 = ct.class_logprobs(det)
        bound = 2 * ct.program.info["err_bound_f32"]
        assert np.max(np.abs(np.exp(lp32 - top) - np.exp(lp64 - top))) <= bound
    ct_tc.close()
    ct_si.close()


@pytest.mark.parametrize("kind,d,p,n", [("surface", 5, 0.08, 400), ("surface", 7, 0.05, 48),
                                        ("toric", 3, 0.05, 128), ("666", 5, 0.08, 128)])
def test_f32x2_marginals_vs_oracle(pkg, oracle, kind, d, p, n):
    """Double-float contraction (pairs of float32, the recheck's default
    arithmetic): marginals within its stated bound of the oracle, a bound
    2^-19 times float32's."""
    t, em, bits, dec = css_case(pkg, oracle, kind, d, p, n, seed=200 + d)
    want = dec.marginals(bits)
    ct = pkg.compile(pkg.TNMMAP(precision="f32"), t, em)
    info = ct.program.info
    assert info["recheck_precision"] == pkg.native.TQEC_F32X2
    bound = info["err_bound_f32x2"]
    assert bound <= info["err_bound_f32"] * 2.0 ** -19 * 1.001
    assert_marginals(ct.class_logprobs(bits, precision="f32x2"), want, 2 * bound)
    ct.close()


@pytest.mark.parametrize("recheck_f64", [False, True])
def test_recheck_every_row(pkg, recheck_f64):
    """A margin no float32 result clears sends every row to the recheck:
    decisions equal float64's outside ties, every row is counted, and each
    row's error bound is the recheck arithmetic's."""
    t = pkg.tanner_graph(pkg.SurfaceCode(7, 7))
    em = pkg.depolarizing(0.08, t.nq)
    ep = pkg.random_error_pattern(em, np.random.default_rng(13), nsamples=600)
    syn = pkg.syndrome_extraction(ep, t)
    bits = np.concatenate([syn.sx, syn.sz], axis=1)
    ct = pkg.compile(pkg.TNMMAP(precision="f32", margin=1e30, recheck_f64=recheck_f64), t, em)
    info = ct.program.info
    want_prec = pkg.native.TQEC_F64 if recheck_f64 else pkg.native.TQEC_F32X2
    assert info["recheck_precision"] == want_prec
    assert info["cluster_blocks"] in (8, 16)  # d=7 is wide: each recheck row on a cluster
    packed = pkg.pack_syndromes(bits)
    logp = np.empty((len(bits), ct.n_classes))
    err = np.empty(len(bits), dtype=np.float32)
    cls = ct.program.decode_packed(packed, logp=logp, err=err)
    assert ct.program.last_recheck_count() == len(bits)
    bound = info["err_bound_f64"] if recheck_f64 else info["err_bound_f32x2"]
    np.testing.assert_allclose(err, np.float32(bound), rtol=1e-6)
    lp64 = ct.class_logprobs(bits, precision="f64")
    # class by class within the recheck arithmetic's bound of float64
    assert_class_logprobs_within(logp, np.exp(lp64), 2 * bound + 1e-15)
    srt = np.sort(lp64, axis=1)
    tie = (srt[:, -1] - srt[:, -2]) <= 1e-9
    assert not ((cls != np.argmax(lp64, axis=1)) & ~tie).any()
    ct.close()


@pytest.mark.parametrize("small_in_smem", [1, 0])
def test_cluster_placements_vs_plain_block_form(pkg, small_in_smem):
    """The plain float64 form at d=7 on 16-block clusters with the small
    intermediates in the first block's shared memory (1) or with every
    intermediate in global memory (0), one row per call and a batch: per
    class within 1e-10 of the one-block form, the same decisions."""
    t = pkg.tanner_graph(pkg.SurfaceCode(7, 7))
    em = pkg.depolarizing(0.07, t.nq)
    ep = pkg.random_error_pattern(em, np.random.default_rng(41), nsamples=64)
    syn = pkg.syndrome_extraction(ep, t)
    bits = np.concatenate([syn.sx, syn.sz], axis=1)
    ct = pkg.compile(pkg.TNMMAP(precision="f64", plain=True), t, em)
    ct.program.set_cluster(pkg.native.TQEC_F64, 0)
    want = np.exp(ct.class_logprobs(bits))
    ct.program.set_cluster(pkg.native.TQEC_F64, 16, 128, small_in_smem)
    assert ct.program.info["cluster_blocks"] == 16
    cls, logp = ct.decode_batch(bits, return_logp=True)
    assert_class_logprobs(logp, want)
    for r in range(0, 64, 13):
        c1, l1 = ct.decode_batch(bits[r:r + 1], return_logp=True)
        assert c1[0] == cls[r]
        assert_class_logprobs(l1, want[r:r + 1])
    srt = np.sort(want, axis=1)
    tie = (srt[:, -1] - srt[:, -2]) <= 1e-9 * srt[:, -1]
    assert not ((cls != np.argmax(want, axis=1)) & ~tie).any()
    ct.close()


def test_f32x2_circuit_level(pkg):
    """Double-float on a circuit-level program (rotated Z-memory d=5, 2
    rounds): within its bound of float64."""
    from tensorqec_gb300 import circuit, dem as demmod

    dm = circuit.detector_error_model(circuit.memory_z_circuit(5, 2, 0.001))
    _, det, _ = demmod.sample_dem(dm, 256, np.random.default_rng(21))
    ct = pkg.compile(pkg.TNMMAP(precision="f32", optimizer=pkg.TreeSA(trials=16, sweeps=1000, restarts=2)), dm)
    lp2 = ct.class_logprobs(det, precision="f32x2")
    lp64 = ct.class_logprobs(det, precision="f64")
    top = lp64.max(axis=1, keepdims=True)
    assert np.max(np.abs(np.exp(lp2 - top) - np.exp(lp64 - top))) <= 2 * ct.program.info["err_bound_f32x2"]
    ct.close()
