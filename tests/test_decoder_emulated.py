"""The Python mirror of the reference's decoder API (compile / decode,
src/decoding/interfaces.jl:74-119, tndecoder.jl) on the CPU: the GPU
program is replaced by the numpy emulator of the same compiled program
(the ``emulated`` fixture), so what runs here is the host side a user calls
— network building, order search, planning, syndrome rows, class choice,
error patterns, DEM and TNMAP decoding — against the oracle.  The same
calls on the GPU are covered by the gpu-marked tests.
"""
import json
import os

import numpy as np
import pytest


def _kat():
    with open(os.path.join(os.path.dirname(__file__), "golden", "reference_kat.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_css_decode_batch_decode_and_patterns(pkg, oracle, emulated, precision):
    t = pkg.tanner_graph(pkg.SurfaceCode(5, 5))
    em = pkg.depolarizing(0.08, t.nq)
    ct = pkg.compile(pkg.TNMMAP(precision=precision, optimizer=pkg.TreeSA(trials=4, sweeps=200, restarts=1)), t, em)
    ep = pkg.random_error_pattern(em, np.random.default_rng(8), nsamples=200)
    syn = pkg.syndrome_extraction(ep, t)
    want = oracle.OracleDecoder(oracle.css_tanner(*oracle.surface_code_stabilizers(5, 5)), em.px, em.py,
                                em.pz).marginals(np.concatenate([syn.sx, syn.sz], axis=1))
    cls, lp = ct.decode_batch(syn, return_logp=True)   # the batched CSSSyndrome itself
    np.testing.assert_allclose(np.exp(lp), want, rtol=1e-10, atol=1e-12 * want.max())
    top = want.max(axis=1)
    assert (want[np.arange(len(cls)), cls] >= top * (1 - 1e-9)).all()
    lx, lz = pkg.logical_operator(t)
    for i in range(10):
        s = pkg.CSSSyndrome(syn.sx[i], syn.sz[i])
        res = pkg.decode(ct, s)
        assert res.success_tag and pkg.syndrome_extraction(res.error_pattern, t) == s
        # the decoded pattern lies in the decoded class: no logical error against
        # the class representative the decoder reports
        e = res.error_pattern
        a = (lx.astype(int) @ e.zerror) % 2
        b = (lz.astype(int) @ e.xerror) % 2
        assert int(a[0]) + 2 * int(b[0]) == cls[i]


def test_reference_x1_decision_kat_through_the_api(pkg, oracle, emulated):
    """test/decoding/tndecoder.jl:60-73: X on qubit 1 with px=0.1 decodes to
    no logical error.  With px=0.26 on qubits 2 and 3 the reference's TNMAP
    decodes it into a logical error (:75-85, test_map.py); TNMMAP does too,
    since its marginal sums every error of a class and the class of X2 X3
    outweighs that of X1 — the decision equals the oracle's argmax."""
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    lx, lz = pkg.logical_operator(t)
    ex = np.zeros(9, np.uint8)
    ex[0] = 1
    truth = pkg.CSSErrorPattern(ex, np.zeros(9, np.uint8))
    syn = pkg.syndrome_extraction(truth, t)
    ot = oracle.css_tanner(*oracle.surface_code_stabilizers(3, 3))
    for p23, logical_error in ((0.1, False), (0.26, True)):
        px = np.full(9, 0.1)
        px[1] = px[2] = p23
        em = pkg.IndependentDepolarizingError(px, np.zeros(9), np.zeros(9))
        res = pkg.decode(pkg.TNMMAP(precision="f64"), t, syn, em)
        assert res.success_tag and pkg.syndrome_extraction(res.error_pattern, t) == syn
        assert bool(pkg.check_logical_error(res.error_pattern, truth, lx, lz)) == logical_error
        want = oracle.OracleDecoder(ot, px, 0.0, 0.0).marginal(syn.bits())
        e = res.error_pattern
        assert int((lz.astype(int) @ e.xerror)[0] % 2) * 2 == int(np.argmax(want))


def test_dem_decode_every_syndrome(pkg, oracle, emulated):
    """The reference's dem.dem (tndecoder.jl:112-121 decodes one sample of
    it): every detector pattern's class against the oracle, and the error
    pattern reproduces the detectors with the decoded logical flips."""
    text = _kat()["dem_small"]["text"]
    dem = pkg.parse_dem_string(text)
    ct = pkg.compile(pkg.TNMMAP(precision="f64", optimizer=pkg.TreeSA(trials=4, sweeps=100)), dem)
    nd = len(dem.detector_list)
    bits = ((np.arange(1 << nd)[:, None] >> np.arange(nd)[None, :]) & 1).astype(np.uint8)
    want = oracle.OracleDEMDecoder(oracle.parse_dem_string(text)).marginals(bits)
    cls = ct.decode_batch([pkg.SimpleSyndrome(b) for b in bits])
    possible = want.max(axis=1) > 0
    assert (cls[possible] == np.argmax(want[possible], axis=1)).all()
    t = pkg.dem2tanner(dem)
    l2q = pkg.logical_map(dem)
    for r in np.flatnonzero(possible)[:16]:
        res = ct.decode(pkg.SimpleSyndrome(bits[r]))
        assert res.success_tag
        e = np.asarray(res.error_pattern)
        np.testing.assert_array_equal(pkg.syndrome_extraction(e, t).s, bits[r])
        flips = sum((int(e[np.array(l) - 1].sum()) % 2) << i for i, l in enumerate(l2q))
        assert flips == cls[r]


def test_tnmap_css_decode(pkg, oracle, emulated):
    """compile(TNMAP(), tanner, em) and decode (tndecoder.jl:33-57 through
    reduce2general): the configuration reproduces the syndrome and is a most
    probable one."""
    from tensorqec_gb300 import network

    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    em = pkg.iid_error(0.05, 0.06, 0.1, t.nq)
    ct = pkg.compile(pkg.TNMAP(), t, em)
    ep = pkg.random_error_pattern(em, np.random.default_rng(2), nsamples=12)
    syn = pkg.syndrome_extraction(ep, t)
    general, ixs, ts = network.reduce2general(t, em)
    bits = np.concatenate([syn.sx, syn.sz], axis=1)
    best = oracle.most_probable_configs(general.H, ixs, ts, bits)
    for r in range(12):
        s = pkg.CSSSyndrome(syn.sx[r], syn.sz[r])
        res = pkg.decode(ct, s)
        assert pkg.syndrome_extraction(res.error_pattern, t) == s
        cfg = np.concatenate([res.error_pattern.xerror, res.error_pattern.zerror])[None, :]
        got = oracle.config_log_probability(ixs, ts, cfg)[0]
        assert abs(got - best[r][0]) <= 1e-12 * abs(best[r][0])


def test_multi_round_qec(pkg, oracle, emulated):
    """multi_round_qec (threshold.jl:1-19) over batches: the X, Z and total
    logical error rates equal those of the oracle's argmax decisions on the
    same sampled errors (same seed)."""
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    em = pkg.depolarizing(0.1, t.nq)
    dec = pkg.TNMMAP(precision="f64", optimizer=pkg.TreeSA(trials=2, sweeps=50, restarts=1))
    rates = pkg.multi_round_qec(t, dec, em, rounds=500, rng=np.random.default_rng(4), batch=128, prior=em)
    rng = np.random.default_rng(4)
    ot = oracle.css_tanner(*oracle.surface_code_stabilizers(3, 3))
    od = oracle.OracleDecoder(ot, em.px, em.py, em.pz)
    nx = nz = nany = ties = 0
    for n in (128, 128, 128, 116):
        ep = pkg.random_error_pattern(em, rng, nsamples=n)
        s = pkg.syndrome_extraction(ep, t)
        mar = od.marginals(np.concatenate([s.sx, s.sz], axis=1))
        cls = np.argmax(mar, axis=1)
        srt = np.sort(mar, axis=1)
        ties += int((srt[:, -1] - srt[:, -2] <= 1e-9 * srt[:, -1]).sum())
        a = (ep.zerror.astype(int) @ od.lx.T.astype(int))[:, 0] % 2
        b = (ep.xerror.astype(int) @ od.lz.T.astype(int))[:, 0] % 2
        xe, ze = (cls >> 1) != b, (cls & 1) != a
        nx, nz, nany = nx + xe.sum(), nz + ze.sum(), nany + (xe | ze).sum()
    # rows whose top two classes tie may resolve either way
    for got, want in zip(rates, (nx, nz, nany)):
        assert abs(got * 500 - want) <= ties
    assert 0 < rates[2] < 0.5 and ties < 100


def test_multi_round_qec_classical(pkg, oracle, emulated):
    """The classical overload (threshold.jl:21-33): TNMAP on the Z checks of
    the d=3 surface code, bit flips at 0.1, logical errors read off the
    Z logical; with the reference's default decoding prior (0.05)."""
    from tensorqec_gb300 import network

    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    lx, lz = pkg.logical_operator(t)
    check = pkg.SimpleTannerGraph(9, [[int(q) + 1 for q in np.flatnonzero(lz[0])]])
    em = pkg.iid_error(0.1, 9)
    rate = pkg.multi_round_qec(t.stgz, pkg.TNMAP(), em, check, rounds=300, rng=np.random.default_rng(6), batch=100)
    rng = np.random.default_rng(6)
    ex = np.concatenate([pkg.random_error_pattern(em, rng, nsamples=100) for _ in range(3)])
    syn = (ex.astype(int) @ t.stgz.H.T.astype(int)) % 2
    ixs = [[i + 1] for i in range(9)]
    ts = [np.array([0.95, 0.05]) for _ in range(9)]
    best = oracle.most_probable_configs(t.stgz.H, ixs, ts, syn)
    # most probable configurations are the minimum-weight ones; count rounds
    # where every one of them is a logical error, and where any is
    always = maybe = 0
    for r in range(300):
        errs = [int(((ex[r] + np.asarray(c)) % 2) @ lz[0] % 2) for c in best[r][1]]
        always += all(errs)
        maybe += any(errs)
    assert always <= rate * 300 <= maybe
    assert 0 < rate < 0.5


def test_reference_threshold_calls(pkg, emulated):
    """test/decoding/threshold.jl:5-12 with TNMAP in place of the integer
    program decoder: the classical form (Z checks decoded, X checks as the
    logical test) returns one rate, the CSS form three."""
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    r = pkg.multi_round_qec(t.stgz, pkg.TNMAP(), pkg.iid_error(0.05, 9), t.stgx, rng=np.random.default_rng(123))
    assert isinstance(r, float) and 0 <= r <= 1
    r3 = pkg.multi_round_qec(t, pkg.TNMAP(), pkg.iid_error(0.05, 0.05, 0.05, 9), rounds=200,
                             rng=np.random.default_rng(123))
    assert isinstance(r3, tuple) and len(r3) == 3 and all(isinstance(x, float) for x in r3)
    assert max(r3[0], r3[1]) <= r3[2] <= r3[0] + r3[1] and r3[2] < 0.5
    r3m = pkg.multi_round_qec(t, pkg.TNMMAP(precision="f64"), pkg.iid_error(0.05, 0.05, 0.05, 9), rounds=200,
                              rng=np.random.default_rng(123))
    assert max(r3m[0], r3m[1]) <= r3m[2] <= r3m[0] + r3m[1]


def test_reference_interface_calls(pkg, emulated):
    """test/decoding/interfaces.jl:5-30 with TNMAP: decode(decoder, tanner,
    syndrome) on a classical problem and compile(decoder, tanner) with the
    default noise then decode on a CSS one both give a DecodingResult whose
    pattern reproduces the syndrome."""
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    e = np.array([0, 0, 0, 1, 0, 0, 0, 0, 0], np.uint8)
    syn = pkg.syndrome_extraction(e, t.stgz)
    res = pkg.decode(pkg.TNMAP(), t.stgz, syn)
    assert isinstance(res, pkg.DecodingResult)
    np.testing.assert_array_equal(pkg.syndrome_extraction(res.error_pattern, t.stgz).s, syn.s)
    em = pkg.iid_error(0.05, 0.06, 0.1, 9)
    ep = pkg.random_error_pattern(em, np.random.default_rng(123))
    s = pkg.syndrome_extraction(ep, t)
    for dec in (pkg.TNMAP(), pkg.TNMMAP(precision="f64")):
        ct = pkg.compile(dec, t)
        r = pkg.decode(ct, s)
        assert isinstance(r, pkg.DecodingResult) and pkg.syndrome_extraction(r.error_pattern, t) == s
