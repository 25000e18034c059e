"""Host-side logic of the product against the oracle and the reference's
known answers (no GPU)."""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_kat.json")


@pytest.fixture(scope="module")
def kat():
    with open(GOLD) as f:
        return json.load(f)


CODES = [("surface", 3), ("surface", 5), ("surface", 7), ("surface", 4), ("toric", 3), ("toric", 4),
         ("488", 5), ("666", 5), ("488", 7), ("666", 7)]


def _codes(pkg, oracle, kind, d):
    if kind == "surface":
        return pkg.SurfaceCode(d, d), oracle.surface_code_stabilizers(d, d)
    if kind == "toric":
        return pkg.ToricCode(d, d), oracle.toric_code_stabilizers(d, d)
    return (pkg.Color488(d) if kind == "488" else pkg.Color666(d)), oracle.color_code_stabilizers(kind, d)


@pytest.mark.parametrize("kind,d", CODES)
def test_stabilizers_and_logicals_match_oracle(pkg, oracle, kind, d):
    code, (ost, onq) = _codes(pkg, oracle, kind, d)
    t = pkg.tanner_graph(code)
    ot = oracle.css_tanner(ost, onq)
    assert t.nq == onq
    assert t.stgx.s2q == [list(s) for s in ot.stgx.s2q]
    assert t.stgz.s2q == [list(s) for s in ot.stgz.s2q]
    lx, lz = pkg.logical_operator(t)
    olx, olz = oracle.logical_operator(ot)
    assert np.array_equal(lx, olx) and np.array_equal(lz, olz)
    # CSS commutation and logical pairing
    assert not ((t.stgx.H.astype(int) @ t.stgz.H.T) % 2).any()
    assert not ((t.stgx.H.astype(int) @ lz.T) % 2).any()
    assert not ((t.stgz.H.astype(int) @ lx.T) % 2).any()
    # row j of lx anticommutes with row j of lz (same_qubit_order, code_distance.jl:84-100)
    assert ((lx.astype(int) * lz).sum(axis=1) % 2 == 1).all()


def test_logical_kat(pkg, kat):
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    lx, lz = pkg.logical_operator(t)
    assert lx.tolist() == kat["surface3_logical_operators"]["lx"]
    assert lz.tolist() == kat["surface3_logical_operators"]["lz"]


def test_row_echelon_kat(pkg, kat):
    k = kat["row_echelon_form"]
    assert pkg.row_echelon_form(np.array(k["H"])).tolist() == k["R"]


def test_toric_kat(pkg, kat):
    st = pkg.stabilizers(pkg.ToricCode(2, 3))
    code = {0: 1, 1: 2, 3: 4}
    assert [[code[o] for o in s.ops] for s in st] == kat["toric_2x3_stabilizers"]["ops"]


def test_parity_tensor_kat(pkg, kat):
    pc = pkg.parity_check_matrix(4)
    for idx, want in kat["parity_check_matrix_4"]["entries"]:
        assert pc[tuple(idx)] == want


@pytest.mark.parametrize("kind,d", [("surface", 3), ("surface", 5), ("toric", 3), ("488", 5)])
def test_factor_graph_matches_oracle(pkg, oracle, kind, d):
    code, (ost, onq) = _codes(pkg, oracle, kind, d)
    t = pkg.tanner_graph(code)
    em = pkg.depolarizing(0.07, t.nq)
    lx, lz = pkg.logical_operator(t)
    g = pkg.tnmmap_css_graph(t, em, lx, lz)
    ot = oracle.css_tanner(ost, onq)
    net = oracle.tnmmap_network(ot, em.px, em.py, em.pz)
    assert g.ixs == net.ixs
    assert g.iy == net.iy
    assert g.syndrome_positions == net.syndrome_positions
    for a, b in zip(g.tensors, net.tensors):
        np.testing.assert_array_equal(a, np.asarray(b).flatten(order="F"))


def test_sampler_semantics(pkg):
    em = pkg.iid_error(0.1, 0.2, 0.3, 5)
    rng = np.random.default_rng(0)
    ep = pkg.random_error_pattern(em, rng, nsamples=200000)
    y = (ep.xerror & ep.zerror).mean()
    x = (ep.xerror & (1 - ep.zerror)).mean()
    z = ((1 - ep.xerror) & ep.zerror).mean()
    assert abs(y - 0.2) < 0.005 and abs(x - 0.1) < 0.005 and abs(z - 0.3) < 0.005


def test_pack_roundtrip(pkg):
    rng = np.random.default_rng(3)
    bits = (rng.random((17, 48)) < 0.3).astype(np.uint8)
    packed = pkg.pack_syndromes(bits)
    assert packed.shape == (17, 6)
    assert np.array_equal(pkg.unpack_syndromes(packed, 48), bits)
    assert packed[0, 0] == sum(int(bits[0, j]) << j for j in range(8))


@pytest.mark.parametrize("d", [3, 5, 7])
def test_error_pattern_reproduces_syndrome_and_class(pkg, d):
    """error_pattern (tndecoder.jl:167-174) for every class: the pattern
    reproduces the syndrome and carries the requested class."""
    from tensorqec_gb300 import gf2  # noqa: F401  (loaded by the fixture)

    t = pkg.tanner_graph(pkg.SurfaceCode(d, d))
    lx, lz = pkg.logical_operator(t)
    px = pkg.gf2.solve_particular(t.stgz.H)
    pz = pkg.gf2.solve_particular(t.stgx.H)
    rng = np.random.default_rng(d)
    em = pkg.depolarizing(0.1, t.nq)
    ep = pkg.random_error_pattern(em, rng, nsamples=20)
    syn = pkg.syndrome_extraction(ep, t)
    for r in range(20):
        ex = px(syn.sz[r])
        ez = pz(syn.sx[r])
        assert np.array_equal((t.stgz.H.astype(int) @ ex) % 2, syn.sz[r])
        assert np.array_equal((t.stgx.H.astype(int) @ ez) % 2, syn.sx[r])


def test_impossible_syndrome_has_no_particular_solution(pkg):
    t = pkg.tanner_graph(pkg.ToricCode(3, 3))
    # toric checks are dependent before removal; after removal every
    # syndrome is reachable, so use an over-complete matrix instead
    H = np.vstack([t.stgz.H, t.stgz.H[:1]])
    solve = pkg.gf2.solve_particular(H)
    s = np.zeros(H.shape[0], dtype=np.uint8)
    s[-1] = 1
    assert solve(s) is None


def test_dem_parse_and_tanner(pkg, oracle, kat):
    text = kat["dem_small"]["text"]
    dem = pkg.parse_dem_string(text)
    odem = oracle.parse_dem_string(text)
    assert dem.flipped_detectors == odem.flipped
    assert dem.detector_list == odem.detector_list and dem.logical_list == odem.logical_list
    t = pkg.dem2tanner(dem)
    ot = oracle.dem2tanner(odem)
    assert t.s2q == ot.s2q
    assert pkg.parse_dem_string(pkg.dem.to_dem_string(dem)).flipped_detectors == dem.flipped_detectors
    with pytest.raises(ValueError):
        pkg.parse_dem_string("repeat 3 {\n}\n")


def test_dem_graph_matches_oracle(pkg, oracle, kat):
    dem = pkg.parse_dem_string(kat["dem_small"]["text"])
    g = pkg.tnmmap_dem_graph(pkg.dem2tanner(dem), pkg.logical_map(dem), dem.error_rates,
                             len(dem.logical_list), True)
    net, _, _ = oracle.dem_network(oracle.parse_dem_string(kat["dem_small"]["text"]), True)
    assert g.ixs == net.ixs and g.iy == net.iy and g.syndrome_positions == net.syndrome_positions
    for a, b in zip(g.tensors, net.tensors):
        np.testing.assert_array_equal(a, np.asarray(b).flatten(order="F"))


@pytest.mark.parametrize("kind,d", [("surface", 5), ("toric", 3), ("488", 5)])
def test_right_inverse(pkg, oracle, kind, d):
    code, _ = _codes(pkg, oracle, kind, d)
    t = pkg.tanner_graph(code)
    rng = np.random.default_rng(d)
    for H in (t.stgx.H, t.stgz.H, np.vstack([t.stgz.H, t.stgz.H[:2]])):
        R, Cc = pkg.gf2.right_inverse(H)
        for _ in range(20):
            e = (rng.random(H.shape[1]) < 0.2).astype(np.int64)
            s = (H.astype(np.int64) @ e) % 2
            e2 = (R.astype(np.int64) @ s) % 2
            assert np.array_equal((H.astype(np.int64) @ e2) % 2, s)
            assert not ((Cc.astype(np.int64) @ s) % 2).any()
        if Cc.shape[0]:
            # a syndrome violating a consistency row is not reachable
            s = np.zeros(H.shape[0], dtype=np.int64)
            s[np.flatnonzero(Cc[0])[0]] = 1
            assert ((Cc.astype(np.int64) @ s) % 2).any()


@pytest.mark.parametrize("m", [3, 4])
def test_toric_logical_pairing(pkg, oracle, m):
    """test/codes/code_distance.jl:97-115: on the toric code, X on the
    support of lx row i anticommutes with lz row i only, and both rows
    commute with every stabiliser."""
    t = pkg.tanner_graph(pkg.ToricCode(m, m))
    lx, lz = pkg.logical_operator(t)
    assert lx.shape == lz.shape == (2, 2 * m * m)
    assert np.array_equal((lx.astype(int) @ lz.T) % 2, np.eye(2, dtype=int))
    assert not ((t.stgz.H.astype(int) @ lx.T) % 2).any()
    assert not ((t.stgx.H.astype(int) @ lz.T) % 2).any()
    olx, olz = oracle.logical_operator(oracle.css_tanner(*oracle.toric_code_stabilizers(m, m)))
    assert np.array_equal(lx, olx) and np.array_equal(lz, olz)


def test_bivariate_bicycle_144_12_12(pkg, oracle):
    """test/codes/codes.jl:160-173: the [[144,12,12]] bivariate bicycle code
    has 132 independent stabilisers and 12 logical qubits; with 11 of its lz
    rows added as Z stabilisers one logical pair remains."""
    code = pkg.BivariateBicycleCode(6, 12, ((3, 0), (0, 1), (0, 2)), ((0, 3), (1, 0), (2, 0)))
    st = pkg.stabilizers(code)
    assert len(st) == 132
    t = pkg.CSSTannerGraph.from_stabilizers(st)
    lx, lz = pkg.logical_operator(t)
    assert lx.shape == lz.shape == (12, 144)
    ost, onq = oracle.bivariate_bicycle_stabilizers(6, 12, ((3, 0), (0, 1), (0, 2)), ((0, 3), (1, 0), (2, 0)))
    olx, olz = oracle.logical_operator(oracle.css_tanner(ost, onq))
    assert np.array_equal(lx, olx) and np.array_equal(lz, olz)
    st2 = list(st) + [pkg.PauliString.of(144, [int(q) + 1 for q in np.flatnonzero(lz[i])], 3) for i in range(11)]
    lx2, lz2 = pkg.logical_operator(pkg.CSSTannerGraph.from_stabilizers(st2))
    assert lx2.shape == lz2.shape == (1, 144)


def test_syndrome_rows_from_single_batched_and_listed_syndromes(pkg):
    """The rows a decoder reads ([sx..., sz...], tndecoder.jl:148-158) from
    one CSSSyndrome, from the batched one syndrome_extraction returns for a
    batch of error patterns, and from a list of single ones."""
    from tensorqec_gb300.decoder import CompiledTNMMAP

    t = pkg.tanner_graph(pkg.SurfaceCode(5, 5))
    em = pkg.depolarizing(0.1, t.nq)
    ep = pkg.random_error_pattern(em, np.random.default_rng(3), nsamples=9)
    syn = pkg.syndrome_extraction(ep, t)
    want = np.concatenate([syn.sx, syn.sz], axis=1)
    np.testing.assert_array_equal(syn.bits(), want)
    rows = CompiledTNMMAP._bits(None, syn)
    np.testing.assert_array_equal(rows, want)
    singles = [pkg.CSSSyndrome(syn.sx[i], syn.sz[i]) for i in range(9)]
    np.testing.assert_array_equal(singles[4].bits(), want[4])
    np.testing.assert_array_equal(CompiledTNMMAP._bits(None, singles[4]), want[4:5])
    np.testing.assert_array_equal(CompiledTNMMAP._bits(None, singles), want)
    np.testing.assert_array_equal(CompiledTNMMAP._bits(None, want), want)


def test_simple_syndrome_rows(pkg):
    """DEM and TNMAP decoders read rows from one SimpleSyndrome, a batched
    one, a list of them, or 0/1 rows."""
    from tensorqec_gb300.decoder import simple_rows

    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3)).stgz
    e = pkg.random_error_pattern(pkg.iid_error(0.2, t.nq), np.random.default_rng(5), nsamples=6)
    syn = pkg.syndrome_extraction(e, t)
    want = np.asarray(syn.s)
    assert want.shape == (6, t.ns)
    np.testing.assert_array_equal(simple_rows(syn), want)
    np.testing.assert_array_equal(simple_rows([pkg.SimpleSyndrome(r) for r in want]), want)
    np.testing.assert_array_equal(simple_rows(pkg.SimpleSyndrome(want[2])), want[2:3])
    np.testing.assert_array_equal(simple_rows(want), want)


def test_dem_with_single_mechanism_checks(pkg, oracle):
    """A detector and a logical flipped by one mechanism each: the factorised
    network keeps them as single parity tensors, and the compiled program
    reproduces the enumeration over all mechanism subsets."""
    from plan_emulator import run_plan

    text = "error(0.1) D0 D1\nerror(0.2) D1\nerror(0.05) D0 L0\nerror(0.15) D2 D1 D0\nerror(0.3) D1 D0\n"
    dem = pkg.parse_dem_string(text)
    t = pkg.dem2tanner(dem)
    g = pkg.tnmmap_dem_graph(t, pkg.logical_map(dem), dem.error_rates, 1, True)
    plan = pkg.native.inspect_plan(g, pkg.optimize_code(g, pkg.TreeSA(trials=2, sweeps=50)))
    bits = ((np.arange(8)[:, None] >> np.arange(3)[None, :]) & 1).astype(np.uint8)
    got = run_plan(plan, bits)
    p = np.array(dem.error_rates)
    want = np.zeros((8, 2))
    for m in range(1 << 5):
        e = (m >> np.arange(5)) & 1
        prob = np.prod(np.where(e == 1, p, 1 - p))
        det = sum(((sum(e[j] for j, f in enumerate(dem.flipped_detectors) if d in f) % 2) << (d - 1))
                  for d in (1, 2, 3))
        lg = sum(e[j] for j, f in enumerate(dem.flipped_detectors) if 4 in f) % 2
        want[det, lg] += prob
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-300)
    dec = oracle.OracleDEMDecoder(oracle.parse_dem_string(text))
    np.testing.assert_allclose(dec.marginals(bits), want, rtol=1e-12, atol=1e-300)


def _code_distance(t, lx, lz):
    """code_distance(::CSSTannerGraph) (code_distance.jl:256-298) by
    enumeration: the least weight of an X-type vector with even overlap with
    every Z check and odd overlap with some row of lz, and the same for Z."""
    from tensorqec_gb300 import gf2

    best = []
    for H, L in ((t.stgz.H, lz), (t.stgx.H, lx)):
        ns = gf2.null_space(np.asarray(H, dtype=np.uint8)).astype(np.int64)
        k = ns.shape[0]
        assert k <= 16
        combos = ((np.arange(1 << k)[:, None] >> np.arange(k)) & 1) @ ns % 2
        odd = ((combos @ np.asarray(L, dtype=np.int64).T) % 2).any(axis=1)
        best.append(int(combos[odd].sum(axis=1).min()))
    return min(best)


@pytest.mark.parametrize("name,make,n_stab,distance", [
    ("steane", lambda p: p.SteaneCode(), 6, 3), ("shor", lambda p: p.ShorCode(), 8, 3),
    ("1573", lambda p: p.Code1573(), 8, 3), ("832", lambda p: p.Code832(), 5, 2),
    ("422", lambda p: p.Code422(), 2, 2), ("surface3", lambda p: p.SurfaceCode(3, 3), 8, 3),
    ("color488_5", lambda p: p.Color488(5), 16, 5), ("color666_5", lambda p: p.Color666(5), 18, 5)])
def test_reference_code_known_answers(pkg, name, make, n_stab, distance):
    """test/codes/codes.jl:42-187: code distances (the reference solves an
    integer program; here the kernel of the check matrix is enumerated) and
    stabiliser counts (n - k; the reference asserts them for the colour
    codes)."""
    code = make(pkg)
    st = pkg.stabilizers(code)
    assert len(st) == n_stab
    t = pkg.tanner_graph(code)
    lx, lz = pkg.logical_operator(t)
    assert _code_distance(t, lx, lz) == distance
    if name == "422":  # codes.jl:127-133: XXXX then ZZZZ
        assert [s.ops for s in st] == [(1, 1, 1, 1), (3, 3, 3, 3)]


def test_bivariate_bicycle_98_6_12_stabilizer_count(pkg):
    """test/codes/codes.jl:154-158."""
    code = pkg.BivariateBicycleCode(7, 7, ((1, 0), (0, 3), (0, 4)), ((0, 1), (3, 0), (4, 0)))
    st = pkg.stabilizers(code)
    assert len(st) == 92
    t = pkg.CSSTannerGraph.from_stabilizers(st)
    lx, lz = pkg.logical_operator(t)
    assert lx.shape == lz.shape == (6, 98)


def test_reference_error_model_known_answers(pkg):
    """test/decoding/error_model.jl:5-40: flip rates of a depolarising
    sample (X part px + py, Z part pz + py) and check_logical_error on the
    d=3 surface code's logical operators."""
    em = pkg.iid_error(0.05, 0.06, 0.1, 100000)
    ep = pkg.random_error_pattern(em, np.random.default_rng(0))
    assert abs(ep.xerror.mean() - 0.11) < 0.05 and abs(ep.zerror.mean() - 0.16) < 0.05
    flips = pkg.random_error_pattern(pkg.iid_error(0.1, 10), np.random.default_rng(1))
    assert flips.shape == (10,) and set(np.unique(flips)) <= {0, 1}
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    lx, lz = pkg.logical_operator(t)
    zero = np.zeros(9, np.uint8)
    assert pkg.check_logical_error(zero, np.array([1, 1, 1, 0, 0, 0, 0, 0, 0], np.uint8), lz)
    assert not pkg.check_logical_error(zero, np.array([1, 1, 0, 1, 1, 0, 0, 0, 0], np.uint8), lz)
    css = pkg.CSSErrorPattern(zero, zero)
    assert not pkg.check_logical_error(css, pkg.CSSErrorPattern(zero.copy(), zero.copy()), lx, lz)


def test_bench_reads_the_committed_traffic_figures():
    """bench.py's roofline traffic comes from profiles/roofline_traffic.txt:
    the full-batch launch's bytes and the gated step's fallback bytes per row."""
    import importlib.util
    import os

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("bench_for_test", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    full = bench.read_traffic()
    per_row = bench.read_traffic(f"tn_contract_f32_d{bench.D}_fallback_bytes_per_row")
    assert full is not None and full > 1e9
    assert per_row is not None and 1e4 < per_row < 1e7
