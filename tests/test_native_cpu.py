"""The native library without a GPU: it loads, exports everything the
header declares, rejects bad input with status codes, and its planner's
program (run by the numpy emulator) reproduces the oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from plan_emulator import run_plan

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    syms = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            syms |= set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\*?(tqec_\w+)\s*\(", text, re.M))
    return syms


def test_library_exports_header_symbols(pkg):
    lib = pkg.native.lib()
    syms = header_symbols()
    assert len(syms) >= 12
    for s in syms:
        assert hasattr(lib, s), s
    assert lib.tqec_version().startswith(b"tqec-gb300")


def _graph(pkg, code, p=0.05):
    t = pkg.tanner_graph(code)
    em = pkg.depolarizing(p, t.nq)
    lx, lz = pkg.logical_operator(t)
    return t, em, pkg.tnmmap_css_graph(t, em, lx, lz)


def test_optimizer_returns_valid_tree(pkg):
    _, _, g = _graph(pkg, pkg.SurfaceCode(5, 5))
    steps, lm, w = pkg.native.optimize_order(g, trials=4, sweeps=50)
    n = g.n_tensors
    used = set()
    for s, (a, b) in enumerate(steps):
        assert 0 <= a < n + s and 0 <= b < n + s and a != b
        assert a not in used and b not in used
        used |= {int(a), int(b)}
    assert len(used) == 2 * n - 2
    assert 10 < lm < 20 and w <= 12


@pytest.mark.parametrize("code,nsyn", [("s3", 64), ("s5", 24), ("s7", 3), ("t3", 8), ("c488", 16),
                                       ("c666", 16)])
def test_plan_emulation_matches_oracle(pkg, oracle, code, nsyn):
    codes = {"s3": (pkg.SurfaceCode(3, 3), lambda: oracle.surface_code_stabilizers(3, 3)),
             "s5": (pkg.SurfaceCode(5, 5), lambda: oracle.surface_code_stabilizers(5, 5)),
             "s7": (pkg.SurfaceCode(7, 7), lambda: oracle.surface_code_stabilizers(7, 7)),
             "t3": (pkg.ToricCode(3, 3), lambda: oracle.toric_code_stabilizers(3, 3)),
             "c488": (pkg.Color488(5), lambda: oracle.color_code_stabilizers("488", 5)),
             "c666": (pkg.Color666(5), lambda: oracle.color_code_stabilizers("666", 5))}
    c, ofn = codes[code]
    t, em, g = _graph(pkg, c, 0.08)
    steps = pkg.optimize_code(g, pkg.TreeSA(trials=4, sweeps=200))
    plan = pkg.native.inspect_plan(g, steps)
    rng = np.random.default_rng(11)
    ep = pkg.random_error_pattern(em, rng, nsamples=nsyn)
    syn = pkg.syndrome_extraction(ep, t)
    bits = np.concatenate([syn.sx, syn.sz], axis=1)
    got = run_plan(plan, bits)
    assert not np.isnan(got).any()
    st, nq = ofn()
    dec = oracle.OracleDecoder(oracle.css_tanner(st, nq), em.px, em.py, em.pz)
    want = dec.marginals(bits)
    np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-12 * want.max())


def test_level_ordered_plan_emulation_matches_oracle(pkg, oracle):
    """The plain form's level-by-level plan (TQEC_FLAG_PLAIN, width >= 12:
    steps reordered, more steps per barrier group, a different arena) computes
    the same marginals as the oracle."""
    t, em, g = _graph(pkg, pkg.SurfaceCode(7, 7), 0.08)
    steps = pkg.optimize_code(g, pkg.TreeSA(trials=4, sweeps=200))
    batch = pkg.native.inspect_plan(g, steps)
    plan = pkg.native.inspect_plan(g, steps, pkg.native.TQEC_FLAG_PLAIN)
    assert plan["width"] >= 12 and plan["arena_elems"] != batch["arena_elems"]
    rng = np.random.default_rng(13)
    ep = pkg.random_error_pattern(em, rng, nsamples=3)
    syn = pkg.syndrome_extraction(ep, t)
    bits = np.concatenate([syn.sx, syn.sz], axis=1)
    got = run_plan(plan, bits)
    st, nq = oracle.surface_code_stabilizers(7, 7)
    want = oracle.OracleDecoder(oracle.css_tanner(st, nq), em.px, em.py, em.pz).marginals(bits)
    np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-12 * want.max())


def test_plan_emulation_dem(pkg, oracle):
    import json

    text = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_kat.json")))["dem_small"]["text"]
    dem = pkg.parse_dem_string(text)
    g = pkg.tnmmap_dem_graph(pkg.dem2tanner(dem), pkg.logical_map(dem), dem.error_rates, 1, True)
    steps = pkg.optimize_code(g, pkg.TreeSA(trials=4, sweeps=100))
    plan = pkg.native.inspect_plan(g, steps)
    bits = ((np.arange(64)[:, None] >> np.arange(6)[None, :]) & 1).astype(np.uint8)
    got = run_plan(plan, bits)
    dec = oracle.OracleDEMDecoder(oracle.parse_dem_string(text))
    want = dec.marginals(bits)
    np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-300)


def test_plan_no_optimizer_order(pkg, oracle):
    """NoOptimizer (tndecoder.jl:64) contracts left to right; on the Steane
    code that folds wide syndrome-independent prefixes on the host."""
    code = pkg.SteaneCode()
    t, em, g = _graph(pkg, code)
    steps = pkg.optimize_code(g, pkg.NoOptimizer())
    plan = pkg.native.inspect_plan(g, steps)
    ns = t.ns
    bits = ((np.arange(1 << ns)[:, None] >> np.arange(ns)[None, :]) & 1).astype(np.uint8)
    got = run_plan(plan, bits)
    ot = oracle.css_tanner([(s_.kind() == 1 and "X" or "Z", tuple(s_.support())) for s_ in pkg.stabilizers(code)], 7)
    lx, lz = oracle.logical_operator(ot)
    brute = oracle.brute_force_marginals(ot, em.px, em.py, em.pz, lx, lz)
    np.testing.assert_allclose(got, brute, rtol=1e-12, atol=1e-300)


def test_zero_syndrome_kat_through_plan(pkg):
    """test/decoding/tndecoder.jl:101-110 through the planner's program."""
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    em = pkg.iid_error(0.1, 0.0, 0.0, 9)
    lx, lz = pkg.logical_operator(t)
    g = pkg.tnmmap_css_graph(t, em, lx, lz)
    plan = pkg.native.inspect_plan(g, pkg.optimize_code(g, pkg.TreeSA(trials=2, sweeps=10)))
    got = run_plan(plan, np.zeros((1, 8), dtype=np.uint8))[0]
    np.testing.assert_allclose(got, [0.3972875040000002, 0.0, 0.004284496000000001, 0.0], atol=1e-10)


def test_invalid_inputs_return_status(pkg):
    t, em, g = _graph(pkg, pkg.SurfaceCode(3, 3))
    steps = pkg.optimize_code(g, pkg.GreedyMethod())
    bad = steps.copy()
    bad[0, 0] = bad[0, 1]
    with pytest.raises(pkg.native.TqecError) as e:
        pkg.native.inspect_plan(g, bad)
    assert e.value.code == -1
    with pytest.raises(pkg.native.TqecError):
        pkg.native.inspect_plan(g, steps[:-1])
    g2 = pkg.FactorGraph(list(g.ixs), list(g.tensors), list(g.iy), list(g.syndrome_positions))
    g2.tensors[0] = np.ones(3)
    with pytest.raises(pkg.native.TqecError) as e:
        pkg.native.inspect_plan(g2, steps)
    assert e.value.code == -4
    assert "2^rank" in pkg.native.last_error()
    lib = pkg.native.lib()
    assert lib.tqec_program_create(None, None, None, None) == -1
    assert lib.tqec_decode_batch(None, None, 0, None, None, None, None) == -1


def test_plan_emulation_tensor_steps(pkg):
    """A circuit-level model (rotated Z-memory d=5, 2 rounds) whose program
    has GEMM-shaped steps (B laid out K-major): the emulated program agrees
    with the C contractor of the oracle on the same tree."""
    from oracle.c_oracle import CContractor
    from tensorqec_gb300 import circuit, dem as demmod

    dm = circuit.detector_error_model(circuit.memory_z_circuit(5, 2, 0.001))
    t = demmod.dem2tanner(dm)
    g = pkg.tnmmap_dem_graph(t, demmod.logical_map(dm), dm.error_rates, len(dm.logical_list), True)
    steps = pkg.optimize_code(g, pkg.TreeSA(trials=16, sweeps=1000, seed=1, restarts=2))
    plan = pkg.native.inspect_plan(g, steps)
    assert any(int(d["flags"]) & 8 for d in plan["steps"]), "expected GEMM-shaped steps"
    rng = np.random.default_rng(5)
    _, det, _ = demmod.sample_dem(dm, 2, rng)
    got = run_plan(plan, det)
    cc = CContractor(g.ixs, [np.asarray(x) for x in g.tensors], g.iy, g.syndrome_positions, steps)
    marg, _ = cc.contract(pkg.pack_syndromes(det))
    want = marg
    np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-300)


def test_tensor_steps_need_a_share_of_the_work(pkg):
    """GEMM-shaped steps are planned for the tensor cores only when they hold
    at least a quarter of the multiply-adds: the surface code d=9 program on
    the default tree search's order (one such step, about 5% of the work) is
    planned without them, the circuit-level
    d=5 program keeps them; the no-tensor-cores flag plans none."""
    from tensorqec_gb300 import circuit, dem as demmod, gf2
    from tensorqec_gb300.network import tnmmap_css_graph

    def share(plan):
        m = np.array([1 << int(d["lh"] + d["lfa"] + d["lfb"] + d["lk"]) for d in plan["steps"]], dtype=np.float64)
        tc = np.array([int(d["flags"]) & 8 != 0 for d in plan["steps"]])
        return m[tc].sum() / m.sum()

    t = pkg.tanner_graph(pkg.SurfaceCode(9, 9))
    em = pkg.depolarizing(0.05, t.nq)
    lx, lz = gf2.logical_operator(t)
    g9 = tnmmap_css_graph(t, em, lx, lz)
    s9 = pkg.optimize_code(g9, pkg.TreeSA())
    assert share(pkg.native.inspect_plan(g9, s9)) == 0.0

    dm = circuit.detector_error_model(circuit.memory_z_circuit(5, 2, 0.001))
    tg = demmod.dem2tanner(dm)
    g = pkg.tnmmap_dem_graph(tg, demmod.logical_map(dm), dm.error_rates, len(dm.logical_list), True)
    steps = pkg.optimize_code(g, pkg.TreeSA(trials=16, sweeps=1000, seed=1, restarts=2))
    assert share(pkg.native.inspect_plan(g, steps)) >= 0.25
    assert share(pkg.native.inspect_plan(g, steps, pkg.native.TQEC_FLAG_NO_TENSOR_CORES)) == 0.0


def test_tensor_aware_order_search(pkg):
    """TreeSA(tensor_discount=D): GEMM-shaped steps cost D times fewer
    multiply-adds in the search, which trades flops for tensor-core work: at
    surface d=7 the default search plans no tensor-core step, a discount of 4
    puts most of the multiply-adds on them (at more flops), and the tree stays
    a valid contraction of the network."""
    from tensorqec_gb300 import gf2
    from tensorqec_gb300.network import tnmmap_css_graph

    def share(plan):
        m = np.array([1 << int(d["lh"] + d["lfa"] + d["lfb"] + d["lk"]) for d in plan["steps"]], dtype=np.float64)
        tc = np.array([int(d["flags"]) & 8 != 0 for d in plan["steps"]])
        return m[tc].sum() / m.sum()

    t = pkg.tanner_graph(pkg.SurfaceCode(7, 7))
    lx, lz = gf2.logical_operator(t)
    g = tnmmap_css_graph(t, pkg.depolarizing(0.05, t.nq), lx, lz)
    plain = pkg.native.inspect_plan(g, pkg.optimize_code(g, pkg.TreeSA(trials=16, sweeps=1000, restarts=2)))
    steps = pkg.optimize_code(g, pkg.TreeSA(trials=16, sweeps=1000, restarts=2, tensor_discount=4.0))
    tensor = pkg.native.inspect_plan(g, steps)
    assert share(plain) == 0.0
    assert share(tensor) >= 0.5
    assert tensor["flops_per_syndrome"] > plain["flops_per_syndrome"]
    # a valid tree: every node id used once, n - 1 steps
    ids = np.asarray(steps).ravel()
    assert len(steps) == g.n_tensors - 1 and len(np.unique(ids)) == len(ids)
