"""Invariants of the compiled contraction program that the numpy emulator
cannot see, checked on the CPU for many programs.

The emulator runs the steps one after another, but the CUDA kernel runs all
steps of a barrier group (the steps up to one whose sync flag is set)
concurrently, and it trusts every offset the planner wrote.  So for every
program this test checks, from the step records alone:

* bounds: every arena range, constant variant, syndrome bit and permutation
  table a step touches lies inside the program's arena, constant and
  permutation arrays, and permutation tables start on 8-entry boundaries (the
  kernel reads them as 16-byte vectors);
* the tree: an arena operand is the whole output of an earlier step in an
  earlier barrier group, and every step's output except the root's is read
  exactly once;
* permutations: a step's output table maps its 2^width outputs one-to-one
  onto its output range;
* no race: while an intermediate is live (from its producer's group through
  its consumer's group; to the end in MAP mode, whose back-tracking reads
  every intermediate again) no other step writes into its range — which also
  makes the outputs of one barrier group pairwise disjoint;
* tensor-core steps have the GEMM shape the tcgen05 path requires and read
  only arena tensors or unselected constants.
"""
import numpy as np
import pytest

from plan_emulator import OP_ARENA, OP_CONST, OP_PARITY, _perm_addr

SYNC, TENSOR = 1, 8


def _perm_entries(lw):
    n, sh = 0, 0
    while sh < lw:
        n += 1 << min(8, lw - sh)
        sh += 8
    return n


def check_plan(plan):
    steps = plan["steps"]
    R = len(steps)
    arena = int(plan["arena_elems"])
    nconst, nperm, nsyn = len(plan["consts"]), len(plan["perm"]), int(plan["n_syndrome"])
    maxp = plan.get("map_mode", False)
    assert R >= 1 and int(steps[-1]["flags"]) & SYNC
    group = np.zeros(R, dtype=np.int64)
    g = 0
    for r, d in enumerate(steps):
        group[r] = g
        if int(d["flags"]) & SYNC:
            g += 1
    lo = np.array([int(d["out_off"]) for d in steps], dtype=np.int64)
    hi = lo + np.array([1 << int(d["lh"] + d["lfa"] + d["lfb"]) for d in steps], dtype=np.int64)
    assert (lo >= 0).all() and (hi <= arena).all(), "output outside the arena"
    consumer = np.full(R, -1, dtype=np.int64)
    for r, d in enumerate(steps):
        lh, lfa, lfb, lk = (int(d[x]) for x in ("lh", "lfa", "lfb", "lk"))
        flags = int(d["flags"])
        for side, size_bits in (("a", lh + lfa + lk), ("b", lh + lk + lfb)):
            kind, ref, prod = int(d[side + "_kind"]), int(d[side + "_ref"]), int(d[side + "_prod"])
            sel = [int(s) for s in d[side + "_sel"]]
            if kind == OP_ARENA:
                assert 0 <= prod < r, (r, side, prod)
                assert group[prod] < group[r], f"step {r} reads step {prod} of its own barrier group"
                assert ref == lo[prod] and hi[prod] - lo[prod] == 1 << size_bits, (r, side)
                assert consumer[prod] < 0, f"step {prod} is read twice"
                consumer[prod] = r
            elif kind == OP_CONST:
                used = [i for i, s in enumerate(sel) if s >= 0]
                assert all(0 <= sel[i] < nsyn for i in used)
                vmax = (1 << (max(used) + 1)) - 1 if used else 0
                assert ref >= 0 and ref + (vmax << size_bits) + (1 << size_bits) <= nconst, (r, side)
            else:
                assert kind == OP_PARITY and 0 <= ref < nsyn, (r, side, kind, ref)
            if flags & TENSOR:
                assert kind == OP_ARENA or (kind == OP_CONST and all(s < 0 for s in sel)), (r, side)
        if flags & TENSOR:
            assert lfa >= 7 and lfb >= 5 and lk >= 5, (r, lfa, lfb, lk)
        po = int(d["perm_off"])
        if po >= 0:
            lw = lh + lfa + lfb
            assert po % 8 == 0 and po + _perm_entries(lw) <= nperm, (r, po)
            addr = _perm_addr(plan["perm"].astype(np.int64), po, np.arange(1 << lw, dtype=np.int64), lw)
            assert np.array_equal(np.sort(addr), np.arange(1 << lw)), f"step {r}: output table is not a permutation"
    assert consumer[R - 1] < 0
    assert (consumer[:R - 1] >= 0).all(), "an intermediate is never read"
    last = group[-1]
    for r in range(R):
        end = last if (maxp or r == R - 1) else group[consumer[r]]
        window = (group >= group[r]) & (group <= end)
        window[r] = False
        clash = window & (lo < hi[r]) & (hi > lo[r])
        assert not clash.any(), f"step {np.flatnonzero(clash)[0]} writes over step {r}'s live output"


def _css_plan(pkg, code, optimizer, flags=0, p=0.05):
    t = pkg.tanner_graph(code)
    em = pkg.depolarizing(p, t.nq)
    lx, lz = pkg.logical_operator(t)
    g = pkg.tnmmap_css_graph(t, em, lx, lz)
    return pkg.native.inspect_plan(g, pkg.optimize_code(g, optimizer), flags)


CSS = [("surface3", lambda p: p.SurfaceCode(3, 3)), ("surface5", lambda p: p.SurfaceCode(5, 5)),
       ("surface7", lambda p: p.SurfaceCode(7, 7)), ("toric3", lambda p: p.ToricCode(3, 3)),
       ("toric4", lambda p: p.ToricCode(4, 4)), ("color488_5", lambda p: p.Color488(5)),
       ("color666_5", lambda p: p.Color666(5)), ("steane", lambda p: p.SteaneCode())]


@pytest.mark.parametrize("name,make", CSS, ids=[c[0] for c in CSS])
@pytest.mark.parametrize("opt", ["treesa", "treesa_seed7", "greedy"])
def test_css_programs(pkg, name, make, opt):
    o = {"treesa": pkg.TreeSA(trials=4, sweeps=200, restarts=1),
         "treesa_seed7": pkg.TreeSA(trials=4, sweeps=200, restarts=1, seed=7),
         "greedy": pkg.GreedyMethod()}[opt]
    check_plan(_css_plan(pkg, make(pkg), o))


def test_left_to_right_programs(pkg):
    """NoOptimizer (tndecoder.jl:64): wide prefixes folded on the host."""
    for code in (pkg.SteaneCode(), pkg.SurfaceCode(3, 3)):
        check_plan(_css_plan(pkg, code, pkg.NoOptimizer()))


def test_surface9_and_no_tensor_cores(pkg):
    code = pkg.SurfaceCode(9, 9)
    for flags in (0, pkg.native.TQEC_FLAG_NO_TENSOR_CORES):
        check_plan(_css_plan(pkg, code, pkg.TreeSA(trials=4, sweeps=300, restarts=1), flags))


def test_dem_programs_with_tensor_steps(pkg):
    """The reference's dem.dem fixture and a circuit-level d=5, 2-round
    model whose program has GEMM-shaped (tensor-core) steps."""
    import json
    import os

    from tensorqec_gb300 import circuit, dem as demmod

    root = os.path.dirname(os.path.abspath(__file__))
    text = json.load(open(os.path.join(root, "golden", "reference_kat.json")))["dem_small"]["text"]
    dem = pkg.parse_dem_string(text)
    g = pkg.tnmmap_dem_graph(pkg.dem2tanner(dem), pkg.logical_map(dem), dem.error_rates, 1, True)
    check_plan(pkg.native.inspect_plan(g, pkg.optimize_code(g, pkg.TreeSA(trials=4, sweeps=100))))

    dm = circuit.detector_error_model(circuit.memory_z_circuit(5, 2, 0.001))
    t = demmod.dem2tanner(dm)
    g = pkg.tnmmap_dem_graph(t, demmod.logical_map(dm), dm.error_rates, len(dm.logical_list), True)
    steps = pkg.optimize_code(g, pkg.TreeSA(trials=16, sweeps=1000, seed=1, restarts=2))
    plan = pkg.native.inspect_plan(g, steps)
    assert any(int(d["flags"]) & TENSOR for d in plan["steps"])
    check_plan(plan)
    check_plan(pkg.native.inspect_plan(g, steps, pkg.native.TQEC_FLAG_NO_TENSOR_CORES))


@pytest.mark.parametrize("d", [3, 5])
def test_map_programs(pkg, d):
    """TNMAP programs keep every intermediate for the back-tracking."""
    from tensorqec_gb300 import decoder, native, network

    t = pkg.tanner_graph(pkg.SurfaceCode(d, d))
    general, ixs, ts = network.reduce2general(t, pkg.iid_error(0.05, 0.06, 0.1, t.nq))
    graph = network.tnmap_graph(general, ixs, ts)
    plan = native.inspect_plan(graph, decoder.optimize_code(graph, decoder.TreeSA(restarts=1)), native.TQEC_FLAG_MAP)
    assert plan["map_mode"]
    check_plan(plan)


def test_invariants_catch_planted_faults(pkg):
    """Each planted fault in a copy of a valid program is reported."""
    plan = _css_plan(pkg, pkg.SurfaceCode(5, 5), pkg.TreeSA(trials=4, sweeps=200, restarts=1))
    check_plan(plan)
    steps = plan["steps"]
    reads = [r for r, d in enumerate(steps) if int(d["a_kind"]) == OP_ARENA]
    r = reads[len(reads) // 2]
    prod = int(steps[r]["a_prod"])

    def faulty(mutate):
        p = dict(plan, steps=plan["steps"].copy())
        mutate(p)
        with pytest.raises(AssertionError):
            check_plan(p)

    # a consumer moved into its producer's barrier group
    def same_group(p):
        for q in range(prod, r):
            p["steps"][q]["flags"] &= ~SYNC
    faulty(same_group)

    # another step writing over a live operand
    def clobber(p):
        other = next(q for q in range(prod + 1, r + 1) if q != prod)
        p["steps"][other]["out_off"] = p["steps"][prod]["out_off"]
    faulty(clobber)

    # an output running past the arena
    def overflow(p):
        p["arena_elems"] = int(max(int(d["out_off"]) + (1 << int(d["lh"] + d["lfa"] + d["lfb"]))
                                   for d in p["steps"])) - 1
    faulty(overflow)

    # a permutation table that is not one-to-one
    permuted = [q for q, d in enumerate(steps) if int(d["perm_off"]) >= 0]
    if permuted:
        q = permuted[0]

        def bad_perm(p):
            p["perm"] = p["perm"].copy()
            p["perm"][int(p["steps"][q]["perm_off"]) + 1] = p["perm"][int(p["steps"][q]["perm_off"])]
        faulty(bad_perm)


def test_benchmark_d7_program(pkg):
    """The d=7 program of the benchmark's order search (the workload of the
    headline number), with its emulated marginals against the C contractor."""
    from oracle.c_oracle import CContractor
    from plan_emulator import run_plan

    t = pkg.tanner_graph(pkg.SurfaceCode(7, 7))
    em = pkg.depolarizing(0.05, t.nq)
    lx, lz = pkg.logical_operator(t)
    g = pkg.tnmmap_css_graph(t, em, lx, lz)
    steps = pkg.optimize_code(g, pkg.TreeSA(trials=128, sweeps=8000, restarts=8, seed=2))
    plan = pkg.native.inspect_plan(g, steps)
    check_plan(plan)
    rng = np.random.default_rng(3)
    ep = pkg.random_error_pattern(em, rng, nsamples=4)
    s = pkg.syndrome_extraction(ep, t)
    bits = np.concatenate([s.sx, s.sz], axis=1)
    cc = CContractor(g.ixs, [np.asarray(x) for x in g.tensors], g.iy, g.syndrome_positions, steps)
    want, _ = cc.contract(pkg.pack_syndromes(bits))
    np.testing.assert_allclose(run_plan(plan, bits), want, rtol=1e-10, atol=1e-300)
