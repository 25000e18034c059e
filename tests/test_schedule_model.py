"""A CPU model of how the contraction kernel spreads a step over a block.

It restates the kernels' step-shape choice (several lanes per output, eight
or four outputs per work item, or one), its per-warp entry test, the
rotation of barrier-group members over the block and the per-syndrome loop
of multi-syndrome blocks (csrc/contract.cu: step_shape, the step loop of
tn_contract_kernel, run_step*, run_step_splitk, run_step_vsplit), and the
cluster form's plans (fill_step_plan: lanes sharing four-output items, small
barrier groups on the first block alone), and checks on real programs that
every output of every syndrome of every step is written exactly once for each
launch shape the autotuner may pick.
"""
import numpy as np
import pytest


def step_shape(lh, lfa, lfb, lk, lg, bd, is_float, flags=0, vsplit=False):
    """SIMT shapes (a tensor-core step covers its outputs tile by tile)."""
    lw = lh + lfa + lfb
    outs = 1 << (lw + lg)
    lt = 0
    while lt < 5 and (outs << (lt + 1)) <= bd and (lt + 1) + 2 <= lk:
        lt += 1
    if lt >= 2:
        kind, total = "splitk", outs << lt
    elif flags & 8:  # K-major B: no vector loads along fb
        kind, total = "scalar", outs
    elif is_float and lfb >= 3 and (outs >> 3) >= bd:
        kind, total = "vec8", outs >> 3
    elif lfb >= 2:
        vl = 0
        while vsplit and vl < 3 and ((outs >> 2) << (vl + 1)) <= bd and lk - (vl + 1) >= 2:
            vl += 1
        kind, total, lt = ("vsplit" if vl else "vec4"), (outs >> 2) << vl, vl
    else:
        kind, total = "scalar", outs
    return kind, lt, (total + 31) & ~31


def _run(kind, lt, lw, lg, one, bd, item_base, enter, cover, gbase):
    """Marks the outputs the block's threads write for one step (one
    syndrome when `one`, else all G of the block)."""
    tid = np.arange(bd)
    vt = (tid + bd - item_base % bd) % bd
    warp_vt = ((tid & ~31) + bd - item_base % bd) % bd
    vt = vt[warp_vt < enter]
    lwg = lw + (0 if one else lg)
    if kind == "splitk":
        total = (1 << lwg) << lt
        tr = (total + 31) & ~31
        for v in vt:
            for x in range(v, tr, bd):
                if x < total and (x & ((1 << lt) - 1)) == 0:
                    item = x >> lt
                    g = 0 if one else item >> lw
                    cover[gbase + g, item & ((1 << lw) - 1)] += 1
        return
    if kind == "vsplit":  # one syndrome: 2^lt lanes per four outputs
        total = (1 << (lw - 2)) << lt
        tr = (total + 31) & ~31
        for v in vt:
            for x in range(v, tr, bd):
                if x < total and (x & ((1 << lt) - 1)) == 0:
                    e0 = (x >> lt) << 2
                    cover[gbase, e0:e0 + 4] += 1
        return
    lv = {"vec8": 3, "vec4": 2, "scalar": 0}[kind]
    lwv = lw - lv
    total = 1 << (lwv + (0 if one else lg))
    stop = total if one else (total + 31) & ~31
    for v in vt:
        for i in range(v, stop, bd):
            if i < total:
                g = 0 if one else i >> lwv
                e0 = (i & ((1 << lwv) - 1)) << lv
                cover[gbase + g, e0:e0 + (1 << lv)] += 1


def check_program(plan, is_float, vsplit=False):
    bad = []
    for G in ((1,) if vsplit else (1, 2, 4, 8)):
        lg = G.bit_length() - 1
        # blocks, and for one syndrome the teams of 2-16-block clusters of
        # 256 or 512 threads (the cluster kernel numbers them rank-major)
        for bd in (128, 256, 512, 1024) + ((2048, 4096, 8192) if G == 1 else ()):
            if not is_float and 512 < bd <= 1024:
                continue
            item_base = 0
            for st, d in enumerate(plan["steps"]):
                lh, lfa, lfb, lk = int(d["lh"]), int(d["lfa"]), int(d["lfb"]), int(d["lk"])
                lw = lh + lfa + lfb
                fl = int(d["flags"])
                kind, lt, tr = step_shape(lh, lfa, lfb, lk, lg, bd, is_float, fl, vsplit)
                k1, lt1, tr1 = step_shape(lh, lfa, lfb, lk, 0, bd, is_float, fl, vsplit)
                per_syndrome = G > 1 and tr1 >= bd
                enter = bd if per_syndrome else tr
                cover = np.zeros((G, 1 << lw), dtype=np.int64)
                if G == 1:
                    _run(kind, lt, lw, 0, True, bd, item_base, enter, cover, 0)
                elif per_syndrome:
                    for g in range(G):
                        _run(k1, lt1, lw, 0, True, bd, item_base, enter, cover, g)
                else:
                    _run(kind, lt, lw, lg, False, bd, item_base, enter, cover, 0)
                if not (cover == 1).all():
                    bad.append((G, bd, st, kind, int(cover.min()), int(cover.max())))
                item_base = 0 if int(d["flags"]) & 1 else item_base + enter
    return bad


def check_cluster_program(plan, is_float, blocks, threads, opts=None):
    """The cluster form (one syndrome per cluster of `blocks` blocks): every
    output written once, and a group planned for the first block alone keeps
    all its items on that block's threads.  `opts`: per-step options the
    autotuner may set (1 no shared items, 2 never on the first block alone,
    4 on the first block whenever the items fit)."""
    steps = plan["steps"]
    n = len(steps)
    sync = [bool(int(d["flags"]) & 1) for d in steps]
    team = blocks * threads

    opts = np.zeros(n, dtype=np.int64) if opts is None else np.asarray(opts)

    def shape(d, bd, st=None):
        share = st is None or not (opts[st] & 1)
        return step_shape(int(d["lh"]), int(d["lfa"]), int(d["lfb"]), int(d["lk"]), 0, bd, is_float,
                          int(d["flags"]), vsplit=share)

    groups, s0 = [], 0
    for st in range(n):
        if sync[st] or st == n - 1:
            groups.append((s0, st))
            s0 = st + 1
    def k_per_lane(d, sh):
        kind, lt, _ = sh
        return (1 << int(d["lk"])) >> lt if kind in ("splitk", "vsplit") else 1 << int(d["lk"])

    bad = []
    for s0, s1 in groups:
        rng = range(s0, s1 + 1)
        solo = (sum(shape(steps[s], threads, s)[2] for s in rng) <= threads and
                not any(opts[s] & 2 for s in rng) and
                all((opts[s] & 4) or k_per_lane(steps[s], shape(steps[s], threads, s)) <=
                    max(8, k_per_lane(steps[s], shape(steps[s], team, s))) for s in rng))
        bd = threads if solo else team
        item_base = 0
        for st in range(s0, s1 + 1):
            d = steps[st]
            lw = int(d["lh"]) + int(d["lfa"]) + int(d["lfb"])
            kind, lt, tr = shape(d, bd, st)
            cover = np.zeros((1, 1 << lw), dtype=np.int64)
            _run(kind, lt, lw, 0, True, bd, item_base, tr, cover, 0)
            if not (cover == 1).all():
                bad.append((blocks, threads, st, kind, solo, int(cover.min()), int(cover.max())))
            item_base += tr
        if solo and item_base > threads:
            bad.append((blocks, threads, s0, "solo group exceeds the first block", item_base))
    return bad


@pytest.mark.parametrize("code", ["surface5", "color488_5", "surface7"])
def test_every_output_written_once(pkg, code):
    from tensorqec_gb300 import decoder, gf2, network, native
    c = {"surface5": lambda: pkg.SurfaceCode(5, 5), "color488_5": lambda: pkg.Color488(5),
         "surface7": lambda: pkg.SurfaceCode(7, 7)}[code]()
    t = pkg.tanner_graph(c)
    em = pkg.depolarizing(0.05, t.nq)
    lx, lz = gf2.logical_operator(t)
    graph = network.tnmmap_css_graph(t, em, lx, lz)
    steps = decoder.optimize_code(graph, decoder.TreeSA(restarts=1))
    plan = native.inspect_plan(graph, steps)
    for is_float in (True, False):
        assert check_program(plan, is_float) == []
        # one syndrome per block with lanes sharing four-output items
        assert check_program(plan, is_float, vsplit=True) == []


@pytest.mark.parametrize("code", ["surface7", "color488_5"])
def test_cluster_plans_write_every_output_once(pkg, code):
    from tensorqec_gb300 import decoder, gf2, network, native
    c = {"color488_5": lambda: pkg.Color488(5), "surface7": lambda: pkg.SurfaceCode(7, 7)}[code]()
    t = pkg.tanner_graph(c)
    em = pkg.depolarizing(0.05, t.nq)
    lx, lz = gf2.logical_operator(t)
    graph = network.tnmmap_css_graph(t, em, lx, lz)
    steps = decoder.optimize_code(graph, decoder.TreeSA(restarts=1))
    kinds = set()
    # the batch plan (the recheck's) and the plain form's level-by-level plan
    rng = np.random.default_rng(3)
    for flags in (0, native.TQEC_FLAG_PLAIN):
        plan = native.inspect_plan(graph, steps, flags)
        for blocks, threads in ((2, 128), (4, 256), (8, 256), (16, 128), (16, 256), (8, 512)):
            assert check_cluster_program(plan, False, blocks, threads) == []
            # options the per-group tuning may set
            for _ in range(3):
                opts = rng.integers(0, 8, size=len(plan["steps"]))
                assert check_cluster_program(plan, False, blocks, threads, opts) == []
            for d in plan["steps"]:
                kinds.add(step_shape(int(d["lh"]), int(d["lfa"]), int(d["lfb"]), int(d["lk"]), 0, blocks * threads,
                                     False, int(d["flags"]), vsplit=True)[0])
    assert "vsplit" in kinds


def test_plain_wide_plans_run_level_by_level(pkg):
    """A wide TQEC_FLAG_PLAIN program orders its steps by level: no step
    shares a barrier group with a step whose output it reads, and the
    groups are fewer than the batch plan's."""
    from tensorqec_gb300 import decoder, gf2, network, native
    t = pkg.tanner_graph(pkg.SurfaceCode(7, 7))
    em = pkg.depolarizing(0.05, t.nq)
    lx, lz = gf2.logical_operator(t)
    graph = network.tnmmap_css_graph(t, em, lx, lz)
    steps = decoder.optimize_code(graph, decoder.TreeSA(restarts=1))
    batch = native.inspect_plan(graph, steps)
    plain = native.inspect_plan(graph, steps, native.TQEC_FLAG_PLAIN)
    assert plain["width"] >= 12 and len(plain["steps"]) == len(batch["steps"])
    groups = lambda pl: int(sum(int(d["flags"]) & 1 for d in pl["steps"]))
    assert groups(plain) < groups(batch)
    # every arena operand comes from an earlier barrier group
    gid, g = [], 0
    for d in plain["steps"]:
        gid.append(g)
        g += int(d["flags"]) & 1
    for i, d in enumerate(plain["steps"]):
        for kind, prod in ((int(d["a_kind"]), int(d["a_prod"])), (int(d["b_kind"]), int(d["b_prod"]))):
            if kind == 0:
                assert 0 <= prod < i and gid[prod] < gid[i]
