"""Malformed networks and trees through the C ABI's host entry points (no
GPU): the planner (tqec_plan_inspect_flags) and the order search
(tqec_optimize_order) must answer every input that stays inside the arrays
it is given with a status code — never a crash — and every program they
accept must satisfy the compiled-program invariants.

Each case mutates one field of a valid d=3 surface-code TNMMAP network or
its tree: node ids of the tree (out of range, reused, self-merged, forward
references), the step count, labels (non-positive, repeated inside a tensor),
tensor sizes, syndrome-leaf positions (out of range, repeated, on a
multi-label tensor), output labels (absent, repeated, NULL).  The cases run
in a child process, so a crash fails the test instead of ending the run.
"""
import os
import subprocess
import sys
import textwrap

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent(r'''
    import ctypes as C, os, sys
    import numpy as np
    sys.path.insert(0, ROOT); sys.path.insert(0, os.path.join(ROOT, "tests"))
    import __graft_entry__ as G
    from test_plan_invariants import check_plan
    pkg = G.load_package()
    nat = pkg.native
    lib = nat.lib()

    def flat(g):
        return [np.array(a, copy=True) for a in g.flat()]

    def run(arrays, n_tensors, steps, n_steps, flags=0, n_out=None, out_null=False):
        ix_off, labels, d_off, data, iy, synd = arrays
        net = nat.Network(n_tensors, nat._ptr(ix_off), nat._ptr(labels), nat._ptr(d_off), nat._ptr(data),
                          len(iy) if n_out is None else n_out, None if out_null else nat._ptr(iy),
                          len(synd), nat._ptr(synd))
        steps = np.ascontiguousarray(steps, dtype=np.int32)
        tree = nat.Tree(n_steps, nat._ptr(steps))
        view = nat.PlanView()
        h = C.c_void_p()
        rc = lib.tqec_plan_inspect_flags(C.byref(net), C.byref(tree), flags, C.byref(view), C.byref(h))
        if rc == 0:
            lib.tqec_plan_release(h)
        out = np.zeros(max(n_tensors - 1, 0) * 2 + 2, dtype=np.int32)
        lm, w = C.c_double(0), C.c_int32(0)
        o = nat.OrderOptions(2, 20, 0, 1.0, 1)
        rc2 = lib.tqec_optimize_order(C.byref(net), C.byref(o), nat._ptr(out), C.byref(lm), C.byref(w))
        return rc, rc2

    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    em = pkg.depolarizing(0.05, t.nq)
    lx, lz = pkg.logical_operator(t)
    g = pkg.tnmmap_css_graph(t, em, lx, lz)
    base = flat(g)
    T = g.n_tensors
    steps = pkg.optimize_code(g, pkg.GreedyMethod())
    rng = np.random.default_rng(5)
    n_cases = n_ok = 0

    def case(arrays=None, st=None, n_steps=None, expect_fail=True, **kw):
        global n_cases, n_ok
        arrays = base if arrays is None else arrays
        st = steps if st is None else st
        rc, rc2 = run(arrays, T, st, len(st) if n_steps is None else n_steps, **kw)
        n_cases += 1
        assert rc <= 0 and rc2 <= 0, (rc, rc2)
        if expect_fail:
            assert rc < 0, "malformed input accepted"
        if rc == 0:
            n_ok += 1

    # the tree
    for _ in range(300):
        st = steps.copy()
        s, side = rng.integers(len(st)), rng.integers(2)
        st[s, side] = rng.integers(-3, T + len(st) + 3)
        rc, _ = run(base, T, st, len(st))
        n_cases += 1
        assert rc <= 0
        if rc == 0:
            plan = nat.inspect_plan(g, st)
            check_plan(plan)
            n_ok += 1
    st = steps.copy(); st[3, 1] = st[3, 0]; case(st=st)                      # self-merge
    st = steps.copy(); st[5] = st[4]; case(st=st)                            # a node used twice
    st = steps.copy(); st[0, 0] = T + 3; case(st=st)                         # forward reference
    case(st=steps[:-1])                                                     # too few steps
    case(st=np.concatenate([steps, steps[:1]]))                             # too many steps
    case(n_steps=-1)
    # labels
    for v in (0, -5):
        a = flat(g); a[1][7] = v; case(arrays=a)
    a = flat(g); lo, hi = a[0][0], a[0][1]; a[1][lo + 1] = a[1][lo]; case(arrays=a)   # repeated label
    # tensor sizes: move one boundary so a tensor has 2^rank - 1 entries
    a = flat(g); a[2][1] -= 1; case(arrays=a)
    # syndrome leaves
    for bad in (-1, T, T + 100):
        a = flat(g); a[5][0] = bad; case(arrays=a)
    a = flat(g); a[5][1] = a[5][0]; case(arrays=a)                         # listed twice
    a = flat(g); a[5][0] = 0; case(arrays=a)                               # a parity tensor
    # output labels
    a = flat(g); a[4][0] = 10 ** 6; case(arrays=a)                         # absent
    a = flat(g); a[4][1] = a[4][0]; case(arrays=a)                         # repeated
    a = flat(g); a[4] = np.concatenate([a[4], np.arange(1, 16, dtype=np.int32)]); case(arrays=a)  # 17 outputs
    case(n_out=-1)
    case(out_null=True)
    # a valid input still passes
    case(expect_fail=False)
    print("cases", n_cases, "accepted", n_ok)
''')


def test_malformed_inputs_return_status(pkg):
    env = dict(os.environ)
    r = subprocess.run([sys.executable, "-c", f"ROOT = {ROOT!r}\n" + CHILD], capture_output=True, text=True,
                       timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "cases" in r.stdout


NULL_CHILD = textwrap.dedent(r'''
    import ctypes as C, os, re, sys
    sys.path.insert(0, ROOT)
    import __graft_entry__ as G
    lib = G.load_package().native.lib()
    text = open(os.path.join(ROOT, "include", "tqec_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    scalar = {"int32_t": C.c_int32, "uint32_t": C.c_uint32, "int": C.c_int, "int64_t": C.c_int64,
              "uint64_t": C.c_uint64, "size_t": C.c_size_t, "float": C.c_float, "double": C.c_double}
    n = 0
    for name, params in re.findall(r"^int\s+(tqec_\w+)\s*\(([^)]*)\)\s*;", text, re.M | re.S):
        types = []
        for p in params.split(","):
            p = " ".join(p.replace("const", " ").split())
            if not p or p == "void":
                continue
            if "*" in p:
                types.append(C.c_void_p)
            else:
                types.append(scalar[p.rsplit(" ", 1)[0]])
        f = getattr(lib, name)
        f.argtypes = types
        f.restype = C.c_int
        rc = f(*[t() for t in types])
        lenient = name.endswith(("_destroy", "_release")) or name == "tqec_last_error"
        assert rc < 0 or (lenient and rc == 0), (name, rc)
        n += 1
    print("entry points", n)
''')


def test_null_arguments_return_status(pkg):
    """Every int-returning entry point of the header, called with NULL
    pointers and zero sizes, returns an error status (destroy and release of
    NULL may succeed) and does not crash."""
    r = subprocess.run([sys.executable, "-c", f"ROOT = {ROOT!r}\n" + NULL_CHILD], capture_output=True, text=True,
                       timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert int(r.stdout.split()[-1]) >= 40
