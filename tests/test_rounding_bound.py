"""The float32 rounding bound the planner derives, against float32
arithmetic on the CPU.

The float32 kernel certifies a decision when the class margin exceeds twice
its rounding bound u * err_terms (u = 2^-24; err_terms = sum over runtime
steps of K + 1, plus one per float32 constant table, csrc/plan.cpp).  Here
the compiled program runs in float32 and in float64 through the numpy
emulator (operands rounded to float32, products and sums in float32, any
summation order), and every class entry of every syndrome must stay within
that relative bound of the float64 value.  The kernel's power-of-two
normalisation is exact and leaves relative errors unchanged, so entries far
from float32's underflow carry the same bound.
"""
import numpy as np
import pytest

from plan_emulator import run_plan


def _css(pkg, code, p, n, seed):
    t = pkg.tanner_graph(code)
    em = pkg.depolarizing(p, t.nq)
    lx, lz = pkg.logical_operator(t)
    g = pkg.tnmmap_css_graph(t, em, lx, lz)
    plan = pkg.native.inspect_plan(g, pkg.optimize_code(g, pkg.TreeSA(trials=4, sweeps=200, restarts=1)))
    rng = np.random.default_rng(seed)
    ep = pkg.random_error_pattern(em, rng, nsamples=n)
    s = pkg.syndrome_extraction(ep, t)
    return plan, np.concatenate([s.sx, s.sz], axis=1)


@pytest.mark.parametrize("kind,d,p,n", [("surface", 5, 0.08, 200), ("surface", 7, 0.05, 12), ("toric", 3, 0.08, 64),
                                        ("488", 5, 0.1, 100)])
def test_float32_error_within_planner_bound(pkg, kind, d, p, n):
    code = {"surface": lambda: pkg.SurfaceCode(d, d), "toric": lambda: pkg.ToricCode(d, d),
            "488": lambda: pkg.Color488(d)}[kind]()
    plan, bits = _css(pkg, code, p, n, seed=40 + d)
    bound = 2.0 ** -24 * plan["err_terms"] * 1.01
    f64 = run_plan(plan, bits)
    f32 = run_plan(plan, bits, dtype=np.float32).astype(np.float64)
    live = f64 > 1e-30
    assert ((f64 == 0) == (f32 == 0)).all()
    rel = np.abs(f32[live] - f64[live]) / f64[live]
    assert rel.max() <= bound, (rel.max(), bound)


def test_float32_bound_of_a_circuit_level_program_with_tensor_steps(pkg):
    """The circuit-level d=5, 2-round model: GEMM-shaped steps add the
    tf32-split terms to the bound; the float32 SIMT arithmetic stays inside
    it (entries above float32's normal range only)."""
    from tensorqec_gb300 import circuit, dem as demmod

    dm = circuit.detector_error_model(circuit.memory_z_circuit(5, 2, 0.001))
    t = demmod.dem2tanner(dm)
    g = pkg.tnmmap_dem_graph(t, demmod.logical_map(dm), dm.error_rates, len(dm.logical_list), True)
    steps = pkg.optimize_code(g, pkg.TreeSA(trials=16, sweeps=1000, seed=1, restarts=2))
    plan = pkg.native.inspect_plan(g, steps)
    _, det, _ = demmod.sample_dem(dm, 3, np.random.default_rng(9))
    bound = 2.0 ** -24 * plan["err_terms"] * 1.01
    f64 = run_plan(plan, det)
    f32 = run_plan(plan, det, dtype=np.float32).astype(np.float64)
    live = f64 > 1e-30
    assert live.any()
    rel = np.abs(f32[live] - f64[live]) / f64[live]
    assert rel.max() <= bound, (rel.max(), bound)
