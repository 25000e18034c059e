"""The committed contraction trees (tensorqec.jl_gb300/orders/) are trees of
their workloads' networks and compile to the programs their headers state;
the text format round-trips (CPU only: planning needs no GPU)."""
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORDERS = os.path.join(ROOT, "tensorqec.jl_gb300", "orders")


def _header_flops(path):
    for line in open(path):
        if "Compiled program:" in line:
            return float(line.split("Compiled program:")[1].split("flops")[0])
    raise AssertionError("no 'Compiled program' line")


def test_surface_d7_tree(pkg):
    path = os.path.join(ORDERS, "surface_d7.tree")
    steps = pkg.load_order(path)
    t = pkg.tanner_graph(pkg.SurfaceCode(7, 7))
    for p in (0.02, 0.11):  # the tree does not depend on p
        em = pkg.depolarizing(p, t.nq)
        lx, lz = pkg.logical_operator(t)
        g = pkg.tnmmap_css_graph(t, em, lx, lz)
        assert steps.shape == (g.n_tensors - 1, 2)
        got = pkg.optimize_code(g, pkg.FixedOrder(steps))
        assert np.array_equal(got, steps)
        info = pkg.native.inspect_plan(g, steps)
        assert info["flops_per_syndrome"] == _header_flops(path)
        assert info["width"] == 14


def test_circuit_tree(pkg):
    from tensorqec_gb300 import circuit as cz

    path = os.path.join(ORDERS, "circuit_d5_r5.tree")
    steps = pkg.load_order(path)
    dem = cz.detector_error_model(cz.memory_z_circuit(5, 5, 0.001))
    g = pkg.tnmmap_dem_graph(pkg.dem2tanner(dem), pkg.logical_map(dem), dem.error_rates, len(dem.logical_list), True)
    info = pkg.native.inspect_plan(g, steps)
    assert info["flops_per_syndrome"] == _header_flops(path)
    assert info["width"] == 20


def test_order_text_round_trip_and_wrong_size(pkg, tmp_path):
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    em = pkg.depolarizing(0.05, t.nq)
    lx, lz = pkg.logical_operator(t)
    g = pkg.tnmmap_css_graph(t, em, lx, lz)
    steps = pkg.optimize_code(g, pkg.TreeSA(trials=2, sweeps=50, restarts=1))
    path = str(tmp_path / "d3.tree")
    pkg.save_order(path, steps, "a d=3 tree\nsecond comment line")
    assert np.array_equal(pkg.load_order(path), steps)
    with pytest.raises(ValueError):
        pkg.optimize_code(g, pkg.FixedOrder(steps[:-1]))
