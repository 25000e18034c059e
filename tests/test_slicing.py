"""Sliced contraction (network.slice_graph, decoder.SlicedProgram) on the
CPU.

Fixing k inner labels splits a contraction into 2^k narrower ones whose
marginals add up to the original.  The slices' compiled programs run here
through the numpy emulator of the kernel's program (a stand-in for
``native.Program`` with the same calls), so the whole decoder path of
``TNMMAP(slices=k)`` — slicing, one program per slice, log-sum-exp, the
float32 margin test and the recheck of low-margin rows, first-maximum
argmax — is checked against the oracle without a GPU.
Tolerance: 1e-10 relative to the row's largest class in float64; classes
equal to the oracle's argmax except where the top two are within 1e-9.
"""
import numpy as np
import pytest

from plan_emulator import run_plan


def _surface(pkg, d, p, n, seed):
    t = pkg.tanner_graph(pkg.SurfaceCode(d, d))
    em = pkg.depolarizing(p, t.nq)
    ep = pkg.random_error_pattern(em, np.random.default_rng(seed), nsamples=n)
    s = pkg.syndrome_extraction(ep, t)
    return t, em, np.concatenate([s.sx, s.sz], axis=1)


def test_slices_sum_to_the_whole_and_narrow_the_tree(pkg, oracle):
    from tensorqec_gb300 import network

    t, em, bits = _surface(pkg, 7, 0.05, 3, 11)
    lx, lz = pkg.logical_operator(t)
    g = pkg.tnmmap_css_graph(t, em, lx, lz)
    steps = pkg.optimize_code(g, pkg.TreeSA(trials=4, sweeps=200, restarts=1))
    sets = network.step_label_sets(g, steps)
    width = max(len(u) for u, _ in sets)
    res_width = max(len(r) for _, r in sets)  # the widest intermediate: a syndrome's working set
    labels = network.choose_slice_labels(g, steps, 3)
    assert len(labels) == 3 and not set(labels) & set(g.iy)
    total = 0
    for v in range(8):
        gs = network.slice_graph(g, labels, v)
        sliced = network.step_label_sets(gs, steps)
        assert max(len(u) for u, _ in sliced) < width
        assert max(len(r) for _, r in sliced) < res_width
        total = total + run_plan(pkg.native.inspect_plan(gs, steps), bits)
    want = oracle.OracleDecoder(oracle.css_tanner(*oracle.surface_code_stabilizers(7, 7)), em.px, em.py,
                                em.pz).marginals(bits)
    np.testing.assert_allclose(total, want, rtol=1e-10, atol=1e-12 * want.max())


def test_outputs_and_syndrome_labels_cannot_be_fixed(pkg):
    from tensorqec_gb300 import network

    t, em, _ = _surface(pkg, 3, 0.05, 1, 1)
    lx, lz = pkg.logical_operator(t)
    g = pkg.tnmmap_css_graph(t, em, lx, lz)
    for lab in (g.iy[0], g.ixs[g.syndrome_positions[0]][0]):
        with pytest.raises(ValueError):
            network.slice_graph(g, [lab], 0)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_sliced_decoder_matches_oracle(pkg, oracle, emulated, precision):
    t, em, bits = _surface(pkg, 5, 0.08, 300, 23)
    ct = pkg.compile(pkg.TNMMAP(precision=precision, slices=2,
                                optimizer=pkg.TreeSA(trials=4, sweeps=200, restarts=1)), t, em)
    assert len(emulated.instances) == 4 and ct.program.info["slices"] == 4
    want = oracle.OracleDecoder(oracle.css_tanner(*oracle.surface_code_stabilizers(5, 5)), em.px, em.py,
                                em.pz).marginals(bits)
    cls, lp = ct.decode_batch(bits, return_logp=True)
    scale = want.max(axis=1, keepdims=True)
    tol = 1e-10 if precision == "f64" else 2 * ct.program.info["err_bound_f32"]
    assert (np.abs(np.exp(lp) - want) / scale).max() <= tol
    top = want.max(axis=1)
    srt = np.sort(want, axis=1)
    tie = srt[:, -1] - srt[:, -2] <= 1e-9 * top
    assert (cls[~tie] == np.argmax(want, axis=1)[~tie]).all()
    assert (want[np.arange(len(cls)), cls] >= top * (1 - 1e-9)).all()
    if precision == "f32":
        # exact ties and near-ties went to the double-float recheck
        rechecked = ct.program.last_recheck_count()
        assert rechecked >= tie.sum()
        assert all(c[0] == 2 for p in emulated.instances for c in p.calls[1:]) or rechecked == 0
    res = ct.decode(pkg.CSSSyndrome(bits[0, :t.stgx.ns], bits[0, t.stgx.ns:]))
    assert res.success_tag and pkg.syndrome_extraction(res.error_pattern, t) == pkg.CSSSyndrome(
        bits[0, :t.stgx.ns], bits[0, t.stgx.ns:])


def test_sliced_dem_decoder_matches_oracle(pkg, oracle, emulated):
    """The reference's dem.dem fixture, every detector pattern, in two slices."""
    import json
    import os

    text = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kat.json")))["dem_small"]["text"]
    dem = pkg.parse_dem_string(text)
    ct = pkg.compile(pkg.TNMMAP(precision="f64", slices=1, optimizer=pkg.TreeSA(trials=4, sweeps=100)), dem)
    nd = len(dem.detector_list)
    bits = ((np.arange(1 << nd)[:, None] >> np.arange(nd)[None, :]) & 1).astype(np.uint8)
    want = oracle.OracleDEMDecoder(oracle.parse_dem_string(text)).marginals(bits)
    lp = ct.class_logprobs(bits)
    live = want > 0
    np.testing.assert_allclose(np.exp(lp[live]), want[live], rtol=1e-10)
    assert np.isneginf(lp[~live]).all()
