"""The workload configurations, decoded on the GPU and checked against the
oracle at the tolerance the plain form promises.

* d=3 surface code, p=0.05: 1,000 seeded Pauli errors decoded in float64
  (plain, one launch per syndrome, and batched): classes equal to the
  oracle's, every class log-probability within 1e-10 relative
  (|logp - log p_ref| <= 1e-10 |log p_ref|), -inf exactly on the classes the
  oracle gives probability 0.
* d=5 and d=7 at p in {0.02, 0.05, 0.08, 0.11}, 8,192 seeded syndromes each:
  float32 + recheck decisions equal to the oracle's outside exact ties;
  float32 class log-probabilities within twice the program's rounding bound;
  float64 within 1e-10 relative per class; bf16 intermediates within their
  bound (the float32 one plus 2^-9 per runtime step).
* circuit-level rotated Z-memory d=5, 5 rounds, p=0.001: 64 sampled detector
  patterns through the float32 decoder (with its recheck) and float64, against
  the oracle's float64 contraction of the same detector error model.
* TNMMAP(slices=2) on the GPU, against the oracle.
* The gated decoder at d=7, p=0.05 (surrogate trained on 2^22 syndromes
  labelled by the float64 contraction): at most 1e-4 decision mismatch
  against the exact decoder on 2^18 fresh syndromes, and its logical error
  rate inside the exact decoder's 95 % interval.

The oracle here is the C contractor (float64, per syndrome, the reference's
one-hot leaves rewritten per row, nothing folded) over the oracle's own
network; it contracts the decoder's tree, which is a tree of that network
because the two networks are equal tensor for tensor (checked here as well).
"""
import os

import numpy as np
import pytest

from conftest import gpu_available
from parity import assert_class_logprobs, assert_class_logprobs_within, assert_decisions, ties

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _c_oracle(oracle, net, steps):
    from oracle.c_oracle import CContractor

    return CContractor(net.ixs, [np.asarray(t) for t in net.tensors], net.iy, net.syndrome_positions, steps)


def _same_network(g, net):
    assert g.ixs == [list(x) for x in net.ixs] and list(g.iy) == list(net.iy)
    assert list(g.syndrome_positions) == list(net.syndrome_positions)
    for a, b in zip(g.tensors, net.tensors):
        np.testing.assert_array_equal(np.asarray(a).ravel(), np.asarray(b).flatten(order="F"))


def _surface(pkg, oracle, d, p, n, seed):
    t = pkg.tanner_graph(pkg.SurfaceCode(d, d))
    em = pkg.depolarizing(p, t.nq)
    rng = np.random.default_rng(seed)
    ep = pkg.random_error_pattern(em, rng, nsamples=n)
    s = pkg.syndrome_extraction(ep, t)
    bits = np.concatenate([s.sx, s.sz], axis=1)
    st, nq = oracle.surface_code_stabilizers(d, d)
    net = oracle.tnmmap_network(oracle.css_tanner(st, nq), em.px, em.py, em.pz)
    return t, em, bits, net


def _oracle_marginals(pkg, oracle, ct, net, bits):
    from oracle.c_oracle import host_cores

    _same_network(ct.graph, net)
    cc = _c_oracle(oracle, net, ct.steps)
    mar, cls = cc.contract(pkg.pack_syndromes(bits), threads=host_cores())
    return mar, cls


def test_config1_d3_thousand_errors_float64(pkg, oracle):
    """d=3, p=0.05, 1,000 seeded Pauli errors: class and the four class
    log-probabilities, plain float64 and batched float64, against the numpy
    oracle's einsum and the C oracle."""
    t, em, bits, net = _surface(pkg, oracle, 3, 0.05, 1000, 0x7E5A0000)
    want_np = oracle.OracleDecoder(oracle.css_tanner(*oracle.surface_code_stabilizers(3, 3)), em.px, em.py,
                                   em.pz).marginals(bits)
    for plain in (True, False):
        ct = pkg.compile(pkg.TNMMAP(precision="f64", plain=plain), t, em)
        want_c, _ = _oracle_marginals(pkg, oracle, ct, net, bits)
        cls, logp = ct.decode_batch(bits, return_logp=True)
        for want in (want_np, want_c):
            assert_decisions(cls, want)
            assert_class_logprobs(logp, want, 1e-10)
        # outside exact ties the class is the oracle's first maximum, bit for bit
        tie = ties(want_c)
        assert np.array_equal(cls[~tie], np.argmax(want_c, axis=1)[~tie])
        ct.close()


@pytest.mark.parametrize("tune", [False, True])
def test_plain_float64_d7_on_clusters_vs_oracle(pkg, oracle, tune):
    """The plain form at d=7: each syndrome contracted in float64 by one
    thread-block cluster (a wide program's default; the autotuner may keep it
    or pick the one-block form), one row per decode call and a batch of
    rows: classes equal to the oracle's outside ties, every class
    log-probability within 1e-10 relative."""
    t, em, bits, net = _surface(pkg, oracle, 7, 0.08, 96, 0x7E5A0017)
    ct = pkg.compile(pkg.TNMMAP(precision="f64", plain=True, optimizer=pkg.FixedOrder(
        pkg.load_order(os.path.join(ROOT, "tensorqec.jl_gb300", "orders", "surface_d7.tree")))), t, em)
    if tune:
        ct.program.autotune(1024)
    else:
        assert ct.program.info["cluster_blocks"] in (8, 16)
    want, _ = _oracle_marginals(pkg, oracle, ct, net, bits)
    cls, logp = ct.decode_batch(bits, return_logp=True)
    assert_decisions(cls, want)
    assert_class_logprobs(logp, want, 1e-10)
    for r in range(0, 96, 19):  # single-syndrome calls, as the drop-in decode makes them
        c1, l1 = ct.decode_batch(bits[r:r + 1], return_logp=True)
        assert c1[0] == cls[r]
        assert_class_logprobs(l1, want[r:r + 1], 1e-10)
    ct.close()


@pytest.mark.parametrize("d", [5, 7])
@pytest.mark.parametrize("p", [0.02, 0.05, 0.08, 0.11])
def test_config2_p_sweep_vs_oracle(pkg, oracle, d, p):
    n = 8192
    t, em, bits, net = _surface(pkg, oracle, d, p, n, 0x7E5A0002 + 1000 * d + int(round(p * 100)))
    ct = pkg.compile(pkg.TNMMAP(precision="f32"), t, em)
    want, _ = _oracle_marginals(pkg, oracle, ct, net, bits)
    info = ct.program.info
    # float32 + double-float recheck: the decoder's classes
    cls, logp = ct.decode_batch(bits, return_logp=True)
    assert_decisions(cls, want)
    # the float32 contraction alone, class by class, within its bound
    assert_class_logprobs_within(ct.class_logprobs(bits, precision="f32"), want, 2 * info["err_bound_f32"])
    # float64 of the same program: 1e-10 relative per class
    assert_class_logprobs(ct.class_logprobs(bits, precision="f64"), want, 1e-10)
    # bf16 intermediates (the float32 program, every stored intermediate rounded
    # to 8 significant bits): within the float32 bound plus 2^-9 per step
    bb = info["err_bound_f32"] + info["n_steps"] * 2.0 ** -9
    assert_class_logprobs_within(ct.class_logprobs(bits, precision="bf16"), want, -np.log1p(-bb))
    ct.close()


def test_config3_circuit_level_vs_oracle(pkg, oracle):
    """Rotated Z-memory d=5, 5 rounds, p=0.001: 64 seeded detector samples."""
    from tensorqec_gb300 import circuit as cz
    from tensorqec_gb300.dem import sample_dem, to_dem_string

    dm = cz.detector_error_model(cz.memory_z_circuit(5, 5, 0.001))
    steps = pkg.load_order(os.path.join(ROOT, "tensorqec.jl_gb300", "orders", "circuit_d5_r5.tree"))
    ct = pkg.compile(pkg.TNMMAP(precision="f32", optimizer=pkg.FixedOrder(steps)), dm)
    _, det, _ = sample_dem(dm, 64, np.random.default_rng(0x7E5A0003))
    net, _, _ = oracle.dem_network(oracle.parse_dem_string(to_dem_string(dm)), True)
    want, _ = _oracle_marginals(pkg, oracle, ct, net, det)
    cls = ct.decode_batch(det)
    assert_decisions(cls, want)
    assert_class_logprobs_within(ct.class_logprobs(det, precision="f32"), want, 2 * ct.program.info["err_bound_f32"])
    assert_class_logprobs(ct.class_logprobs(det, precision="f64"), want, 1e-10)
    ct.close()


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_sliced_program_on_gpu_vs_oracle(pkg, oracle, precision):
    """TNMMAP(slices=2): four narrower programs whose marginals are summed."""
    t, em, bits, net = _surface(pkg, oracle, 5, 0.08, 2000, 23)
    ct = pkg.compile(pkg.TNMMAP(precision=precision, slices=2,
                                optimizer=pkg.TreeSA(trials=8, sweeps=400, restarts=1)), t, em)
    assert ct.program.info["slices"] == 4
    want = oracle.OracleDecoder(oracle.css_tanner(*oracle.surface_code_stabilizers(5, 5)), em.px, em.py,
                                em.pz).marginals(bits)
    cls, logp = ct.decode_batch(bits, return_logp=True)
    assert_decisions(cls, want)
    if precision == "f64":
        assert_class_logprobs(logp, want, 1e-10)
    else:
        # rows outside the float32 margin keep float32 values, the rest double-float
        assert_class_logprobs_within(logp, want, 2 * ct.program.info["err_bound_f32"])
    ct.close()


@pytest.mark.parametrize("slices", [0, 2])
def test_circuit_d5_r7_width25_vs_oracle_fixture(pkg, slices):
    """Rotated Z-memory d=5, 7 rounds, p=0.001: a width-25 contraction tree
    (a 62-million-element arena per sample), whole and in 2^2 slices (each
    slice a program of its own, marginals summed), on the seeded samples whose
    oracle marginals tests/golden/circuit_d5_r7.json holds
    (tests/golden/make_circuit_d5_r7.py)."""
    import json

    from tensorqec_gb300 import circuit as cz
    from tensorqec_gb300.dem import sample_dem

    fx = json.load(open(os.path.join(ROOT, "tests", "golden", "circuit_d5_r7.json")))
    dm = cz.detector_error_model(cz.memory_z_circuit(5, 7, 0.001))
    _, det, _ = sample_dem(dm, fx["samples"], np.random.default_rng(fx["seed"]))
    assert np.array_equal(det.astype(int), np.array(fx["detectors"]))
    want = np.array(fx["marginals"])
    steps = pkg.load_order(os.path.join(ROOT, "tensorqec.jl_gb300", "orders", "circuit_d5_r7.tree"))
    for precision in ("f32", "f64"):
        ct = pkg.compile(pkg.TNMMAP(precision=precision, optimizer=pkg.FixedOrder(steps), slices=slices), dm)
        assert ct.program.info["width"] >= 24
        if slices:
            assert ct.program.info["slices"] == 1 << slices
        cls, logp = ct.decode_batch(det, return_logp=True)
        assert_decisions(cls, want)
        assert np.array_equal(cls, np.array(fx["classes"]))
        if precision == "f64":
            assert_class_logprobs(logp, want, 1e-10)
        else:
            assert_class_logprobs_within(logp, want, 2 * ct.program.info["err_bound_f32"])
        ct.close()


def test_config5_gated_d7_mismatch_and_ler(pkg):
    """Surrogate trained on 2^22 syndromes labelled by float64 contraction,
    calibrated at half the 1e-4 budget; on 2^18 fresh syndromes the gated
    decoder differs from the exact one on at most 1e-4 of the rows, and its
    logical error rate lies in the exact decoder's 95 % Wilson interval."""
    from tensorqec_gb300.surrogate import GatedDecoder, calibrate, train_surrogate

    t = pkg.tanner_graph(pkg.SurfaceCode(7, 7))
    em = pkg.depolarizing(0.05, t.nq)
    ct = pkg.compile(pkg.TNMMAP(precision="f32", optimizer=pkg.FixedOrder(
        pkg.load_order(os.path.join(ROOT, "tensorqec.jl_gb300", "orders", "surface_d7.tree")))), t, em)
    sur, stats = train_surrogate(ct, n_train=1 << 22, batch=16384, epochs=16, lr=3e-3, hidden=512, n_layers=4,
                                 seed=0x7E5A0005, label_precision="f64")
    assert stats["label_precision"] == "f64"
    thr, _ = calibrate(sur, ct, n_val=1 << 20, target_mismatch=5e-5, seed=0x7E5A0006)
    gd = GatedDecoder(ct, sur, thr)
    n = 1 << 18
    rng = np.random.default_rng(0x7E5A0007)
    ep = pkg.random_error_pattern(em, rng, nsamples=n)
    s = pkg.syndrome_extraction(ep, t)
    packed = pkg.pack_syndromes(np.concatenate([s.sx, s.sz], axis=1))
    exact = ct.program.decode_packed(packed)
    gated = gd.decode_packed(packed)
    mismatch = float(np.mean(gated != exact))
    assert mismatch <= 1e-4, mismatch
    assert gd.last_fallback < n  # the surrogate answered some rows itself
    a = (ep.zerror.astype(np.int64) @ ct.lx.T.astype(np.int64)) % 2
    b = (ep.xerror.astype(np.int64) @ ct.lz.T.astype(np.int64)) % 2
    truth = a[:, 0] + 2 * b[:, 0]
    k_ex, k_g = int((exact != truth).sum()), int((gated != truth).sum())
    z = 1.96
    ph = k_ex / n
    den = 1 + z * z / n
    c = (ph + z * z / (2 * n)) / den
    h = z * np.sqrt(ph * (1 - ph) / n + z * z / (4 * n * n)) / den
    assert c - h <= k_g / n <= c + h, (k_ex, k_g)
    sur.close()
    ct.close()
