"""GPU tests of the learned surrogate: gradients against the float64 CPU
oracle, training that reduces the loss, checkpoint round trip, and the
gated decoder's decisions against the exact contraction.

Gradient tolerance: relative L2 error 2e-3 against the oracle with bf16
rounding at the kernels' rounding points (float32 accumulation order is the
only other difference), and 0.2 against the unquantised float64 network
(the size of bf16 rounding in a small network).
"""
import os

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("n_in,hidden,layers,n_out,rows", [(8, 32, 3, 4, 64), (48, 64, 4, 4, 300),
                                                            (70, 96, 4, 16, 130)])
def test_gradients_match_cpu_float64(pkg, n_in, hidden, layers, n_out, rows):
    from oracle import mlp_oracle

    from tensorqec_gb300.surrogate import Surrogate

    rng = np.random.default_rng(n_in)
    sur = Surrogate(n_in, n_out, hidden, layers, seed=3)
    bits = (rng.random((rows, n_in)) < 0.3).astype(np.uint8)
    packed = pkg.pack_syndromes(bits)
    t = rng.random((rows, n_out)).astype(np.float32)
    t /= t.sum(axis=1, keepdims=True)
    p = sur.params()
    g, loss = sur.gradients(packed, t)
    l64, g64 = mlp_oracle.forward_backward(p, packed, t, n_in, hidden, layers, n_out, bf16=True)
    _, gx = mlp_oracle.forward_backward(p, packed, t, n_in, hidden, layers, n_out, bf16=False)
    assert abs(loss - l64) < 1e-3 * max(1.0, abs(l64))
    assert rel_l2(g, g64) < 2e-3, rel_l2(g, g64)
    assert rel_l2(g, gx) < 0.2  # bf16 quantisation of weights and activations
    sur.close()


def test_training_reduces_loss_and_checkpoint_roundtrip(pkg, tmp_path):
    from tensorqec_gb300.surrogate import Surrogate, soft_labels

    t = pkg.tanner_graph(pkg.SurfaceCode(5, 5))
    em = pkg.depolarizing(0.05, t.nq)
    ct = pkg.compile(pkg.TNMMAP(precision="f32"), t, em)
    rng = np.random.default_rng(4)
    ep = pkg.random_error_pattern(em, rng, nsamples=1 << 16)
    syn = pkg.syndrome_extraction(ep, t)
    bits = np.concatenate([syn.sx, syn.sz], axis=1)
    packed = pkg.pack_syndromes(bits)
    tgt = soft_labels(ct.class_logprobs(bits))
    sur = Surrogate(t.ns, 4, 128, 4, seed=5)
    first = sur.train_step(packed[:4096], tgt[:4096], 2e-3)
    for s in range(1, 120):
        j = (s * 4096) % (len(packed) - 4096)
        last = sur.train_step(packed[j:j + 4096], tgt[j:j + 4096], 2e-3)
    assert last < 0.6 * first
    cls, conf = sur.infer(packed)
    exact = ct.decode_batch(bits)
    assert (cls == exact).mean() > 0.9
    path = os.path.join(tmp_path, "sur.bin")
    sur.save(path)
    sur2 = Surrogate(t.ns, 4, 128, 4, seed=99)
    sur2.load(path)
    np.testing.assert_array_equal(sur2.params(), sur.params())
    cls2, conf2 = sur2.infer(packed)
    np.testing.assert_array_equal(cls2, cls)
    sur.close()
    sur2.close()
    ct.close()


def test_gated_decoder_matches_exact_where_it_answers(pkg):
    from tensorqec_gb300.surrogate import GatedDecoder, calibrate, train_surrogate

    t = pkg.tanner_graph(pkg.SurfaceCode(5, 5))
    em = pkg.depolarizing(0.05, t.nq)
    ct = pkg.compile(pkg.TNMMAP(precision="f32"), t, em)
    sur, stats = train_surrogate(ct, n_train=1 << 17, batch=4096, epochs=2, hidden=128, n_layers=4, seed=6)
    thr, cst = calibrate(sur, ct, n_val=1 << 16, target_mismatch=1e-3, seed=7)
    assert 0.0 < cst["accept_fraction"] <= 1.0
    gd = GatedDecoder(ct, sur, thr)
    rng = np.random.default_rng(8)
    ep = pkg.random_error_pattern(em, rng, nsamples=1 << 16)
    syn = pkg.syndrome_extraction(ep, t)
    bits = np.concatenate([syn.sx, syn.sz], axis=1)
    got = gd.decode_batch(bits)
    exact = ct.decode_batch(bits)
    cls, conf = sur.infer(pkg.pack_syndromes(bits))
    # rows the gate sent to the exact path are exact; answered rows are the surrogate's
    fb = conf < thr
    assert gd.last_fallback == int(fb.sum())
    np.testing.assert_array_equal(got[fb], exact[fb])
    np.testing.assert_array_equal(got[~fb], cls[~fb])
    assert (got != exact).mean() < 5e-3
    sur.close()
    ct.close()


def test_tensor_core_gemm_matches_simt(pkg):
    """The tcgen05 hidden-layer GEMM against the SIMT GEMM on the same bf16
    weights: both accumulate in float32, so logits agree to bf16 rounding of
    the hidden activations (max difference 3e-2 of the largest logit)."""
    from tensorqec_gb300.surrogate import Surrogate

    rng = np.random.default_rng(21)
    for n_in, rows in ((48, 1000), (80, 4096 + 77)):
        sur = Surrogate(n_in, 4, 512, 4, seed=9)
        p = sur.params()
        sur.set_params(p * 3.0)  # larger activations: a wider check of the accumulator path
        bits = (rng.random((rows, n_in)) < 0.2).astype(np.uint8)
        packed = pkg.pack_syndromes(bits)
        sur.use_tensor_cores(False)
        ref = sur.logits(packed)
        sur.use_tensor_cores(True)
        got = sur.logits(packed)
        scale = np.abs(ref).max()
        assert np.abs(got - ref).max() <= 3e-2 * scale, np.abs(got - ref).max() / scale
        assert (got.argmax(1) == ref.argmax(1)).mean() > 0.99
        sur.close()


def test_device_resident_step_equals_host_step(pkg):
    """A training step on rows gathered from a device-resident set matches
    the host step on the same batch; an index outside the set is reported
    (and reads row 0, never outside the buffers)."""
    torch = pytest.importorskip("torch")
    from tensorqec_gb300.surrogate import Surrogate

    rng = np.random.default_rng(12)
    n_set, n_in, n_out, batch = 5000, 48, 4, 1024
    packed = pkg.pack_syndromes((rng.random((n_set, n_in)) < 0.2).astype(np.uint8))
    t = rng.random((n_set, n_out)).astype(np.float32)
    t /= t.sum(axis=1, keepdims=True)
    idx = rng.permutation(n_set)[:batch].astype(np.int32)
    a = Surrogate(n_in, n_out, 256, 4, seed=5)
    b = Surrogate(n_in, n_out, 256, 4, seed=5)
    la = a.train_step(packed[idx], t[idx], 1e-3)
    d_syn, d_t, d_idx = (torch.from_numpy(x).cuda() for x in (packed, t, idx))
    lb = b.train_step_rows(d_syn.data_ptr(), d_t.data_ptr(), n_set, d_idx.data_ptr(), batch, 1e-3, with_loss=True)
    # weight gradients are summed with atomics, so only the order of float32
    # additions differs: the loss to float32 rounding, and after one Adam step
    # (a step of about lr per parameter) at most a sign flip where a gradient
    # is near zero
    assert abs(la - lb) <= 1e-5 * abs(la)
    diff = np.abs(a.params() - b.params())
    assert diff.max() <= 2.5e-3 and (diff > 1e-6).mean() < 1e-3
    bad = torch.tensor([0, n_set], dtype=torch.int32, device="cuda")
    with pytest.raises(pkg.native.TqecError):
        b.train_step_rows(d_syn.data_ptr(), d_t.data_ptr(), n_set, bad.data_ptr(), 2, 1e-3, with_loss=True)
    a.close()
    b.close()


@pytest.mark.parametrize("rows", [1000, 65536 + 77])
def test_fused_forward_matches_layer_by_layer(pkg, rows):
    """The fused tcgen05 forward (all layers in one persistent kernel, the
    default for inference) against the layer-by-layer tcgen05 GEMMs: the
    hidden activations are the same bf16 values, so the logits differ only by
    the float32 summation order of the output layer (1e-4 relative), and the
    classes agree wherever the top two logits are not that close."""
    from tensorqec_gb300.surrogate import Surrogate

    rng = np.random.default_rng(rows)
    sur = Surrogate(48, 4, 512, 4, seed=9)
    packed = pkg.pack_syndromes((rng.random((rows, 48)) < 0.15).astype(np.uint8))
    sur.use_tensor_cores(True)
    lf = sur.logits(packed)
    cf, pf = sur.infer(packed)
    sur.use_tensor_cores(2)
    ll = sur.logits(packed)
    cl, pl = sur.infer(packed)
    assert np.max(np.abs(lf - ll) / (1.0 + np.abs(ll))) <= 1e-4
    srt = np.sort(ll, axis=1)
    close = (srt[:, -1] - srt[:, -2]) <= 1e-3
    assert not ((cf != cl) & ~close).any()
    assert np.max(np.abs(pf - pl)) <= 1e-4
    sur.close()


def test_fused_gate_matches_gate_on_the_logits(pkg):
    """The gate fused into the forward's last epilogue (the default
    inference path, and the gated decoder's): the first maximum of each row's
    logits and the softmax confidence 1 / sum(exp(l - max)), as the separate
    gate kernel computes them from the same logits."""
    from tensorqec_gb300.surrogate import Surrogate

    rng = np.random.default_rng(31)
    sur = Surrogate(48, 4, 512, 4, seed=11)
    sur.set_params(sur.params() * 2.0)
    packed = pkg.pack_syndromes((rng.random((70000, 48)) < 0.15).astype(np.uint8))
    sur.use_tensor_cores(True)
    lf = sur.logits(packed).astype(np.float64)
    cf, pf = sur.infer(packed)
    assert np.array_equal(cf, np.argmax(lf, axis=1))
    want = 1.0 / np.exp(lf - lf.max(axis=1, keepdims=True)).sum(axis=1)
    assert np.max(np.abs(pf - want)) <= 1e-5
    sur.close()
