"""Several programs in one persistent launch per batch (csrc/multi.cu).

Uneven code sizes (surface d=3/5/7, colour 4.8.8 d=5, toric L=4 with 16
classes) with their own noise rates are decoded batch by batch, directly and
through a captured CUDA graph replayed once per batch; every class must equal
the single-program decoder's (float32 + recheck) except on exact ties.
"""
import numpy as np
import pytest

from conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]


def _specs(pkg):
    return [(pkg.SurfaceCode(3, 3), 0.08, 500), (pkg.SurfaceCode(5, 5), 0.05, 700), (pkg.Color488(5), 0.06, 300),
            (pkg.ToricCode(4, 4), 0.04, 200), (pkg.SurfaceCode(7, 7), 0.05, 150)]


def _oracle_stabilizers(oracle, i):
    """The oracle's stabilisers of _specs(pkg)[i]."""
    return [lambda: oracle.surface_code_stabilizers(3, 3), lambda: oracle.surface_code_stabilizers(5, 5),
            lambda: oracle.color_code_stabilizers("488", 5), lambda: oracle.toric_code_stabilizers(4, 4),
            lambda: oracle.surface_code_stabilizers(7, 7)][i]()


def _setup(pkg):
    specs = _specs(pkg)
    progs = []
    for i, (code, p, n) in enumerate(specs):
        t = pkg.tanner_graph(code)
        em = pkg.depolarizing(p, t.nq)
        ct = pkg.compile(pkg.TNMMAP(precision="f32"), t, em)
        rng = np.random.default_rng(40 + i)
        ep = pkg.random_error_pattern(em, rng, nsamples=n)
        s = pkg.syndrome_extraction(ep, t)
        bits = np.concatenate([s.sx, s.sz], axis=1)
        progs.append((ct, bits))
    return progs


def _check(pkg, progs, got):
    for (ct, bits), cls in zip(progs, got):
        want = ct.decode_batch(bits)
        lp = ct.class_logprobs(bits, precision="f64")
        srt = np.sort(lp, axis=1)
        tie = (srt[:, -1] - srt[:, -2]) <= 1e-9
        bad = (cls != want) & ~tie
        assert not bad.any(), (np.flatnonzero(bad)[:10], cls[bad][:10], want[bad][:10])


def test_multi_program_batches_match_single_program(pkg):
    import torch

    progs = _setup(pkg)
    md = pkg.native.MultiDecoder([ct.program for ct, _ in progs])
    info = md.info()
    assert info["grid"] > 0 and len(info["groups"]) == len(progs)
    syn = [torch.from_numpy(pkg.pack_syndromes(b)).cuda() for _, b in progs]
    cls = [torch.full((b.shape[0],), -1, dtype=torch.int32, device="cuda") for _, b in progs]
    # three uneven batches: cumulative end rows per program
    n = np.array([b.shape[0] for _, b in progs])
    ends = np.stack([n * 1 // 5, n * 3 // 5, n])
    md.set_work(ends, [x.data_ptr() for x in syn], [x.data_ptr() for x in cls])
    stream = torch.cuda.current_stream()
    md.reset(stream.cuda_stream)
    for _ in range(ends.shape[0] + 1):  # one launch past the last batch does nothing
        md.launch(stream.cuda_stream)
    torch.cuda.synchronize()
    got = [c.cpu().numpy() for c in cls]
    assert all((g >= 0).all() for g in got)
    _check(pkg, progs, got)

    # the same work through a CUDA graph replayed once per batch
    for c in cls:
        c.fill_(-1)
    side = torch.cuda.Stream()
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        md.reset(side.cuda_stream)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side):
            md.launch(side.cuda_stream)
        md.reset(side.cuda_stream)
        for _ in range(ends.shape[0]):
            g.replay()
    torch.cuda.synchronize()
    got = [c.cpu().numpy() for c in cls]
    assert all((g_ >= 0).all() for g_ in got)
    _check(pkg, progs, got)
    md.close()
    for ct, _ in progs:
        ct.close()


def test_multi_programs_must_agree_on_recheck(pkg):
    """One recheck launch serves every program: programs whose recheck
    arithmetic differs (TQEC_FLAG_RECHECK_F64 on one of them) are refused."""
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    em = pkg.depolarizing(0.05, t.nq)
    a = pkg.compile(pkg.TNMMAP(precision="f32"), t, em)
    b = pkg.compile(pkg.TNMMAP(precision="f32", recheck_f64=True), t, em)
    with pytest.raises(pkg.native.TqecError):
        pkg.native.MultiDecoder([a.program, b.program])
    md = pkg.native.MultiDecoder([b.program, b.program])
    md.close()
    a.close()
    b.close()


def test_multi_program_launch_vs_oracle(pkg, oracle):
    """The persistent multi-program launch (float32 + one recheck launch for
    every program) decides each row like the oracle's float64 contraction of
    that row's own code, outside exact ties (tests/parity.py)."""
    import torch
    from oracle.c_oracle import CContractor, host_cores
    from parity import assert_decisions

    progs = _setup(pkg)
    md = pkg.native.MultiDecoder([ct.program for ct, _ in progs])
    syn = [torch.from_numpy(pkg.pack_syndromes(b)).cuda() for _, b in progs]
    cls = [torch.full((b.shape[0],), -1, dtype=torch.int32, device="cuda") for _, b in progs]
    n = np.array([b.shape[0] for _, b in progs])
    ends = np.stack([n // 2, n])
    md.set_work(ends, [x.data_ptr() for x in syn], [x.data_ptr() for x in cls])
    stream = torch.cuda.current_stream()
    md.reset(stream.cuda_stream)
    for _ in range(ends.shape[0]):
        md.launch(stream.cuda_stream)
    torch.cuda.synchronize()
    for i, ((ct, bits), c) in enumerate(zip(progs, cls)):
        st, nq = _oracle_stabilizers(oracle, i)
        em = ct.em
        net = oracle.tnmmap_network(oracle.css_tanner(st, nq), em.px, em.py, em.pz)
        assert ct.graph.ixs == net.ixs
        cc = CContractor(net.ixs, [np.asarray(t) for t in net.tensors], net.iy, net.syndrome_positions, ct.steps)
        want, _ = cc.contract(pkg.pack_syndromes(bits), threads=host_cores())
        assert_decisions(c.cpu().numpy(), want)
    md.close()
    for ct, _ in progs:
        ct.close()


@pytest.mark.parametrize("order", [(7, 9), (9, 7)])
def test_multi_wide_programs_with_different_cluster_forms(pkg, order):
    """Two wide programs (surface d=7 and d=9) recheck on thread-block
    clusters whose shared-memory sizes differ; whichever is set up last, both
    cluster launches run, directly and from a captured graph, and decide
    like their single-program decoders."""
    import torch

    progs = []
    for i, d in enumerate(order):
        t = pkg.tanner_graph(pkg.SurfaceCode(d, d))
        em = pkg.depolarizing(0.06, t.nq)
        ct = pkg.compile(pkg.TNMMAP(precision="f32"), t, em)
        ep = pkg.random_error_pattern(em, np.random.default_rng(90 + d), nsamples=120)
        s = pkg.syndrome_extraction(ep, t)
        progs.append((ct, np.concatenate([s.sx, s.sz], axis=1)))
    assert all(ct.program.info["cluster_blocks"] in (8, 16) for ct, _ in progs)
    md = pkg.native.MultiDecoder([ct.program for ct, _ in progs])
    syn = [torch.from_numpy(pkg.pack_syndromes(b)).cuda() for _, b in progs]
    cls = [torch.full((b.shape[0],), -1, dtype=torch.int32, device="cuda") for _, b in progs]
    n = np.array([b.shape[0] for _, b in progs])
    ends = np.stack([n // 3, n])
    md.set_work(ends, [x.data_ptr() for x in syn], [x.data_ptr() for x in cls])
    stream = torch.cuda.current_stream()
    md.reset(stream.cuda_stream)
    for _ in range(ends.shape[0]):
        md.launch(stream.cuda_stream)
    torch.cuda.synchronize()
    _check(pkg, progs, [c.cpu().numpy() for c in cls])

    for c in cls:
        c.fill_(-1)
    side = torch.cuda.Stream()
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        md.reset(side.cuda_stream)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side):
            md.launch(side.cuda_stream)
        md.reset(side.cuda_stream)
        for _ in range(ends.shape[0]):
            g.replay()
    torch.cuda.synchronize()
    _check(pkg, progs, [c.cpu().numpy() for c in cls])
    md.close()
    for ct, _ in progs:
        ct.close()
