"""The multi-GPU path is replicas (syndromes shard with no data exchange):
two gloo ranks on the CPU check the per-rank streams and the reductions the
benchmark uses."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import sys

    import torch.distributed as dist

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import __graft_entry__ as G

    pkg = G.load_package()
    from tensorqec_gb300 import replicas

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = pkg.tanner_graph(pkg.SurfaceCode(3, 3))
    em = pkg.depolarizing(0.1, t.nq)
    rng = np.random.default_rng(replicas.rank_seed(1234, rank))
    ep = pkg.random_error_pattern(em, rng, nsamples=200)
    syn = pkg.syndrome_extraction(ep, t)
    bits = np.concatenate([syn.sx, syn.sz], axis=1)
    step_ms = [1.0 + rank, 5.0 - rank]
    mx = replicas.reduce_max(step_ms, dist)
    errs = replicas.reduce_sum([int(bits.sum()), rank + 1], dist)
    out[rank] = {"mx": mx, "errs": errs, "first": bits[:5].tolist(), "own": int(bits.sum()),
                 "offset": replicas.sample_offset(rank, 1000)}
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
        assert p.exitcode == 0
    a, b = out[0], out[1]
    # the slowest rank sets each step; counters add up
    assert a["mx"] == b["mx"] == [2.0, 5.0]
    assert a["errs"] == b["errs"] == [a["own"] + b["own"], 3]
    # disjoint streams: different host seeds, adjacent counter ranges
    assert a["first"] != b["first"]
    assert (a["offset"], b["offset"]) == (0, 1000)
    assert replicas_rate() == 2 * 65536 / 2.0e-3


def replicas_rate():
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import __graft_entry__ as G

    G.load_package()
    from tensorqec_gb300.replicas import job_rate

    return job_rate(2, 65536, 2.0)
