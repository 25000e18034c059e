"""Order-independent known answers beyond d=3: class marginals from coset
weight enumerators.

When a qubit's X and Z errors are independent (rates qx and qz), the qubit
tensor of the TNMMAP network (src/decoding/tndecoder.jl:118-121,
``[1-px-py-pz pz; px py]``) is the outer product of ``[1-qx, qx]`` and
``[1-qz, qz]``: px = qx(1-qz), pz = (1-qx)qz, py = qx*qz.  The class marginal
of a CSS code then factorises, for a syndrome (sx, sz):

    mar[a + 2^k b] = Z(a) * X(b)
    X(b) = sum over ex with Hz ex = sz and lz ex = b of qx^|ex| (1-qx)^(n-|ex|)
    Z(a) = sum over ez with Hx ez = sx and lx ez = a of qz^|ez| (1-qz)^(n-|ez|)

(class index in Julia's linear order of ``mar[a..., b...]``, a_i = lx_i.ez,
b_i = lz_i.ex).  The ex solving Hz ex = sz form e0 + rowspace(Hx) + span(lx),
so each X(b) is a sum of weight enumerators of cosets of rowspace(Hx), which
are counted here by enumerating the 2^rank(Hx) coset members as bit masks
(2^24 at d=7).  Nothing in this computation depends on a contraction order,
a network layout or the planner, so it pins the oracle's contraction, the
oracle's C contractor and the planner's compiled program (run by the numpy
emulator) at d=5, d=7, the toric code L=4 (k=2, 16 classes) and the 6.6.6
colour code d=5.  It is itself checked against the reference-restated
enumeration over all 4^9 Pauli errors at d=3.

Tolerance: 1e-10 relative to the row's largest class (float64 sums).
"""
import numpy as np
import pytest

from plan_emulator import run_plan

QX, QZ = 0.06, 0.04


def _masks(H):
    """Rows of a 0/1 matrix as integer bit masks (bit j = column j)."""
    w = 1 << np.arange(H.shape[1], dtype=np.uint64)
    return [int((np.asarray(r, dtype=np.uint64) * w).sum()) for r in np.atleast_2d(H)]


def _basis(masks):
    """A GF(2) basis of the span of `masks` (xor elimination)."""
    basis = []
    for m in masks:
        for b in basis:
            m = min(m, m ^ b)
        if m:
            basis.append(m)
    return basis


def _solve(H, s):
    """One x with H x = s over GF(2), as a bit mask (Gauss-Jordan)."""
    A = np.concatenate([np.asarray(H, dtype=np.uint8) % 2, np.asarray(s, dtype=np.uint8).reshape(-1, 1) % 2], axis=1)
    m, n = H.shape
    piv, r = [], 0
    for c in range(n):
        rows = np.flatnonzero(A[r:, c]) + r
        if len(rows) == 0:
            continue
        A[[r, rows[0]]] = A[[rows[0], r]]
        for i in np.flatnonzero(A[:, c]):
            if i != r:
                A[i] ^= A[r]
        piv.append(c)
        r += 1
        if r == m:
            break
    assert not A[r:, n].any(), "syndrome outside the column space"
    x = 0
    for i, c in enumerate(piv):
        if A[i, n]:
            x |= 1 << c
    return x


def _span(gens):
    out = np.zeros(1, dtype=np.uint64)
    for g in gens:
        out = np.concatenate([out, out ^ np.uint64(g)])
    return out


def _coset_weights(gens, v, n):
    """Number of members of v + span(gens) of each Hamming weight 0..n."""
    low, high = _span(gens[:16]), _span(gens[16:])
    counts = np.zeros(n + 1, dtype=np.int64)
    for i in range(0, len(high), 16):
        block = low[None, :] ^ (high[i:i + 16, None] ^ np.uint64(v))
        counts += np.bincount(np.bitwise_count(block).ravel(), minlength=n + 1)
    return counts


def _weight_sum(counts, q):
    n = len(counts) - 1
    w = np.arange(n + 1)
    return float((counts * q ** w * (1 - q) ** (n - w)).sum())


def _parity(a, b):
    return bin(a & b).count("1") & 1


def enumerator_marginal(Hx, Hz, lx, lz, qx, qz, sx, sz):
    """mar (Julia linear order, 4^k entries) for independent X/Z noise."""
    n = Hx.shape[1]
    k = lx.shape[0]
    gx, gz = _basis(_masks(Hx)), _basis(_masks(Hz))
    assert len(gx) + len(gz) + k == n
    mlx, mlz = _masks(lx), _masks(lz)

    def part(H_check, s, stab_gens, reps, duals, q):
        # members of {e : H_check e = s} = e0 + span(stab_gens) + span(reps);
        # the class bit i is duals_i . e
        e0 = _solve(H_check, s)
        out = np.zeros(1 << k)
        for t in range(1 << k):
            v = e0
            for j in range(k):
                if t >> j & 1:
                    v ^= reps[j]
            c = sum(_parity(duals[i], v) << i for i in range(k))
            out[c] += _weight_sum(_coset_weights(stab_gens, v, n), q)
        return out

    X = part(Hz, sz, gx, mlx, mlz, qx)  # indexed by b
    Z = part(Hx, sx, gz, mlz, mlx, qz)  # indexed by a
    return np.outer(X, Z).ravel()  # index b * 2^k + a


def _independent_rates(n):
    px, pz, py = QX * (1 - QZ), (1 - QX) * QZ, QX * QZ
    return np.full(n, px), np.full(n, py), np.full(n, pz)


def _code(oracle, kind, d):
    if kind == "surface":
        st, nq = oracle.surface_code_stabilizers(d, d)
    elif kind == "toric":
        st, nq = oracle.toric_code_stabilizers(d, d)
    else:
        st, nq = oracle.color_code_stabilizers(kind, d)
    return oracle.css_tanner(st, nq)


def _syndromes(oracle, t, n, seed):
    """Zero syndrome first, then syndromes of sampled independent X/Z errors."""
    rng = np.random.default_rng(seed)
    ex = (rng.random((n, t.nq)) < QX).astype(np.uint8)
    ez = (rng.random((n, t.nq)) < QZ).astype(np.uint8)
    ex[0] = 0
    ez[0] = 0
    sx, sz = oracle.syndrome_extraction(ex, ez, t)
    return np.concatenate([sx, sz], axis=1).astype(np.uint8)


def _expected(t, lx, lz, bits):
    nsx = t.stgx.ns
    return np.stack([enumerator_marginal(t.stgx.H, t.stgz.H, lx, lz, QX, QZ, b[:nsx], b[nsx:]) for b in bits])


def _close(got, want):
    scale = want.max(axis=1, keepdims=True)
    err = np.abs(got - want) / scale
    assert err.max() <= 1e-10, f"max relative error {err.max():.3e}"


def test_enumerator_matches_pauli_enumeration_d3(oracle):
    t = _code(oracle, "surface", 3)
    lx, lz = oracle.logical_operator(t)
    px, py, pz = _independent_rates(t.nq)
    brute = oracle.brute_force_marginals(t, px, py, pz, lx, lz)
    ns = t.ns
    bits = ((np.arange(1 << ns)[:, None] >> np.arange(ns)[None, :]) & 1).astype(np.uint8)
    want = _expected(t, lx, lz, bits)
    _close(brute[oracle.syndrome_index(bits)], want)


@pytest.mark.parametrize("kind,d,n", [("surface", 5, 6), ("surface", 7, 3), ("toric", 4, 4), ("666", 5, 6)])
def test_oracle_contraction_matches_enumerator(oracle, kind, d, n):
    t = _code(oracle, kind, d)
    lx, lz = oracle.logical_operator(t)
    bits = _syndromes(oracle, t, n, seed=100 + d)
    want = _expected(t, lx, lz, bits)
    px, py, pz = _independent_rates(t.nq)
    got = oracle.OracleDecoder(t, px, py, pz).marginals(bits)
    _close(got, want)


def _package_graph(pkg, kind, d):
    code = {"surface": lambda: pkg.SurfaceCode(d, d), "toric": lambda: pkg.ToricCode(d, d),
            "666": lambda: pkg.Color666(d)}[kind]()
    t = pkg.tanner_graph(code)
    px, py, pz = _independent_rates(t.nq)
    em = pkg.IndependentDepolarizingError(px, py, pz)
    lx, lz = pkg.logical_operator(t)
    return t, lx, lz, pkg.tnmmap_css_graph(t, em, lx, lz)


@pytest.mark.parametrize("kind,d,n", [("surface", 5, 6), ("surface", 7, 3), ("toric", 4, 3)])
def test_planner_program_matches_enumerator(pkg, oracle, kind, d, n):
    """The compiled program the CUDA kernel receives (steps, folded
    constants, select tables, layouts), run in float64 by the emulator."""
    t, lx, lz, g = _package_graph(pkg, kind, d)
    ot = _code(oracle, kind, d)
    np.testing.assert_array_equal(t.stgx.H, ot.stgx.H)
    np.testing.assert_array_equal(t.stgz.H, ot.stgz.H)
    steps = pkg.optimize_code(g, pkg.TreeSA(trials=4, sweeps=200))
    plan = pkg.native.inspect_plan(g, steps)
    bits = _syndromes(oracle, ot, n, seed=200 + d)
    got = run_plan(plan, bits)
    _close(got, _expected(ot, lx, lz, bits))


def test_c_contractor_matches_enumerator_d7(pkg, oracle):
    """The float64 C contractor: the comparator of the GPU parity tests and
    the timed CPU baseline."""
    from oracle.c_oracle import CContractor

    t, lx, lz, g = _package_graph(pkg, "surface", 7)
    ot = _code(oracle, "surface", 7)
    steps = pkg.optimize_code(g, pkg.TreeSA(trials=4, sweeps=200))
    cc = CContractor(g.ixs, [np.asarray(x) for x in g.tensors], g.iy, g.syndrome_positions, steps)
    bits = _syndromes(oracle, ot, 4, seed=307)
    marg, cls = cc.contract(pkg.pack_syndromes(bits))
    want = _expected(ot, lx, lz, bits)
    _close(marg, want)
    np.testing.assert_array_equal(cls, [oracle.julia_findmax(w) for w in want])
