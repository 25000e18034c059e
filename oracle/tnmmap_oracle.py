"""CPU oracle for the TNMMAP decoder path (test infrastructure only).

This module is the oracle, never the product: only the tests, the smoke
entry point and the CPU-baseline leg of the benchmark may import it.  It is a
plain numpy restatement of TensorQEC.jl's tensor-network marginal-MAP decoder,
written line by line from the reference sources (paths below are relative to
the TensorQEC.jl project root):

* code construction     -- src/codes/codes.jl:37-66 (rotated surface),
                           :184-244 (bivariate bicycle / toric),
                           :256-421 (4.8.8 and 6.6.6 colour codes)
* Tanner graphs          -- src/codes/ldpc.jl:44-52, :101-115
* GF(2) elimination      -- src/codes/gaussian_elimination.jl:1-15, :32-102
* logical operators      -- src/codes/code_distance.jl:24-100, :300-304
* stabiliser bimatrix    -- src/codes/encoder.jl:40-47
* error model / syndrome -- src/decoding/error_model.jl:97-181
* TNMMAP network         -- src/decoding/tndecoder.jl:42-44, :97-174
* DEM network            -- src/decoding/tndecoder.jl:186-271,
                           src/decoding/dem.jl:150-160,
                           src/stim_parser/stim_parser.jl:342-375
* TNMAP (most probable   -- src/decoding/tndecoder.jl:33-57,
  configuration)           src/decoding/general_decoding.jl:24-32

The contraction itself lives in OMEinsum (a Julia dependency, compat "0.9",
not vendored with the reference).  Its published semantics are plain einsum:
the output is the sum over all non-output labels of the product of all
tensors.  ``contract`` below evaluates that sum pairwise in float64 along a
greedy order of its own; any order gives the same value up to rounding.

Parity of this oracle is pinned against the reference's own known answers
(``tests/golden/reference_kat.json``): the zero-syndrome d=3 marginal of
test/decoding/tndecoder.jl:101-110, the parity tensor entries of
test/decoding/tndecoder.jl:8-14, the d=3 logical operators of
test/codes/code_distance.jl:54-59, the row-echelon form of
test/codes/code_distance.jl:18-39 and the toric stabilisers of
test/codes/codes.jl:5-22; plus a brute-force enumeration over all 4^9 Pauli
errors at d=3 that is independent of any contraction order.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field

import numpy as np

# ---------------------------------------------------------------------------
# Codes (src/codes/codes.jl)
# ---------------------------------------------------------------------------


def surface_code_stabilizers(m: int, n: int):
    """Rotated surface code stabilisers, codes.jl:37-66.

    Returns a list of ('X'|'Z', sorted 1-based qubit tuple) in the
    reference's push order.  ``qubit_config = reshape(1:m*n, n, m)'`` means
    qubit (i, j) (1-based row i, column j) is ``(i-1)*n + j``.
    """
    q = lambda i, j: (i - 1) * n + j  # noqa: E731
    out = []
    for i in range(1, m):            # for i in 1:m-1, j in 1:n-1 (j fastest)
        for j in range(1, n):
            if (i + j) % 2 == 0:
                out.append(("X", (q(i, j), q(i + 1, j), q(i, j + 1), q(i + 1, j + 1))))
    for i in range(1, m // 2 + 1):
        if 2 * i + (n + 1) % 2 <= m:
            out.append(("X", (q(2 * i - 1 + (n + 1) % 2, n), q(2 * i + (n + 1) % 2, n))))
        if 2 * i + 1 <= m:
            out.append(("X", (q(2 * i, 1), q(2 * i + 1, 1))))
    for i in range(1, m):
        for j in range(1, n):
            if (i + j) % 2 == 1:
                out.append(("Z", (q(i, j), q(i + 1, j), q(i, j + 1), q(i + 1, j + 1))))
    for j in range(1, n // 2 + 1):
        out.append(("Z", (q(1, 2 * j - 1), q(1, 2 * j))))
        if 2 * j + m % 2 <= n:
            out.append(("Z", (q(m, 2 * j - 1 + m % 2), q(m, 2 * j + m % 2))))
    return [(t, tuple(sorted(s))) for t, s in out], m * n


def _mod1(i, m):
    return (i - 1) % m + 1


def bivariate_bicycle_stabilizers(m, n, vc, hd, rm_linear_dependency=True):
    """codes.jl:190-227.  Vertical edges are 1..m*n, horizontal m*n+1..2m*n,
    both column-major ``reshape(1:m*n, m, n)``."""
    nsite = m * n
    nq = 2 * nsite
    ve = lambda i, j: (j - 1) * m + i  # noqa: E731
    he = lambda i, j: nsite + (j - 1) * m + i  # noqa: E731
    out = []
    for j in range(1, n + 1):          # for j in 1:n, i in 1:m (i fastest)
        for i in range(1, m + 1):
            st = [ve(_mod1(i + s, m), _mod1(j + t, n)) for (s, t) in hd]
            st += [he(_mod1(i + s, m), _mod1(j + t, n)) for (s, t) in vc]
            out.append(("X", tuple(sorted(set(st)))))
    for j in range(1, n + 1):
        for i in range(1, m + 1):
            st = [ve(_mod1(i - s, m), _mod1(j - t, n)) for (s, t) in vc]
            st += [he(_mod1(i - s, m), _mod1(j - t, n)) for (s, t) in hd]
            out.append(("Z", tuple(sorted(set(st)))))
    if rm_linear_dependency:
        out = remove_linear_dependency(out, nq)
    return out, nq


def toric_code_stabilizers(m, n):
    """``ToricCode(m,n) = BivariateBicycleCode(m,n,((1,0),(0,0)),((0,1),(0,0)))``,
    codes.jl:244."""
    return bivariate_bicycle_stabilizers(m, n, ((1, 0), (0, 0)), ((0, 1), (0, 0)))


def _color488_checks(d):
    """codes.jl:256-334 restated (1-based column indices)."""
    n = (d * d + 2 * d - 1) // 2
    num_checks = (n - 1) // 2
    num_layers = (d - 1) // 2
    checks = np.zeros((num_checks, n + 1), dtype=bool)  # column 0 unused
    i = 1
    cw = 0
    for layer in range(1, num_layers + 1):
        num_8 = layer - 1
        cw -= num_8
        for j in range(1, num_8 + 1):
            checks[cw, i + 2 * layer + 1 + (j - 1) * 2] = 1
            checks[cw, i + 2 * layer + j * 2] = 1
            off = 1 if (layer == num_layers and num_layers % 2 == 0) else 0
            checks[cw, (2 * layer + 1) + i + 2 * layer + 1 + (j - 1) * 2 - off] = 1
            checks[cw, (2 * layer + 1) + i + 2 * layer + j * 2 - off] = 1
            cw += 1
        for j in range(0, layer):
            checks[cw, i + j * 2] = 1
            checks[cw, i + 1 + j * 2] = 1
            checks[cw, i + 2 * layer + j * 2] = 1
            checks[cw, i + 2 * layer + 1 + j * 2] = 1
            cw += 1
        if layer % 2 == 1:
            checks[cw, i] = 1
            checks[cw, i + 2 * layer] = 1
            checks[cw, i + 4 * layer] = 1
            checks[cw, i + 4 * layer + 1] = 1
            cw += 1
        else:
            checks[cw, i + 1 + (layer - 1) * 2] = 1
            checks[cw, i + 2 * layer + 1 + (layer - 1) * 2] = 1
            off = 1 if layer == num_layers else 0
            checks[cw, (i + 4 * layer) + layer * 2 - off] = 1
            checks[cw, (i + 4 * layer) + 1 + layer * 2 - off] = 1
            cw += 1
        for j in range(0, layer):
            checks[cw, i + 2 * layer + j * 2] = 1
            checks[cw, i + 2 * layer + 1 + j * 2] = 1
            off = 1 if (layer == num_layers and num_layers % 2 == 0) else 0
            checks[cw, (2 * layer + 1) + i + 2 * layer + j * 2 - off] = 1
            checks[cw, (2 * layer + 1) + i + 2 * layer + 1 + j * 2 - off] = 1
            cw += 1
        i += 4 * layer
    return checks[:, 1:], n


def _color666_checks(d):
    """codes.jl:336-408 restated (1-based column indices)."""
    n = (3 * d * d + 1) // 4
    num_checks = (n - 1) // 2
    num_layers = (d - 1) // 2
    checks = np.zeros((num_checks, n + 1), dtype=bool)
    i = 1
    cw = 0
    for layer in range(1, num_layers + 1):
        num_6 = layer - 1
        cw -= num_6
        for j in range(1, num_6 + 1):
            init = i + 2 * (j - 1)
            checks[cw, init + 2 * (layer - 1) + 1] = 1
            checks[cw, init + 2 * (layer - 1) + 2] = 1
            cw += 1
        checks[cw, i] = 1
        checks[cw, i + (layer - 1) * 2 + 1] = 1
        checks[cw, i + 2 + 4 * (layer - 1)] = 1
        checks[cw, i + 2 + 4 * (layer - 1) + 1] = 1
        cw += 1
        checks[cw, i + 1 + 4 * (layer - 1)] = 1
        checks[cw, i + 1 + 4 * (layer - 1) + layer * 2] = 1
        checks[cw, i + 5 + 8 * (layer - 1)] = 1
        checks[cw, i + 5 + 8 * (layer - 1) + 1] = 1
        cw += 1
        for j in range(1, layer):
            b = i + (j - 1) * 2
            for c in (b + 1, b + 2, b + 2 + 2 * (layer - 1), b + 2 + 2 * (layer - 1) + 1,
                      b + 2 + 2 * (layer - 1) + layer * 2, b + 2 + 2 * (layer - 1) + layer * 2 + 1):
                checks[cw, c] = 1
            cw += 1
        for j in range(1, layer):
            init = i + (j - 1) * 2 + (layer - 1) * 2 + 1
            for c in (init, init + 1, init + 2 * layer, init + 2 * layer + 1,
                      init + 4 * layer, init + 4 * layer + 1):
                checks[cw, c] = 1
            cw += 1
        for j in range(0, layer):
            init = i + 2 * j + 2 + 4 * (layer - 1)
            for c in (init, init + 1, init + 2 * layer, init + 2 * layer + 1):
                checks[cw, c] = 1
            cw += 1
        i += 4 + 6 * (layer - 1)
    return checks[:, 1:], n


def color_code_stabilizers(kind: str, d: int):
    """TriangularColorCode stabilisers, codes.jl:410-421: all X checks then
    the same supports as Z checks."""
    checks, n = (_color488_checks if kind == "488" else _color666_checks)(d)
    out = [("X", tuple(int(c) + 1 for c in np.flatnonzero(row))) for row in checks]
    out += [("Z", tuple(int(c) + 1 for c in np.flatnonzero(row))) for row in checks]
    return out, n


# ---------------------------------------------------------------------------
# Tanner graphs (src/codes/ldpc.jl)
# ---------------------------------------------------------------------------


@dataclass
class TannerGraph:
    """SimpleTannerGraph, ldpc.jl:27-52 (s2q 1-based, H as uint8)."""
    nq: int
    s2q: list
    H: np.ndarray = field(init=False)

    def __post_init__(self):
        self.H = np.zeros((len(self.s2q), self.nq), dtype=np.uint8)
        for i, c in enumerate(self.s2q):
            for q in c:
                self.H[i, q - 1] = 1

    @property
    def ns(self):
        return len(self.s2q)


@dataclass
class CSSTanner:
    """CSSTannerGraph, ldpc.jl:72-115."""
    stgx: TannerGraph
    stgz: TannerGraph

    @property
    def nq(self):
        return self.stgx.nq

    @property
    def ns(self):
        return self.stgx.ns + self.stgz.ns


def css_tanner(stabs, nq):
    """ldpc.jl:105-111: X-type checks in order, then Z-type checks."""
    xs = [list(s) for t, s in stabs if t == "X"]
    zs = [list(s) for t, s in stabs if t == "Z"]
    return CSSTanner(TannerGraph(nq, xs), TannerGraph(nq, zs))


# ---------------------------------------------------------------------------
# GF(2) elimination (src/codes/gaussian_elimination.jl, code_distance.jl)
# ---------------------------------------------------------------------------


class Bimatrix:
    """SimpleBimatrix / CSSBimatrix, encoder.jl:14-33 (matrix is bool,
    Q is the row-operation record, ordering 1-based)."""

    def __init__(self, matrix, ordering=None, Q=None, css_qubits=None, xcodenum=0):
        self.matrix = np.array(matrix, dtype=bool)
        nr = self.matrix.shape[0]
        self.Q = np.eye(nr, dtype=bool) if Q is None else np.array(Q, dtype=bool)
        ncols = self.matrix.shape[1]
        nord = ncols if css_qubits is None else css_qubits
        self.ordering = list(range(1, nord + 1)) if ordering is None else list(ordering)
        self.css_qubits = css_qubits
        self.xcodenum = xcodenum

    def switch_qubits(self, i, j):
        """gaussian_elimination.jl:1-15 (1-based i, j)."""
        o = self.ordering
        o[i - 1], o[j - 1] = o[j - 1], o[i - 1]
        M = self.matrix
        M[:, [i - 1, j - 1]] = M[:, [j - 1, i - 1]]
        if self.css_qubits is not None:
            q = self.css_qubits
            M[:, [q + i - 1, q + j - 1]] = M[:, [q + j - 1, q + i - 1]]


def gaussian_elimination(b: Bimatrix, rows, col_offset, qubit_offset, allow_col_operation=True):
    """gaussian_elimination.jl:32-96.  ``rows`` is a 1-based inclusive
    (start, stop) pair, like Julia's UnitRange."""
    r0, r1 = rows
    M = b.matrix
    ncol = M.shape[1]
    start_col = col_offset + qubit_offset + 1
    zero_row = 0
    zero_col = 0
    for i in range(r0, r1 + 1):
        if allow_col_operation:
            offset = i - r0 - zero_row
            nz = np.flatnonzero(M[i - 1, start_col - 1:])
            if nz.size == 0:
                zero_row += 1
                continue
            j = int(nz[0]) + 1
            b.switch_qubits(qubit_offset + offset + 1, j + qubit_offset)
        else:
            if i + zero_col > ncol:
                return b
            col = M[i - 1:, i + zero_col - 1]
            nz = np.flatnonzero(col)
            while nz.size == 0:
                zero_col += 1
                if i + zero_col > ncol:
                    return b
                nz = np.flatnonzero(M[i - 1:, i + zero_col - 1])
            j = i + int(nz[0])
            if j != i:
                b.Q[[i - 1, j - 1], :] = b.Q[[j - 1, i - 1], :]
                M[[i - 1, j - 1], :] = M[[j - 1, i - 1], :]
            offset = i - r0 + zero_col
        for k in range(r0, r1 + 1):
            if k != i and M[k - 1, offset + start_col - 1]:
                M[k - 1, :] ^= M[i - 1, :]
                b.Q[k - 1, :] ^= b.Q[i - 1, :]
    return b


def row_echelon_form(H):
    """code_distance.jl:24-28."""
    b = Bimatrix(H)
    gaussian_elimination(b, (1, b.matrix.shape[0]), 0, 0, allow_col_operation=False)
    return b.matrix


def null_space(H):
    """code_distance.jl:30-51."""
    H = np.array(H, dtype=bool)
    reH = row_echelon_form(H)
    m, n = H.shape
    pivots = []
    for i in range(m):
        nz = np.flatnonzero(reH[i])
        if nz.size:
            pivots.append(int(nz[0]))
    rank = len(pivots)
    ns = np.zeros((n - rank, n), dtype=bool)
    rc = 0
    for j in range(n):
        if j not in pivots:
            ns[rc, j] = True
            for i, p in enumerate(pivots):
                if reH[i, j]:
                    ns[rc, p] = True
            rc += 1
    return ns


def _logical_operator_pair(Hx, Hz):
    """code_distance.jl:53-64."""
    kerHx = null_space(Hx)
    H = np.vstack([np.array(Hz, dtype=bool), kerHx])
    b = gaussian_elimination(Bimatrix(H), (1, H.shape[0]), 0, 0)
    lz = b.matrix[Hz.shape[0]:, :]
    lz = lz[lz.any(axis=1)]
    out = np.zeros_like(lz)
    out[:, np.array(b.ordering) - 1] = lz
    return out.astype(np.uint8)


def _same_qubit_order(lx, lz):
    """code_distance.jl:84-100."""
    lx_new = np.zeros_like(lx)
    lxc = lx.copy()
    for j in range(lz.shape[0]):
        hits = [i for i in range(lxc.shape[0]) if (int(lxc[i] @ lz[j]) % 2) == 1]
        assert hits, "The logical operator is linearly dependent!"
        lx_new[j] = lxc[hits[0]]
        for i in hits[1:]:
            lxc[i] = (lxc[i] + lxc[hits[0]]) % 2
    return lx_new, lz


def logical_operator(t: CSSTanner):
    """code_distance.jl:78-82: returns (lx, lz) as uint8 k x nq."""
    hx = t.stgx.H.astype(bool)
    hz = t.stgz.H.astype(bool)
    lz = _logical_operator_pair(hx, hz)
    lx = _logical_operator_pair(hz, hx)
    return _same_qubit_order(lx, lz)


def remove_linear_dependency(stabs, nq):
    """code_distance.jl:300-304 over stabilizers2bimatrix (encoder.jl:40-47)
    and the CSS elimination (gaussian_elimination.jl:97-102)."""
    xs = [s for s in stabs if s[0] == "X"]
    zs = [s for s in stabs if s[0] == "Z"]
    assert len(xs) + len(zs) == len(stabs)
    A = np.zeros((len(xs), nq), dtype=bool)
    B = np.zeros((len(zs), nq), dtype=bool)
    for r, (_, s) in enumerate(xs):
        A[r, np.array(s) - 1] = True
    for r, (_, s) in enumerate(zs):
        B[r, np.array(s) - 1] = True
    M = np.zeros((len(stabs), 2 * nq), dtype=bool)
    M[: len(xs), :nq] = A
    M[len(xs):, nq:] = B
    b = Bimatrix(M, css_qubits=nq, xcodenum=len(xs))
    gaussian_elimination(b, (1, b.xcodenum), 0, 0)
    gaussian_elimination(b, (b.xcodenum + 1, M.shape[0]), nq, b.xcodenum)
    keep = b.matrix.any(axis=1)
    return [s for s, k in zip(stabs, keep) if k]


# ---------------------------------------------------------------------------
# Error model (src/decoding/error_model.jl)
# ---------------------------------------------------------------------------


def sample_depolarizing(rng: np.random.Generator, px, py, pz, nsamples):
    """error_model.jl:97-117: one uniform per qubit; Y if r<py, X if
    r<px+py, Z if r<px+py+pz.  Returns (ex, ez) uint8 arrays (nsamples, nq).
    The uniform stream is numpy's, not Julia's."""
    px, py, pz = (np.asarray(v, dtype=np.float64) for v in (px, py, pz))
    r = rng.random((nsamples, px.size))
    y = r < py
    x = (~y) & (r < px + py)
    z = (~y) & (~x) & (r < px + py + pz)
    return (x | y).astype(np.uint8), (z | y).astype(np.uint8)


def syndrome_extraction(ex, ez, t: CSSTanner):
    """error_model.jl:131-146: sx = Hx*ez, sz = Hz*ex (mod 2)."""
    sx = (np.atleast_2d(ez).astype(np.int64) @ t.stgx.H.T.astype(np.int64)) % 2
    sz = (np.atleast_2d(ex).astype(np.int64) @ t.stgz.H.T.astype(np.int64)) % 2
    return sx.astype(np.uint8), sz.astype(np.uint8)


def check_logical_error(ex1, ez1, ex2, ez2, lx, lz):
    """error_model.jl:161-181."""
    dz = (np.asarray(ez1) + np.asarray(ez2)) % 2
    dx = (np.asarray(ex1) + np.asarray(ex2)) % 2
    return bool(((lx.astype(np.int64) @ dz) % 2).any() or ((lz.astype(np.int64) @ dx) % 2).any())


# ---------------------------------------------------------------------------
# Network construction (src/decoding/tndecoder.jl)
# ---------------------------------------------------------------------------


def parity_check_matrix(q):
    """tndecoder.jl:42-44: rank q+1, entry 1 where the index sum is even."""
    idx = np.indices((2,) * (q + 1)).sum(axis=0)
    return (1 - idx % 2).astype(np.float64)


@dataclass
class Network:
    ixs: list            # list of lists of 1-based variable labels
    tensors: list        # numpy float64 arrays, axis j <-> ixs[j]
    iy: list             # output labels
    syndrome_positions: list  # tensor positions (0-based) of the one-hot leaves


def tnmmap_network(t: CSSTanner, px, py, pz, lx=None, lz=None):
    """compile(::TNMMAP, ::IndependentDepolarizingDecodingProblem),
    tndecoder.jl:97-146 (without the order optimisation)."""
    nq = t.nq
    if lx is None:
        lx, lz = logical_operator(t)
    lxs = [list(np.flatnonzero(r) + 1) for r in lx]
    lzs = [list(np.flatnonzero(r) + 1) for r in lz]
    ns = t.ns
    k = lx.shape[0]
    nvars = 2 * nq + ns + k + lz.shape[0]
    ixs, tensors = [], []
    for i, c in enumerate(t.stgx.s2q, 1):
        ixs.append([q + nq for q in c] + [i + 2 * nq])
        tensors.append(parity_check_matrix(len(c)))
    for i, c in enumerate(t.stgz.s2q, 1):
        ixs.append(list(c) + [i + 2 * nq + t.stgx.ns])
        tensors.append(parity_check_matrix(len(c)))
    px, py, pz = (np.broadcast_to(np.asarray(v, dtype=np.float64), (nq,)) for v in (px, py, pz))
    for i in range(1, nq + 1):
        a, b, c = px[i - 1], py[i - 1], pz[i - 1]
        ixs.append([i, i + nq])
        tensors.append(np.array([[1 - a - b - c, c], [a, b]], dtype=np.float64))
    for i, il in enumerate(lzs, 1):
        ixs.append([int(v) for v in il] + [i + 2 * nq + ns + lz.shape[0]])
        tensors.append(parity_check_matrix(len(il)))
    for i, il in enumerate(lxs, 1):
        ixs.append([int(v) + nq for v in il] + [i + 2 * nq + ns])
        tensors.append(parity_check_matrix(len(il)))
    synd_pos = []
    for v in range(2 * nq + 1, 2 * nq + ns + 1):
        synd_pos.append(len(ixs))
        ixs.append([v])
        tensors.append(np.array([1.0, 0.0]))
    iy = list(range(2 * nq + ns + 1, nvars + 1))
    return Network(ixs, tensors, iy, synd_pos)


def update_syndrome(net: Network, bits):
    """tndecoder.jl:148-158 / :240-246: one-hot leaves, sx bits then sz."""
    tensors = list(net.tensors)
    for p, s in zip(net.syndrome_positions, bits):
        tensors[p] = np.array([0.0, 1.0]) if s else np.array([1.0, 0.0])
    return tensors


# ---------------------------------------------------------------------------
# DEM path (stim_parser.jl, dem.jl, tndecoder.jl:186-271)
# ---------------------------------------------------------------------------


@dataclass
class DEM:
    error_rates: list
    flipped: list          # 1-based detector ids, logicals renumbered after detectors
    detector_list: list
    logical_list: list


def parse_dem_string(content: str) -> DEM:
    """stim_parser.jl:342-375."""
    rates, dets, logs = [], [], []
    for line in content.split("\n"):
        if not line:
            continue
        s = line.split()
        if s[0].startswith("error("):
            rates.append(float(s[0][6:-1]))
            d = [int(x[1:]) + 1 for x in s[1:] if x.startswith("D")]
            lg = [int(x[1:]) + 1 for x in s[1:] if x.startswith("L")]
            dets.append(d)
            logs.append(lg)
        elif s[0].startswith("repeat"):
            raise ValueError("repeat is not supported")
    largest = max(max(d) for d in dets if d)
    logs = [[x + largest for x in lg] for lg in logs]
    largest_l = max((max(lg) if lg else 0) for lg in logs)
    flipped = [sorted(set(d) | set(lg), key=(d + lg).index) for d, lg in zip(dets, logs)]
    return DEM(rates, flipped, list(range(1, largest + 1)), list(range(largest + 1, largest_l + 1)))


def dem2tanner(dem: DEM) -> TannerGraph:
    """dem.jl:150-160."""
    nq = len(dem.error_rates)
    q2s = [[v for v in f if v not in dem.logical_list] for f in dem.flipped]
    ns = max(dem.detector_list)
    s2q = [[j + 1 for j in range(nq) if i in q2s[j]] for i in range(1, ns + 1)]
    return TannerGraph(nq, s2q)


def _push_check_node(ixs, tensors, c, node, nvars, factorize):
    """tndecoder.jl:221-238 (a check over fewer than three bits is one
    parity tensor: the reference's chain fails on a single-bit check)."""
    L = len(c)
    if not factorize or L <= 2:
        ixs.append(list(c) + [node])
        tensors.append(parity_check_matrix(L))
    else:
        ixs.append([c[0], c[1], nvars + 1])
        tensors.append(parity_check_matrix(2))
        for j in range(3, L):
            ixs.append([nvars + j - 1, c[j - 1], nvars + j - 2])
            tensors.append(parity_check_matrix(2))
        ixs.append([node, c[L - 1], nvars + L - 2])
        tensors.append(parity_check_matrix(2))
        nvars += L - 2
    return nvars


def dem_network(dem: DEM, factorize=True):
    """compile(::TNMMAP, ::DetectorErrorModel), tndecoder.jl:186-219."""
    t = dem2tanner(dem)
    l2q = [[j + 1 for j, f in enumerate(dem.flipped) if i in f] for i in dem.logical_list]
    nq, ns = t.nq, t.ns
    nvars = nq + ns + len(dem.logical_list)
    iy = list(range(nq + ns + 1, nvars + 1))
    ixs, tensors = [], []
    for i, c in enumerate(t.s2q, 1):
        nvars = _push_check_node(ixs, tensors, c, i + nq, nvars, factorize)
    for i, c in enumerate(l2q, 1):
        nvars = _push_check_node(ixs, tensors, c, i + nq + ns, nvars, factorize)
    for i, p in enumerate(dem.error_rates, 1):
        ixs.append([i])
        tensors.append(np.array([1 - p, p]))
    synd = []
    for v in range(nq + 1, nq + ns + 1):
        synd.append(len(ixs))
        ixs.append([v])
        tensors.append(np.array([1.0, 0.0]))
    return Network(ixs, tensors, iy, synd), t, l2q


# ---------------------------------------------------------------------------
# Contraction (OMEinsum semantics: sum over non-output labels of the product)
# ---------------------------------------------------------------------------


def greedy_order(ixs, iy, seed=None):
    """A greedy pairwise order of the oracle's own: repeatedly merge the pair
    of tensors sharing a label whose result is smallest relative to its
    inputs.  Returns [(a, b), ...] over node ids (leaves 0..n-1, step j makes
    node n+j)."""
    rng = np.random.default_rng(seed) if seed is not None else None
    nodes = {i: set(ix) for i, ix in enumerate(ixs)}
    out = set(iy)
    nid = len(ixs)
    steps = []

    def kept(a, b):
        u = nodes[a] | nodes[b]
        rest = set()
        for k, v in nodes.items():
            if k != a and k != b:
                rest |= v
        return {x for x in u if x in out or x in rest}

    while len(nodes) > 1:
        best = None
        keys = list(nodes)
        by_label = {}
        for k in keys:
            for x in nodes[k]:
                by_label.setdefault(x, []).append(k)
        cands = set()
        for lst in by_label.values():
            for i in range(len(lst)):
                for j in range(i + 1, len(lst)):
                    cands.add((min(lst[i], lst[j]), max(lst[i], lst[j])))
        if not cands:
            cands = {(keys[0], keys[1])}
        for a, b in sorted(cands):
            kp = kept(a, b)
            cost = 2.0 ** len(kp) - 2.0 ** len(nodes[a]) - 2.0 ** len(nodes[b])
            if rng is not None:
                cost += rng.random() * 1e-3
            if best is None or cost < best[0]:
                best = (cost, a, b, kp)
        _, a, b, kp = best
        del nodes[a], nodes[b]
        nodes[nid] = kp
        steps.append((a, b))
        nid += 1
    return steps


def contract(ixs, tensors, iy, order=None):
    """Float64 pairwise contraction.  Returns an array whose axes follow iy."""
    if order is None:
        order = greedy_order(ixs, iy)
    live = {i: (list(ix), np.asarray(t, dtype=np.float64)) for i, (ix, t) in enumerate(zip(ixs, tensors))}
    out = set(iy)
    nid = len(ixs)
    for a, b in order:
        ia, ta = live.pop(a)
        ib, tb = live.pop(b)
        rest = set()
        for v in live.values():
            rest |= set(v[0])
        union = list(dict.fromkeys(ia + ib))
        keep = [x for x in union if x in out or x in rest]
        lab = {x: i for i, x in enumerate(union)}
        tc = np.einsum(ta, [lab[x] for x in ia], tb, [lab[x] for x in ib], [lab[x] for x in keep])
        live[nid] = (keep, tc)
        nid += 1
    (ix, t), = live.values()
    # sum any label not in the output (only when nothing was merged)
    lab = {x: i for i, x in enumerate(dict.fromkeys(ix + list(iy)))}
    return np.einsum(t, [lab[x] for x in ix], [lab[x] for x in iy])


def julia_findmax(mar):
    """findmax over a Julia column-major array: first maximum in linear
    (first-index-fastest) order.  Returns the 0-based linear index."""
    flat = np.asarray(mar).flatten(order="F")
    return int(np.argmax(flat))


def marginal_column_major(mar):
    """The marginal flattened in Julia linear order (first index fastest)."""
    return np.asarray(mar).flatten(order="F")


class OracleDecoder:
    """compile + decode for TNMMAP over a CSS code, tndecoder.jl:97-174.
    ``marginals(bits)`` returns the unnormalised class marginal in Julia
    linear order for each syndrome row (sx bits then sz bits)."""

    def __init__(self, tanner: CSSTanner, px, py, pz, seed=None):
        self.tanner = tanner
        self.lx, self.lz = logical_operator(tanner)
        self.net = tnmmap_network(tanner, px, py, pz, self.lx, self.lz)
        self.order = greedy_order(self.net.ixs, self.net.iy, seed)

    def marginal(self, bits):
        ts = update_syndrome(self.net, bits)
        return marginal_column_major(contract(self.net.ixs, ts, self.net.iy, self.order))

    def marginals(self, syndromes):
        return np.stack([self.marginal(s) for s in np.atleast_2d(syndromes)])


class OracleDEMDecoder:
    """compile + decode for TNMMAP over a detector error model,
    tndecoder.jl:186-253."""

    def __init__(self, dem: DEM, factorize=True, seed=None):
        self.dem = dem
        self.net, self.tanner, self.l2q = dem_network(dem, factorize)
        self.order = greedy_order(self.net.ixs, self.net.iy, seed)

    def marginal(self, bits):
        ts = update_syndrome(self.net, bits)
        return marginal_column_major(contract(self.net.ixs, ts, self.net.iy, self.order))

    def marginals(self, syndromes):
        return np.stack([self.marginal(s) for s in np.atleast_2d(syndromes)])


def brute_force_marginals(tanner: CSSTanner, px, py, pz, lx, lz):
    """Exact class marginals for every syndrome by enumerating all 4^nq
    Pauli errors (small codes only).  Independent of any contraction: for
    each error, P(e) is added to mar[syndrome][class] where
    class = a + 2^k * b (Julia linear order of mar[a..., b...]),
    a_i = lx_i . ez, b_i = lz_i . ex."""
    nq = tanner.nq
    assert nq <= 12
    px, py, pz = (np.broadcast_to(np.asarray(v, dtype=np.float64), (nq,)) for v in (px, py, pz))
    n = 1 << nq
    bits = ((np.arange(n)[:, None] >> np.arange(nq)[None, :]) & 1).astype(np.uint8)
    ns_x, ns_z = tanner.stgx.ns, tanner.stgz.ns
    k = lx.shape[0]
    ncls = 1 << (2 * k)
    out = np.zeros((1 << (ns_x + ns_z), ncls), dtype=np.float64)
    # probability table per (ex, ez) via per-qubit factors
    p00 = 1 - px - py - pz
    for exi in range(n):
        ex = bits[exi]
        ez = bits  # all ez at once
        # per-qubit factor: ex=0,ez=0 -> p00, 0/1 -> pz, 1/0 -> px, 1/1 -> py
        f0 = np.where(ex[None, :] == 1, np.where(ez == 1, py, px), np.where(ez == 1, pz, p00))
        prob = np.prod(f0, axis=1)
        sz = (tanner.stgz.H.astype(np.int64) @ ex) % 2
        sx = (ez.astype(np.int64) @ tanner.stgx.H.T.astype(np.int64)) % 2
        a = (ez.astype(np.int64) @ lx.T.astype(np.int64)) % 2
        b = (lz.astype(np.int64) @ ex) % 2
        sidx = (sx * (1 << np.arange(ns_x))).sum(axis=1) + int((sz * (1 << (ns_x + np.arange(ns_z)))).sum())
        cidx = (a * (1 << np.arange(k))).sum(axis=1) + int((b * (1 << (k + np.arange(k)))).sum())
        np.add.at(out, (sidx, cidx), prob)
    return out


def syndrome_index(bits):
    """Integer id of a syndrome row (bit i of the row -> 2^i)."""
    bits = np.atleast_2d(bits).astype(np.int64)
    return (bits << np.arange(bits.shape[1])).sum(axis=1)


def contraction_cost(ixs, iy, order):
    """(multiply-adds, log2 of the largest intermediate) of a pairwise order."""
    nodes = {i: set(ix) for i, ix in enumerate(ixs)}
    out = set(iy)
    nid = len(ixs)
    macs = 0
    width = 0
    for a, b in order:
        sa, sb = nodes.pop(a), nodes.pop(b)
        rest = set()
        for v in nodes.values():
            rest |= v
        u = sa | sb
        keep = {x for x in u if x in out or x in rest}
        macs += 2 ** len(u)
        width = max(width, len(keep))
        nodes[nid] = keep
        nid += 1
    return macs, width


# ---------------------------------------------------------------------------
# TNMAP: most probable configuration (src/decoding/tndecoder.jl:33-57)
# ---------------------------------------------------------------------------


def most_probable_configs(H, prior_ixs, prior_tensors, syndromes):
    """The reference's TNMAP answer by enumeration: for each syndrome row,
    the maximum over all bit configurations e with H e = s (mod 2) of the
    product of the prior tensors (stg2uaimodel, tndecoder.jl:33-40, with the
    syndrome as evidence, :46-57; TensorInference's most_probable_config is a
    max-product contraction of that model).  Returns (natural log of the
    maximum, mask of all maximisers) per row; only for nq <= 22 bits.

    ``prior_tensors`` are flattened in Julia column-major order over their
    labels (1-based bits)."""
    H = np.asarray(H, dtype=np.int64)
    nq = H.shape[1]
    if nq > 22:
        raise ValueError("enumeration is limited to 22 bits")
    cfg = (np.arange(1 << nq, dtype=np.int64)[:, None] >> np.arange(nq)) & 1
    logw = np.zeros(1 << nq)
    with np.errstate(divide="ignore"):
        for ix, t in zip(prior_ixs, prior_tensors):
            flat = np.asarray(t, dtype=np.float64).ravel(order="F")
            idx = np.zeros(1 << nq, dtype=np.int64)
            for j, v in enumerate(ix):
                idx |= cfg[:, v - 1] << j
            logw += np.log(flat[idx])
    syn = (cfg @ H.T) % 2
    key = (syn * (1 << np.arange(H.shape[0]))).sum(1)
    out = []
    for s in np.atleast_2d(syndromes):
        k = int((np.asarray(s, dtype=np.int64) * (1 << np.arange(H.shape[0]))).sum())
        m = key == k
        best = logw[m].max() if m.any() else -np.inf
        out.append((best, cfg[m & (logw == best)] if np.isfinite(best) else cfg[:0]))
    return out


def config_log_probability(prior_ixs, prior_tensors, cfg):
    """Natural log of the product of the prior tensors at configurations
    ``cfg`` (rows of 0/1 over all bits)."""
    cfg = np.atleast_2d(np.asarray(cfg, dtype=np.int64))
    out = np.zeros(cfg.shape[0])
    with np.errstate(divide="ignore"):
        for ix, t in zip(prior_ixs, prior_tensors):
            flat = np.asarray(t, dtype=np.float64).ravel(order="F")
            idx = np.zeros(cfg.shape[0], dtype=np.int64)
            for j, v in enumerate(ix):
                idx |= cfg[:, v - 1] << j
            out += np.log(flat[idx])
    return out
