"""GF(2) linear algebra on bit-packed rows.

Rows are Python ints (bit j = column j, 0-based).  The elimination order is
the reference's own (src/codes/gaussian_elimination.jl:32-96): the logical
operators it yields fix TensorQEC's class labels, so ``logical_operator``
must reproduce them exactly, not merely span the same space.
"""
from __future__ import annotations

import numpy as np


def rows_from_matrix(M) -> list[int]:
    M = np.asarray(M).astype(np.uint8) & 1
    out = []
    for r in M:
        v = 0
        for j in np.flatnonzero(r):
            v |= 1 << int(j)
        out.append(v)
    return out


def matrix_from_rows(rows, ncols) -> np.ndarray:
    M = np.zeros((len(rows), ncols), dtype=np.uint8)
    for i, r in enumerate(rows):
        j = 0
        while r:
            if r & 1:
                M[i, j] = 1
            r >>= 1
            j += 1
    return M


def _swap_bits(v: int, i: int, j: int) -> int:
    bi = (v >> i) & 1
    bj = (v >> j) & 1
    if bi != bj:
        v ^= (1 << i) | (1 << j)
    return v


class BitMatrix:
    """A binary matrix with the row-operation record ``Q`` and the column
    ``ordering`` of TensorQEC's SimpleBimatrix / CSSBimatrix
    (src/codes/encoder.jl:14-33).  ``css_qubits`` set means columns q and
    css_qubits + q swap together (the CSS form)."""

    def __init__(self, rows, ncols, css_qubits=None, xcodenum=0):
        self.rows = list(rows)
        self.ncols = ncols
        self.q = [1 << i for i in range(len(self.rows))]
        n_ord = ncols if css_qubits is None else css_qubits
        self.ordering = list(range(n_ord))
        self.css_qubits = css_qubits
        self.xcodenum = xcodenum

    def switch_qubits(self, i: int, j: int):
        """gaussian_elimination.jl:1-15 (0-based i, j)."""
        o = self.ordering
        o[i], o[j] = o[j], o[i]
        n = self.css_qubits
        for r in range(len(self.rows)):
            v = _swap_bits(self.rows[r], i, j)
            if n is not None:
                v = _swap_bits(v, n + i, n + j)
            self.rows[r] = v

    def eliminate(self, r0: int, r1: int, col_offset: int, qubit_offset: int,
                  allow_col_operation: bool = True):
        """gaussian_elimination!(bimat, r0:r1, col_offset, qubit_offset),
        gaussian_elimination.jl:32-96, with 0-based inclusive rows r0..r1."""
        rows = self.rows
        start = col_offset + qubit_offset  # 0-based first column
        zero_row = 0
        zero_col = 0
        for i in range(r0, r1 + 1):
            if allow_col_operation:
                offset = i - r0 - zero_row
                tail = rows[i] >> start
                if tail == 0:
                    zero_row += 1
                    continue
                j = (tail & -tail).bit_length() - 1          # first nonzero, relative
                self.switch_qubits(qubit_offset + offset, j + qubit_offset)
            else:
                # column i + zero_col (0-based), searched from row i down
                if i + zero_col >= self.ncols:
                    return self
                col = i + zero_col
                piv = next((r for r in range(i, len(rows)) if (rows[r] >> col) & 1), None)
                while piv is None:
                    zero_col += 1
                    col = i + zero_col
                    if col >= self.ncols:
                        return self
                    piv = next((r for r in range(i, len(rows)) if (rows[r] >> col) & 1), None)
                if piv != i:
                    rows[i], rows[piv] = rows[piv], rows[i]
                    self.q[i], self.q[piv] = self.q[piv], self.q[i]
                offset = i - r0 + zero_col
            c = offset + start
            for k in range(r0, r1 + 1):
                if k != i and (rows[k] >> c) & 1:
                    rows[k] ^= rows[i]
                    self.q[k] ^= self.q[i]
        return self


def row_echelon_form(H) -> np.ndarray:
    """code_distance.jl:24-28."""
    H = np.asarray(H)
    m, n = H.shape
    b = BitMatrix(rows_from_matrix(H), n)
    b.eliminate(0, m - 1, 0, 0, allow_col_operation=False)
    return matrix_from_rows(b.rows, n)


def null_space(H) -> np.ndarray:
    """code_distance.jl:30-51: one basis vector per non-pivot column."""
    H = np.asarray(H)
    m, n = H.shape
    b = BitMatrix(rows_from_matrix(H), n)
    b.eliminate(0, m - 1, 0, 0, allow_col_operation=False)
    pivots = []
    for r in b.rows:
        if r:
            pivots.append((r & -r).bit_length() - 1)
    pset = set(pivots)
    out = []
    for j in range(n):
        if j in pset:
            continue
        v = 1 << j
        for i, p in enumerate(pivots):
            if (b.rows[i] >> j) & 1:
                v |= 1 << p
        out.append(v)
    return matrix_from_rows(out, n)


def _logical_pair(Hx: np.ndarray, Hz: np.ndarray) -> np.ndarray:
    """code_distance.jl:53-64."""
    n = Hx.shape[1]
    ker = rows_from_matrix(null_space(Hx))
    rows = rows_from_matrix(Hz) + ker
    b = BitMatrix(rows, n)
    b.eliminate(0, len(rows) - 1, 0, 0)
    lz = [r for r in b.rows[Hz.shape[0]:] if r]
    out = []
    for r in lz:
        v = 0
        for c in range(n):  # lz[:, ordering] = lz  (column c moves to ordering[c])
            if (r >> c) & 1:
                v |= 1 << b.ordering[c]
        out.append(v)
    return matrix_from_rows(out, n)


def _same_qubit_order(lx: np.ndarray, lz: np.ndarray):
    """code_distance.jl:84-100."""
    lxc = lx.copy()
    lx_new = np.zeros_like(lx)
    for j in range(lz.shape[0]):
        hits = [i for i in range(lxc.shape[0]) if int(lxc[i].astype(np.int64) @ lz[j]) % 2 == 1]
        if not hits:
            raise ValueError("the logical operators are linearly dependent")
        lx_new[j] = lxc[hits[0]]
        for i in hits[1:]:
            lxc[i] ^= lxc[hits[0]]
    return lx_new, lz


def logical_operator(tanner):
    """logical_operator(tanner::CSSTannerGraph), code_distance.jl:78-82.
    Returns (lx, lz) as uint8 arrays of shape (k, nq)."""
    hx = tanner.stgx.H
    hz = tanner.stgz.H
    lz = _logical_pair(hx, hz)
    lx = _logical_pair(hz, hx)
    return _same_qubit_order(lx, lz)


def solve_particular(H: np.ndarray):
    """A right-inverse map for H (m x n over GF(2)): returns a function that
    maps a syndrome s (length m) to one e with H e = s, or None when s is
    outside the column space.  Replaces the reference's integer-programming
    call that only needs *some* syndrome-consistent error
    (src/decoding/ipdecoder.jl:150-169)."""
    H = np.asarray(H).astype(np.uint8)
    m, n = H.shape
    # eliminate on [H | I] by rows, recording pivots
    rows = rows_from_matrix(H)
    rec = [1 << i for i in range(m)]
    pivots = []
    r = 0
    for c in range(n):
        piv = next((k for k in range(r, m) if (rows[k] >> c) & 1), None)
        if piv is None:
            continue
        rows[r], rows[piv] = rows[piv], rows[r]
        rec[r], rec[piv] = rec[piv], rec[r]
        for k in range(m):
            if k != r and (rows[k] >> c) & 1:
                rows[k] ^= rows[r]
                rec[k] ^= rec[r]
        pivots.append(c)
        r += 1
        if r == m:
            break
    rank = r
    piv_rows = rec[:rank]
    null_checks = rec[rank:]

    def particular(s):
        sv = 0
        for i in np.flatnonzero(np.asarray(s).astype(np.uint8) & 1):
            sv |= 1 << int(i)
        for c in null_checks:
            if bin(c & sv).count("1") & 1:
                return None
        e = np.zeros(n, dtype=np.uint8)
        for i, c in enumerate(pivots):
            if bin(piv_rows[i] & sv).count("1") & 1:
                e[c] = 1
        return e

    return particular


def remove_linear_dependency_rows(x_rows, z_rows, nq):
    """remove_linear_dependency (code_distance.jl:300-304) over the CSS
    bimatrix of stabilizers2bimatrix (encoder.jl:40-47) and the CSS
    elimination (gaussian_elimination.jl:97-102).  Inputs are bit rows over
    nq qubits; returns the indices (into x_rows + z_rows) that are kept."""
    rows = list(x_rows) + [r << nq for r in z_rows]
    b = BitMatrix(rows, 2 * nq, css_qubits=nq, xcodenum=len(x_rows))
    b.eliminate(0, b.xcodenum - 1, 0, 0)
    b.eliminate(b.xcodenum, len(rows) - 1, nq, b.xcodenum)
    return [i for i, r in enumerate(b.rows) if r]


def right_inverse(H: np.ndarray):
    """(R, C) over GF(2) for an m x n matrix H: R (n x m) maps every
    reachable syndrome s to an e = R s with H e = s; the rows of C (r x m)
    all have even overlap with s exactly when s is reachable."""
    H = np.asarray(H).astype(np.uint8)
    m, n = H.shape
    rows = rows_from_matrix(H)
    rec = [1 << i for i in range(m)]
    pivots = []
    r = 0
    for c in range(n):
        piv = next((k for k in range(r, m) if (rows[k] >> c) & 1), None)
        if piv is None:
            continue
        rows[r], rows[piv] = rows[piv], rows[r]
        rec[r], rec[piv] = rec[piv], rec[r]
        for k in range(m):
            if k != r and (rows[k] >> c) & 1:
                rows[k] ^= rows[r]
                rec[k] ^= rec[r]
        pivots.append(c)
        r += 1
        if r == m:
            break
    R = np.zeros((n, m), dtype=np.uint8)
    for i, c in enumerate(pivots):
        R[c] = matrix_from_rows([rec[i]], m)[0]
    C = matrix_from_rows(rec[r:], m) if r < m else np.zeros((0, m), dtype=np.uint8)
    return R, C
