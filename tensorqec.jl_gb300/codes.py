"""Quantum codes and Tanner graphs (TensorQEC's src/codes/codes.jl, ldpc.jl).

Stabilisers are returned as ``PauliString`` values over 1-based qubits in the
reference's push order; ``CSSTannerGraph`` takes the X-type checks in order
as ``stgx`` and the Z-type checks as ``stgz`` (ldpc.jl:105-111), which fixes
the syndrome bit order ``[sx..., sz...]`` used everywhere downstream.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import gf2

_I, _X, _Y, _Z = 0, 1, 2, 3


@dataclass(frozen=True)
class PauliString:
    """A Pauli string over ``n`` qubits: ``ops[q]`` in {0:I, 1:X, 2:Y, 3:Z}
    for 0-based qubit q (src/clifford/paulistring.jl:71-92)."""
    ops: tuple

    @staticmethod
    def of(n, support, pauli):
        ops = [_I] * n
        for q in support:
            ops[q - 1] = pauli
        return PauliString(tuple(ops))

    @property
    def n(self):
        return len(self.ops)

    def support(self):
        return [q + 1 for q, o in enumerate(self.ops) if o != _I]

    def kind(self):
        first = next((o for o in self.ops if o != _I), _I)
        return first

    def __str__(self):
        return "".join("IXYZ"[o] for o in self.ops)


# ---------------------------------------------------------------------------
# code families
# ---------------------------------------------------------------------------


@dataclass(frozen=True)
class SurfaceCode:
    """Rotated surface code with m rows and n columns (codes.jl:9-12)."""
    m: int
    n: int


@dataclass(frozen=True)
class BivariateBicycleCode:
    m: int
    n: int
    vc: tuple
    hd: tuple


def ToricCode(m: int, n: int) -> BivariateBicycleCode:
    """codes.jl:244."""
    return BivariateBicycleCode(m, n, ((1, 0), (0, 0)), ((0, 1), (0, 0)))


@dataclass(frozen=True)
class Color488:
    d: int


@dataclass(frozen=True)
class Color666:
    d: int


@dataclass(frozen=True)
class SteaneCode:
    pass


@dataclass(frozen=True)
class ShorCode:
    pass


@dataclass(frozen=True)
class Code832:
    pass


@dataclass(frozen=True)
class Code422:
    pass


@dataclass(frozen=True)
class Code1573:
    pass


def _surface(code: SurfaceCode):
    """codes.jl:37-66: qubit (i, j) (1-based) is (i-1)*n + j."""
    m, n = code.m, code.n
    nq = m * n

    def q(i, j):
        return (i - 1) * n + j

    xs, zs = [], []
    for i in range(1, m):
        for j in range(1, n):
            if (i + j) % 2 == 0:
                xs.append((q(i, j), q(i + 1, j), q(i, j + 1), q(i + 1, j + 1)))
    for i in range(1, m // 2 + 1):
        if 2 * i + (n + 1) % 2 <= m:
            xs.append((q(2 * i - 1 + (n + 1) % 2, n), q(2 * i + (n + 1) % 2, n)))
        if 2 * i + 1 <= m:
            xs.append((q(2 * i, 1), q(2 * i + 1, 1)))
    for i in range(1, m):
        for j in range(1, n):
            if (i + j) % 2 == 1:
                zs.append((q(i, j), q(i + 1, j), q(i, j + 1), q(i + 1, j + 1)))
    for j in range(1, n // 2 + 1):
        zs.append((q(1, 2 * j - 1), q(1, 2 * j)))
        if 2 * j + m % 2 <= n:
            zs.append((q(m, 2 * j - 1 + m % 2), q(m, 2 * j + m % 2)))
    return ([PauliString.of(nq, s, _X) for s in xs] + [PauliString.of(nq, s, _Z) for s in zs])


def _bivariate_bicycle(code: BivariateBicycleCode, rm_linear_dependency=True):
    """codes.jl:190-227 (qubits: vertical edges 1..mn then horizontal,
    both numbered column-major over the m x n torus)."""
    m, n = code.m, code.n
    ns = m * n
    nq = 2 * ns

    def ve(i, j):
        return (j - 1) * m + i

    def he(i, j):
        return ns + (j - 1) * m + i

    def wrap(i, k):
        return (i - 1) % k + 1

    out = []
    for j in range(1, n + 1):
        for i in range(1, m + 1):
            st = [ve(wrap(i + s, m), wrap(j + t, n)) for s, t in code.hd]
            st += [he(wrap(i + s, m), wrap(j + t, n)) for s, t in code.vc]
            out.append(PauliString.of(nq, set(st), _X))
    for j in range(1, n + 1):
        for i in range(1, m + 1):
            st = [ve(wrap(i - s, m), wrap(j - t, n)) for s, t in code.vc]
            st += [he(wrap(i - s, m), wrap(j - t, n)) for s, t in code.hd]
            out.append(PauliString.of(nq, set(st), _Z))
    if rm_linear_dependency:
        out = remove_linear_dependency(out)
    return out


def _color488_check_matrix(d):
    """codes.jl:256-334 (column indices are the reference's 1-based ones)."""
    n = (d * d + 2 * d - 1) // 2
    checks = [set() for _ in range((n - 1) // 2)]
    layers = (d - 1) // 2
    i, w = 1, 0
    for layer in range(1, layers + 1):
        w -= layer - 1
        last_even = layer == layers and layers % 2 == 0
        for j in range(1, layer):
            off = 1 if last_even else 0
            checks[w] |= {i + 2 * layer + 1 + (j - 1) * 2, i + 2 * layer + j * 2,
                          (2 * layer + 1) + i + 2 * layer + 1 + (j - 1) * 2 - off,
                          (2 * layer + 1) + i + 2 * layer + j * 2 - off}
            w += 1
        for j in range(layer):
            checks[w] |= {i + j * 2, i + 1 + j * 2, i + 2 * layer + j * 2, i + 2 * layer + 1 + j * 2}
            w += 1
        if layer % 2 == 1:
            checks[w] |= {i, i + 2 * layer, i + 4 * layer, i + 4 * layer + 1}
        else:
            off = 1 if layer == layers else 0
            checks[w] |= {i + 1 + (layer - 1) * 2, i + 2 * layer + 1 + (layer - 1) * 2,
                          (i + 4 * layer) + layer * 2 - off, (i + 4 * layer) + 1 + layer * 2 - off}
        w += 1
        for j in range(layer):
            off = 1 if last_even else 0
            checks[w] |= {i + 2 * layer + j * 2, i + 2 * layer + 1 + j * 2,
                          (2 * layer + 1) + i + 2 * layer + j * 2 - off,
                          (2 * layer + 1) + i + 2 * layer + 1 + j * 2 - off}
            w += 1
        i += 4 * layer
    return checks, n


def _color666_check_matrix(d):
    """codes.jl:336-408."""
    n = (3 * d * d + 1) // 4
    checks = [set() for _ in range((n - 1) // 2)]
    layers = (d - 1) // 2
    i, w = 1, 0
    for layer in range(1, layers + 1):
        w -= layer - 1
        for j in range(1, layer):
            p0 = i + 2 * (j - 1)
            checks[w] |= {p0 + 2 * (layer - 1) + 1, p0 + 2 * (layer - 1) + 2}
            w += 1
        checks[w] |= {i, i + (layer - 1) * 2 + 1, i + 2 + 4 * (layer - 1), i + 2 + 4 * (layer - 1) + 1}
        w += 1
        checks[w] |= {i + 1 + 4 * (layer - 1), i + 1 + 4 * (layer - 1) + layer * 2,
                      i + 5 + 8 * (layer - 1), i + 5 + 8 * (layer - 1) + 1}
        w += 1
        for j in range(1, layer):
            b = i + (j - 1) * 2 + 2 + 2 * (layer - 1)
            checks[w] |= {i + (j - 1) * 2 + 1, i + (j - 1) * 2 + 2, b, b + 1, b + layer * 2, b + layer * 2 + 1}
            w += 1
        for j in range(1, layer):
            p0 = i + (j - 1) * 2 + (layer - 1) * 2 + 1
            checks[w] |= {p0, p0 + 1, p0 + 2 * layer, p0 + 2 * layer + 1, p0 + 4 * layer, p0 + 4 * layer + 1}
            w += 1
        for j in range(layer):
            p0 = i + 2 * j + 2 + 4 * (layer - 1)
            checks[w] |= {p0, p0 + 1, p0 + 2 * layer, p0 + 2 * layer + 1}
            w += 1
        i += 4 + 6 * (layer - 1)
    return checks, n


def _small_code(code):
    """codes.jl:75-163."""
    if isinstance(code, SteaneCode):
        n, sup = 7, [(1, 3, 5, 7), (2, 3, 6, 7), (4, 5, 6, 7)]
        return [PauliString.of(n, s, _X) for s in sup] + [PauliString.of(n, s, _Z) for s in sup]
    if isinstance(code, ShorCode):
        n = 9
        return ([PauliString.of(n, s, _X) for s in [(1, 2, 3, 4, 5, 6), (1, 2, 3, 7, 8, 9)]]
                + [PauliString.of(n, s, _Z) for s in [(1, 2), (1, 3), (4, 5), (4, 6), (7, 8), (7, 9)]])
    if isinstance(code, Code832):
        n = 8
        return ([PauliString.of(n, range(1, 9), _X), PauliString.of(n, range(1, 9), _Z)]
                + [PauliString.of(n, s, _Z) for s in [(1, 3, 5, 7), (1, 2, 3, 4), (1, 2, 5, 6)]])
    if isinstance(code, Code422):
        return [PauliString.of(4, range(1, 5), _X), PauliString.of(4, range(1, 5), _Z)]
    if isinstance(code, Code1573):
        n = 15
        sup = [range(8, 16), list(range(4, 8)) + list(range(12, 16)), (2, 3, 6, 7, 10, 11, 14, 15),
               range(1, 16, 2)]
        return [PauliString.of(n, s, _X) for s in sup] + [PauliString.of(n, s, _Z) for s in sup]
    raise TypeError(f"unknown code {code!r}")


def stabilizers(code) -> list:
    """stabilizers(code), codes.jl:37-421."""
    if isinstance(code, SurfaceCode):
        return _surface(code)
    if isinstance(code, BivariateBicycleCode):
        return _bivariate_bicycle(code)
    if isinstance(code, (Color488, Color666)):
        checks, n = (_color488_check_matrix if isinstance(code, Color488) else _color666_check_matrix)(code.d)
        return ([PauliString.of(n, sorted(c), _X) for c in checks]
                + [PauliString.of(n, sorted(c), _Z) for c in checks])
    return _small_code(code)


def remove_linear_dependency(sts: list) -> list:
    """code_distance.jl:300-304 for CSS stabiliser lists."""
    n = sts[0].n
    xs = [s for s in sts if all(o in (_I, _X) for o in s.ops)]
    zs = [s for s in sts if all(o in (_I, _Z) for o in s.ops)]
    if len(xs) + len(zs) != len(sts):
        raise ValueError("remove_linear_dependency expects CSS stabilisers")

    def row(s):
        v = 0
        for q in s.support():
            v |= 1 << (q - 1)
        return v

    keep = gf2.remove_linear_dependency_rows([row(s) for s in xs], [row(s) for s in zs], n)
    # the bimatrix lists X rows then Z rows; the reference indexes the
    # original list with that row mask
    return [sts[i] for i in keep]


# ---------------------------------------------------------------------------
# Tanner graphs (ldpc.jl)
# ---------------------------------------------------------------------------


@dataclass
class SimpleTannerGraph:
    """ldpc.jl:27-58: nq bits, s2q[i] = 1-based bits of check i."""
    nq: int
    s2q: list
    H: np.ndarray = field(init=False, repr=False)
    q2s: list = field(init=False, repr=False)

    def __post_init__(self):
        self.s2q = [list(c) for c in self.s2q]
        self.H = np.zeros((len(self.s2q), self.nq), dtype=np.uint8)
        for i, c in enumerate(self.s2q):
            for q in c:
                self.H[i, q - 1] = 1
        self.q2s = [[i + 1 for i, c in enumerate(self.s2q) if q in c] for q in range(1, self.nq + 1)]

    @property
    def ns(self):
        return len(self.s2q)


@dataclass
class CSSTannerGraph:
    """ldpc.jl:72-115."""
    stgx: SimpleTannerGraph
    stgz: SimpleTannerGraph

    @property
    def nq(self):
        return self.stgx.nq

    @property
    def ns(self):
        return self.stgx.ns + self.stgz.ns

    @staticmethod
    def from_code(code) -> "CSSTannerGraph":
        return CSSTannerGraph.from_stabilizers(stabilizers(code))

    @staticmethod
    def from_stabilizers(sts) -> "CSSTannerGraph":
        nq = sts[0].n
        xs = [s.support() for s in sts if s.kind() == _X]
        zs = [s.support() for s in sts if s.kind() == _Z]
        return CSSTannerGraph(SimpleTannerGraph(nq, xs), SimpleTannerGraph(nq, zs))


def tanner_graph(code) -> CSSTannerGraph:
    """CSSTannerGraph(code) (ldpc.jl:113-115)."""
    return CSSTannerGraph.from_code(code)
