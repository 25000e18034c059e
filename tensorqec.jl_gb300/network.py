"""Factor graphs of the TNMMAP decoder (TensorQEC's src/decoding/tndecoder.jl).

A ``FactorGraph`` holds the reference's ``ixs`` (labels per tensor),
``tensors`` (float64, flattened in Julia column-major order: the entry with
index bits (x_0, ..., x_{r-1}) sits at offset sum_j x_j 2^j), the output
labels ``iy`` and the positions of the one-hot syndrome leaves.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def parity_tensor(rank: int) -> np.ndarray:
    """parity_check_matrix(rank - 1) (tndecoder.jl:42-44) flattened:
    1 where the sum of the indices is even."""
    idx = np.arange(1 << rank, dtype=np.int64)
    pc = np.zeros_like(idx)
    for b in range(rank):
        pc += (idx >> b) & 1
    return (1 - (pc & 1)).astype(np.float64)


def parity_check_matrix(q: int) -> np.ndarray:
    """The reference's ``parity_check_matrix(q)`` as a (2,)*(q+1) array
    indexed [x_1, ..., x_{q+1}] (tndecoder.jl:42-44)."""
    return parity_tensor(q + 1).reshape((2,) * (q + 1), order="F")


@dataclass
class FactorGraph:
    ixs: list
    tensors: list
    iy: list
    syndrome_positions: list
    # most-probable-configuration graphs: ``iy`` lists the reported labels
    # and the contraction reduces everything to a scalar
    map_mode: bool = False

    @property
    def n_tensors(self):
        return len(self.ixs)

    def flat(self):
        """The arrays of the native ``tqec_network`` struct."""
        ix_off = np.zeros(len(self.ixs) + 1, dtype=np.int32)
        ix_off[1:] = np.cumsum([len(ix) for ix in self.ixs])
        labels = np.array([v for ix in self.ixs for v in ix], dtype=np.int32)
        d_off = np.zeros(len(self.tensors) + 1, dtype=np.int64)
        d_off[1:] = np.cumsum([t.size for t in self.tensors])
        data = np.concatenate([np.asarray(t, dtype=np.float64).ravel() for t in self.tensors])
        return (ix_off, labels, d_off, data, np.asarray(self.iy, dtype=np.int32),
                np.asarray(self.syndrome_positions, dtype=np.int32))


def tnmmap_css_graph(tanner, em, lx, lz) -> FactorGraph:
    """compile(::TNMMAP, ::IndependentDepolarizingDecodingProblem),
    tndecoder.jl:97-139.  Labels: xerr 1..nq, zerr nq+1..2nq, X-check
    syndromes, Z-check syndromes, logical-x outputs, logical-z outputs."""
    nq = tanner.nq
    ns = tanner.ns
    nsx = tanner.stgx.ns
    k = lx.shape[0]
    ixs, tensors = [], []
    for i, c in enumerate(tanner.stgx.s2q, 1):
        ixs.append([q + nq for q in c] + [i + 2 * nq])
        tensors.append(parity_tensor(len(c) + 1))
    for i, c in enumerate(tanner.stgz.s2q, 1):
        ixs.append(list(c) + [i + 2 * nq + nsx])
        tensors.append(parity_tensor(len(c) + 1))
    for i in range(nq):
        px, py, pz = float(em.px[i]), float(em.py[i]), float(em.pz[i])
        ixs.append([i + 1, i + 1 + nq])
        # [1-px-py-pz pz; px py] in column-major order
        tensors.append(np.array([1 - px - py - pz, px, pz, py], dtype=np.float64))
    for i in range(lz.shape[0]):
        sup = [int(q) + 1 for q in np.flatnonzero(lz[i])]
        ixs.append(sup + [i + 1 + 2 * nq + ns + lz.shape[0]])
        tensors.append(parity_tensor(len(sup) + 1))
    for i in range(k):
        sup = [int(q) + 1 + nq for q in np.flatnonzero(lx[i])]
        ixs.append(sup + [i + 1 + 2 * nq + ns])
        tensors.append(parity_tensor(len(sup) + 1))
    synd = []
    for v in range(2 * nq + 1, 2 * nq + ns + 1):
        synd.append(len(ixs))
        ixs.append([v])
        tensors.append(np.array([1.0, 0.0]))
    iy = list(range(2 * nq + ns + 1, 2 * nq + ns + 2 * k + 1))
    return FactorGraph(ixs, tensors, iy, synd)


def push_check_node(ixs, tensors, c, node, nvars, factorize):
    """tndecoder.jl:221-238: a parity check over bits c and label `node`,
    optionally as a chain of rank-3 parity tensors over new labels.  A check
    over fewer than three bits is one parity tensor either way (the
    reference's chain reads c[2] and fails on a check over a single bit)."""
    L = len(c)
    if not factorize or L <= 2:
        ixs.append(list(c) + [node])
        tensors.append(parity_tensor(L + 1))
        return nvars
    ixs.append([c[0], c[1], nvars + 1])
    tensors.append(parity_tensor(3))
    for j in range(3, L):
        ixs.append([nvars + j - 1, c[j - 1], nvars + j - 2])
        tensors.append(parity_tensor(3))
    ixs.append([node, c[L - 1], nvars + L - 2])
    tensors.append(parity_tensor(3))
    return nvars + L - 2


def tnmmap_dem_graph(tanner, l2q, error_rates, n_logicals, factorize=True) -> FactorGraph:
    """compile(::TNMMAP, ::DetectorErrorModel), tndecoder.jl:186-212.
    Labels: errors 1..nq, detectors nq+1..nq+ns, logicals, then chain
    auxiliaries."""
    nq, ns = tanner.nq, tanner.ns
    nvars = nq + ns + n_logicals
    iy = list(range(nq + ns + 1, nvars + 1))
    ixs, tensors = [], []
    for i, c in enumerate(tanner.s2q, 1):
        nvars = push_check_node(ixs, tensors, c, i + nq, nvars, factorize)
    for i, c in enumerate(l2q, 1):
        nvars = push_check_node(ixs, tensors, c, i + nq + ns, nvars, factorize)
    for i, p in enumerate(error_rates, 1):
        ixs.append([i])
        tensors.append(np.array([1 - p, p], dtype=np.float64))
    synd = []
    for v in range(nq + 1, nq + ns + 1):
        synd.append(len(ixs))
        ixs.append([v])
        tensors.append(np.array([1.0, 0.0]))
    return FactorGraph(ixs, tensors, iy, synd)


def tnmap_graph(tanner, prior_ixs, prior_tensors) -> FactorGraph:
    """stg2uaimodel (tndecoder.jl:33-40) with the syndrome evidence of
    compile(::TNMAP, ...) (:46-50) as one-hot leaves.  Labels: bits
    1..nq, syndromes nq+1..nq+ns; every bit label is reported (the root is a
    scalar: the probability of the most probable configuration)."""
    nq, ns = tanner.nq, tanner.ns
    ixs, tensors = [], []
    for s, c in enumerate(tanner.s2q, 1):
        ixs.append(list(c) + [s + nq])
        tensors.append(parity_tensor(len(c) + 1))
    for ix, t in zip(prior_ixs, prior_tensors):
        ixs.append(list(ix))
        tensors.append(np.asarray(t, dtype=np.float64).ravel(order="F"))
    synd = []
    for v in range(nq + 1, nq + ns + 1):
        synd.append(len(ixs))
        ixs.append([v])
        tensors.append(np.array([1.0, 0.0]))
    return FactorGraph(ixs, tensors, list(range(1, nq + 1)), synd, map_mode=True)


def reduce2general(tanner, em):
    """reduce2general(tanner::CSSTannerGraph, pvec) (general_decoding.jl:
    24-32): a SimpleTannerGraph over 2nq bits (x errors 1..nq, z errors
    nq+1..2nq) whose checks are the X checks on the z-error bits followed by
    the Z checks on the x-error bits, and one prior [1-p pz; px py] over
    (x_i, z_i) per qubit.  ``em`` may instead be a tensor network given as
    (ixs, tensors) over those 2nq labels (general_decoding.jl:29-32)."""
    from .codes import SimpleTannerGraph
    nq = tanner.nq
    general = SimpleTannerGraph(2 * nq, [[q + nq for q in c] for c in tanner.stgx.s2q] +
                                [list(c) for c in tanner.stgz.s2q])
    if isinstance(em, tuple):
        ixs, ts = em
        return general, [list(ix) for ix in ixs], [np.asarray(t, dtype=np.float64) for t in ts]
    ixs = [[i + 1, i + 1 + nq] for i in range(nq)]
    ts = []
    for i in range(nq):
        px, py, pz = float(em.px[i]), float(em.py[i]), float(em.pz[i])
        ts.append(np.array([1 - px - py - pz, px, pz, py], dtype=np.float64))
    return general, ixs, ts


# ---------------------------------------------------------------------------
# sliced contraction: fixing a few inner labels splits one wide contraction
# into 2^k narrower ones whose marginals add up to the original
# ---------------------------------------------------------------------------


def slice_graph(graph: FactorGraph, labels, value: int) -> FactorGraph:
    """The network with label ``labels[j]`` fixed to bit j of ``value``:
    every tensor carrying a fixed label keeps only the entries with that
    index (the label disappears; a tensor that loses every label becomes a
    scalar).  Summing the marginals of all 2^k slices gives the marginal of
    ``graph``.  Output labels and the labels of syndrome leaves cannot be
    fixed."""
    fixed = {int(l): (value >> j) & 1 for j, l in enumerate(labels)}
    synd_labels = {v for p in graph.syndrome_positions for v in graph.ixs[p]}
    bad = set(fixed) & (set(graph.iy) | synd_labels)
    if bad:
        raise ValueError(f"labels {sorted(bad)} are outputs or syndrome labels")
    ixs, tensors = [], []
    for ix, t in zip(graph.ixs, graph.tensors):
        t = np.asarray(t, dtype=np.float64)
        if not any(v in fixed for v in ix):
            ixs.append(list(ix))
            tensors.append(t)
            continue
        arr = t.reshape((2,) * len(ix), order="F") if ix else t.reshape(())
        index = tuple(fixed[v] if v in fixed else slice(None) for v in ix)
        ixs.append([v for v in ix if v not in fixed])
        tensors.append(np.ascontiguousarray(arr[index]).ravel(order="F"))
    return FactorGraph(ixs, tensors, list(graph.iy), list(graph.syndrome_positions), graph.map_mode)


def step_label_sets(graph: FactorGraph, steps):
    """Per tree step: (labels of the step's product, labels of its result).
    The result keeps a label while a tensor outside the subtree or the
    output still carries it."""
    total = {}
    for ix in graph.ixs:
        for v in ix:
            total[v] = total.get(v, 0) + 1
    for v in graph.iy:
        total[v] = total.get(v, 0) + 1
    n = graph.n_tensors
    count = [dict() for _ in range(n + len(steps))]
    keep = [set(ix) for ix in graph.ixs] + [set() for _ in steps]
    for i, ix in enumerate(graph.ixs):
        for v in ix:
            count[i][v] = count[i].get(v, 0) + 1
    out = []
    for s, (a, b) in enumerate(np.asarray(steps, dtype=np.int64).reshape(-1, 2)):
        c = dict(count[a])
        for v, k in count[b].items():
            c[v] = c.get(v, 0) + k
        union = keep[a] | keep[b]
        res = {v for v in union if c[v] < total[v]}
        count[n + s] = c
        keep[n + s] = res
        out.append((union, res))
    return out


def choose_slice_labels(graph: FactorGraph, steps, k: int):
    """k labels to fix, chosen greedily: each time the label carried by the
    most of the widest intermediate results (the working set of a syndrome),
    ties broken by the widest step products it occurs in (the multiply-adds);
    output and syndrome labels are never fixed."""
    synd_labels = {v for p in graph.syndrome_positions for v in graph.ixs[p]}
    banned = set(graph.iy) | synd_labels
    chosen = []
    for _ in range(k):
        g = slice_graph(graph, chosen, 0) if chosen else graph
        sets = step_label_sets(g, steps)
        widest_res = max(len(r) for _, r in sets)
        widest_u = max(len(u) for u, _ in sets)
        score = {}
        for u, r in sets:
            for v in (r if len(r) >= widest_res - 1 else ()):
                if v not in banned and v not in chosen:
                    s = score.get(v, (0, 0))
                    score[v] = (s[0] + (2 if len(r) == widest_res else 1), s[1])
            for v in (u if len(u) >= widest_u - 1 else ()):
                if v not in banned and v not in chosen:
                    s = score.get(v, (0, 0))
                    score[v] = (s[0], s[1] + (2 if len(u) == widest_u else 1))
        if not score:
            break
        chosen.append(max(sorted(score), key=lambda v: score[v]))
    return chosen
