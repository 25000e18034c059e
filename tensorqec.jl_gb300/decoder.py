"""The decoder API: TNMMAP / compile / decode, as in TensorQEC
(src/decoding/interfaces.jl:58-105, src/decoding/tndecoder.jl:59-271).

``compile`` builds the reference's factor graph on the host, finds a
contraction order (the role of OMEinsum's ``optimize_code``) and hands both to
the native library, which plans and owns the GPU program.  ``decode`` then
contracts on the GPU; batched calls (``decode_batch``, ``class_logprobs``)
push thousands of syndromes through one launch.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import gf2, native
from .codes import CSSTannerGraph, SimpleTannerGraph
from .dem import DetectorErrorModel, dem2tanner, logical_map
from .error_model import (CSSErrorPattern, CSSSyndrome, DecodingResult, IndependentDepolarizingError,
                          IndependentFlipError, SimpleSyndrome, iid_error, pack_syndromes, random_error_pattern,
                          syndrome_extraction)
from .network import (FactorGraph, choose_slice_labels, reduce2general, slice_graph, tnmap_graph, tnmmap_css_graph,
                      tnmmap_dem_graph)


def simple_rows(syndromes) -> np.ndarray:
    """0/1 syndrome rows from a SimpleSyndrome (one, or a batch with a 2-D
    ``s``), a list of them, or rows already."""
    if isinstance(syndromes, SimpleSyndrome):
        syndromes = syndromes.s
    elif isinstance(syndromes, (list, tuple)) and syndromes and isinstance(syndromes[0], SimpleSyndrome):
        syndromes = np.stack([np.asarray(x.s) for x in syndromes])
    return np.atleast_2d(np.asarray(syndromes, dtype=np.uint8)) & 1


# ---------------------------------------------------------------------------
# contraction-order optimisers (stand-ins for OMEinsum's CodeOptimizer)
# ---------------------------------------------------------------------------


@dataclass
class TreeSA:
    """Randomised greedy passes refined by simulated annealing over tree
    rotations (our own search; OMEinsum's TreeSA plays this role in the
    reference, tndecoder.jl:78)."""
    trials: int = 16
    sweeps: int = 1000
    target_width: int = 0
    width_penalty: float = 1.0
    seed: int = 1
    restarts: int = 4
    # > 1: GEMM-shaped steps (the planner's tensor-core criterion) cost this
    # many times fewer multiply-adds in the search
    tensor_discount: float = 0.0


@dataclass
class GreedyMethod:
    trials: int = 1
    seed: int = 1


@dataclass
class NoOptimizer:
    """tndecoder.jl:64: contract the tensors left to right."""


@dataclass
class FixedOrder:
    """A contraction tree found earlier (OMEinsum accepts an already
    optimised code the same way): an (n_tensors - 1, 2) array of node ids in
    the tqec_tree convention, e.g. read by ``load_order``."""
    steps: np.ndarray


def save_order(path, steps, comment=""):
    """Writes a contraction tree as text: '#' comment lines, then one
    'a b' pair of node ids per binary step."""
    steps = np.asarray(steps, dtype=np.int64).reshape(-1, 2)
    with open(path, "w") as f:
        for line in comment.splitlines():
            f.write(f"# {line}\n")
        for a, b in steps:
            f.write(f"{a} {b}\n")


def load_order(path) -> np.ndarray:
    """Reads a tree written by ``save_order``."""
    rows = [ln.split() for ln in open(path) if ln.strip() and not ln.startswith("#")]
    return np.array([[int(a), int(b)] for a, b in rows], dtype=np.int32).reshape(-1, 2)


def optimize_code(graph: FactorGraph, optimizer) -> np.ndarray:
    """Returns the tree as an (n_tensors - 1, 2) array of node ids."""
    if graph.map_mode:
        # the root of a most-probable-configuration contraction is a scalar
        return optimize_code(FactorGraph(graph.ixs, graph.tensors, [], graph.syndrome_positions), optimizer)
    n = graph.n_tensors
    if isinstance(optimizer, FixedOrder):
        steps = np.ascontiguousarray(optimizer.steps, dtype=np.int32).reshape(-1, 2)
        if steps.shape[0] != max(n - 1, 0):
            raise ValueError(f"the fixed order has {steps.shape[0]} steps; the network needs {max(n - 1, 0)}")
        return steps
    if isinstance(optimizer, NoOptimizer) or n == 1:
        steps = np.zeros((max(n - 1, 0), 2), dtype=np.int32)
        acc = 0
        for i in range(1, n):
            steps[i - 1] = (acc, i)
            acc = n + i - 1
        return steps
    if isinstance(optimizer, GreedyMethod):
        steps, _, _ = native.optimize_order(graph, trials=optimizer.trials, sweeps=0, seed=optimizer.seed)
        return steps
    if isinstance(optimizer, TreeSA):
        if optimizer.restarts <= 1:
            steps, _, _ = native.optimize_order(graph, trials=optimizer.trials, sweeps=optimizer.sweeps,
                                                target_width=optimizer.target_width,
                                                width_penalty=optimizer.width_penalty, seed=optimizer.seed,
                                                tensor_discount=optimizer.tensor_discount)
            return steps
        return _search_fitting(graph, optimizer)
    raise TypeError(f"unknown optimizer {optimizer!r}")


# per-syndrome working set that still lets a thread block keep it in shared
# memory (float32), with room for the step records
_SMEM_ARENA_BYTES = 200 * 1024


def _estimated_cost(plan):
    """Relative runtime estimate of a compiled program: runtime flops, tripled
    when the float32 working set spills out of shared memory."""
    fits = plan["arena_elems"] * 4 <= _SMEM_ARENA_BYTES
    return plan["flops_per_syndrome"] * (1.0 if fits else 3.0)


def _search_fitting(graph, opt):
    """Several annealing restarts (and narrower width targets) scored by the
    planner's own flops and working-set size; the cheapest tree wins.  A
    given target width is searched at that width only."""
    best = None
    widths = [opt.target_width] if opt.target_width else [0]
    for r in range(opt.restarts):
        for tw in widths:
            steps, _, w = native.optimize_order(graph, trials=opt.trials, sweeps=opt.sweeps, target_width=tw,
                                                width_penalty=max(2.0, opt.width_penalty) if tw else opt.width_penalty,
                                                seed=opt.seed + r, tensor_discount=opt.tensor_discount)
            plan = native.inspect_plan(graph, steps)
            cost = _estimated_cost(plan)
            if best is None or cost < best[0]:
                best = (cost, steps, plan)
        if best[2]["arena_elems"] * 4 > _SMEM_ARENA_BYTES and len(widths) == 1 and not opt.target_width:
            widths.append(best[2]["width"] - 1)
    return best[1]


# ---------------------------------------------------------------------------
# decoders
# ---------------------------------------------------------------------------


@dataclass
class TNMMAP:
    """Marginal-MAP decoder over logical classes (tndecoder.jl:77-80).

    ``precision``: "f64" contracts in float64 (the reference's arithmetic);
    "f32" contracts in float32 with power-of-two renormalisation and
    re-contracts every syndrome whose class margin is below the
    rounding-error bound, in double-float (pairs of float32, about 48
    significant bits; GB300 runs float64 at 1/64 of the float32 rate) or, with
    ``recheck_f64``, in float64.  ``plain`` launches one syndrome at a time
    (the drop-in form of the reference's per-syndrome ``decode``).
    ``slices`` > 0 fixes that many inner labels of the tree and contracts the
    2^slices narrower networks (``SlicedProgram``), for networks too wide to
    contract whole.  ``shared_items``: in blocks of one syndrome, lanes share
    the work items of steps that would leave threads idle."""
    optimizer: object = field(default_factory=TreeSA)
    factorize: bool = True
    precision: str = "f32"
    plain: bool = False
    margin: float = -1.0
    device: int = 0
    group: int = 0
    threads: int = 0
    split_arena: bool = False
    big_elems: int = 0
    tensor_cores: bool = True
    recheck_f64: bool = False
    slices: int = 0
    shared_items: bool = False

    def _native_precision(self):
        return {"f64": native.TQEC_F64, "f32": native.TQEC_F32}[self.precision]

    def _flags(self):
        return ((native.TQEC_FLAG_PLAIN if self.plain else 0) |
                (native.TQEC_FLAG_SPLIT_ARENA if self.split_arena else 0) |
                (0 if self.tensor_cores else native.TQEC_FLAG_NO_TENSOR_CORES) |
                (native.TQEC_FLAG_RECHECK_F64 if self.recheck_f64 else 0) |
                (native.TQEC_FLAG_SHARED_ITEMS if self.shared_items else 0))

    def _program(self, graph, steps):
        """The GPU program of a compiled network: whole, or sliced."""
        args = (self._native_precision(), self._flags(), self.device, self.group, self.threads, self.margin,
                self.big_elems)
        if self.slices > 0:
            return SlicedProgram.build(graph, steps, choose_slice_labels(graph, steps, self.slices), *args)
        return native.Program(graph, steps, *args)


class SlicedProgram:
    """A network contracted in 2^k slices: one program per value of k fixed
    inner labels (network.slice_graph), whose marginals add up to the
    network's (the whole contraction of tndecoder.jl:162).  It answers the
    calls the decoders make on a ``native.Program``.  ``decode_packed``
    follows tqec_decode_batch: the slices contract without their own
    recheck, their marginals are summed (log-sum-exp), and with float32 the
    rows whose log-margin is below twice the largest slice bound (a sum of
    non-negative terms keeps the largest relative error of its terms) are
    contracted again in double-float, or float64 with recheck_f64, before
    the first maximum (Julia's findmax order) is taken."""

    def __init__(self, parts, labels, precision, recheck_precision, recheck=True, margin=-1.0):
        self.parts = list(parts)
        self.labels = list(labels)
        self.precision = precision
        self.recheck_precision = recheck_precision
        self.recheck = recheck
        self.margin = margin
        self.last_recheck = 0
        info = dict(self.parts[0].info)
        for key in ("err_bound_f32", "err_bound_f64", "err_bound_f32x2", "arena_elems", "width"):
            if key in info:
                info[key] = max(p.info[key] for p in self.parts)
        info["flops_per_syndrome"] = sum(p.info["flops_per_syndrome"] for p in self.parts)
        info["slices"] = len(self.parts)
        self.info = info

    @classmethod
    def build(cls, graph, steps, labels, precision, flags, device=0, group=0, threads=0, margin=-1.0, big_elems=0):
        parts = []
        try:
            for v in range(1 << len(labels)):
                parts.append(native.Program(slice_graph(graph, labels, v), steps, precision,
                                            flags | native.TQEC_FLAG_NORECHECK, device, group, threads, margin,
                                            big_elems))
        except Exception:
            for p in parts:
                p.close()
            raise
        recheck = precision == native.TQEC_F32 and not flags & native.TQEC_FLAG_NORECHECK
        rp = native.TQEC_F64 if flags & native.TQEC_FLAG_RECHECK_F64 else native.TQEC_F32X2
        return cls(parts, labels, precision, rp, recheck, margin)

    @property
    def n_classes(self):
        return self.parts[0].n_classes

    @property
    def syndrome_bytes(self):
        return self.parts[0].syndrome_bytes

    def contract_packed(self, packed, precision, logp=None):
        lps = []
        for p in self.parts:
            lps.append(p.contract_packed(packed, precision))
            # wide slices (more than 2^22 intermediate elements a syndrome)
            # free their arenas before the next slice allocates its own
            if p.info["arena_elems"] > (1 << 22):
                p.trim()
        lps = np.stack(lps)
        top = lps.max(axis=0)
        safe = np.where(np.isfinite(top), top, 0.0)
        with np.errstate(divide="ignore"):
            out = safe + np.log(np.exp(lps - safe).sum(axis=0))
        out[~np.isfinite(top)] = -np.inf
        if logp is not None:
            logp[...] = out
            return logp
        return out

    def _bound(self, precision):
        key = {native.TQEC_F32: "err_bound_f32", native.TQEC_F64: "err_bound_f64",
               native.TQEC_F32X2: "err_bound_f32x2"}[precision]
        return self.info[key]

    def decode_packed(self, packed, classes=None, logp=None, err=None, stream=None):
        packed = np.ascontiguousarray(packed, dtype=np.uint8)
        n = packed.shape[0]
        lp = self.contract_packed(packed, self.precision)
        bound = np.full(n, self._bound(self.precision))
        self.last_recheck = 0
        if self.recheck and n and self.n_classes > 1:
            thr = self.margin if self.margin >= 0 else 2.0 * self._bound(self.precision)
            top2 = np.sort(lp, axis=1)[:, -2:]
            with np.errstate(invalid="ignore"):
                low = ~(top2[:, 1] - top2[:, 0] >= thr) | (top2[:, 1] == -np.inf)
            rows = np.flatnonzero(low)
            if rows.size:
                lp[rows] = self.contract_packed(packed[rows], self.recheck_precision)
                bound[rows] = self._bound(self.recheck_precision)
            self.last_recheck = int(rows.size)
        cls = np.argmax(lp, axis=1).astype(np.int32)  # first maximum; a row of -inf gives 0
        if classes is None:
            classes = cls
        else:
            classes[...] = cls
        if logp is not None:
            logp[...] = lp
        if err is not None:
            err[...] = bound
        return classes

    def last_recheck_count(self):
        return self.last_recheck

    def autotune(self, n_probe=4096):
        for p in self.parts:
            p.autotune(n_probe)

    def save(self, path):
        """Each slice is its own program: ``parts[i].save`` keeps slice i."""
        raise TypeError("a sliced program is saved slice by slice: SlicedProgram.parts[i].save(path)")

    def close(self):
        for p in self.parts:
            p.close()


class CompiledTNMMAP:
    """CompiledTNMMAP (tndecoder.jl:85-92) with its GPU program."""

    def __init__(self, decoder: TNMMAP, tanner: CSSTannerGraph, em: IndependentDepolarizingError):
        self.decoder = decoder
        self.tanner = tanner
        self.em = em
        self.lx, self.lz = gf2.logical_operator(tanner)
        self.graph = tnmmap_css_graph(tanner, em, self.lx, self.lz)
        self.steps = optimize_code(self.graph, decoder.optimizer)
        self.program = decoder._program(self.graph, self.steps)
        self._px = gf2.solve_particular(tanner.stgz.H)   # ex from sz
        self._pz = gf2.solve_particular(tanner.stgx.H)   # ez from sx
        self.k = self.lx.shape[0]

    @property
    def n_syndrome(self):
        return self.tanner.ns

    @property
    def n_classes(self):
        return self.program.n_classes

    def _bits(self, syndromes):
        """Syndrome rows from one CSSSyndrome, a batched one (2-D sx, sz), a
        list of them, or 0/1 rows [sx..., sz...]."""
        if isinstance(syndromes, CSSSyndrome):
            return np.atleast_2d(syndromes.bits())
        if isinstance(syndromes, (list, tuple)) and syndromes and isinstance(syndromes[0], CSSSyndrome):
            return np.stack([s.bits() for s in syndromes])
        b = np.asarray(syndromes, dtype=np.uint8)
        return np.atleast_2d(b) & 1

    def decode_batch(self, syndromes, return_logp=False):
        """Argmax classes (Julia linear index of ``mar``) for a batch of
        syndrome rows ([sx..., sz...] bits)."""
        packed = pack_syndromes(self._bits(syndromes))
        n = packed.shape[0]
        logp = np.empty((n, self.n_classes), dtype=np.float64) if return_logp else None
        cls = self.program.decode_packed(packed, logp=logp)
        return (cls, logp) if return_logp else cls

    def class_logprobs(self, syndromes, precision=None):
        """Natural log of the unnormalised marginal ``mar`` for each syndrome
        (Julia linear order), contracted in the given precision."""
        packed = pack_syndromes(self._bits(syndromes))
        prec = self.decoder._native_precision() if precision is None else \
            {"f64": native.TQEC_F64, "f32": native.TQEC_F32, "f32x2": native.TQEC_F32X2,
             "bf16": native.TQEC_F32_BF16}[precision]
        return self.program.contract_packed(packed, prec)

    def error_pattern(self, cls: int, syndrome: CSSSyndrome):
        """error_pattern(pos, ct, syndrome), tndecoder.jl:167-174, with a
        GF(2) particular solution in place of the integer program
        (ipdecoder.jl:150-169).  Returns None for a syndrome no error
        produces."""
        ex = self._px(np.asarray(syndrome.sz))
        ez = self._pz(np.asarray(syndrome.sx))
        if ex is None or ez is None:
            return None
        k = self.k
        for i in range(k):
            a_i = (cls >> i) & 1
            b_i = (cls >> (k + i)) & 1
            if int(self.lz[i].astype(np.int64) @ ex) % 2 != b_i:
                ex = ex ^ self.lx[i]
            if int(self.lx[i].astype(np.int64) @ ez) % 2 != a_i:
                ez = ez ^ self.lz[i]
        return CSSErrorPattern(ex, ez)

    def _pattern_decoder(self):
        if getattr(self, "_patterns", None) is None:
            self._patterns = native.PatternDecoder(self.tanner, self.lx, self.lz, self.decoder.device)
        return self._patterns

    def decode_patterns(self, syndromes, classes=None):
        """Batched ``decode``: classes (argmax of the marginal, unless given)
        and the rebuilt (ex, ez) error patterns of every row, all on the GPU.
        Returns (classes, ex, ez, ok) with ex/ez as (n, nq) 0/1 arrays and
        ok = 0 for syndromes no error produces."""
        bits = self._bits(syndromes)
        packed = pack_syndromes(bits)
        if classes is None:
            classes = self.program.decode_packed(packed)
        ex, ez, ok = self._pattern_decoder().decode(packed, np.asarray(classes, dtype=np.int32))
        return classes, ex, ez, ok

    def decode(self, syndrome: CSSSyndrome) -> DecodingResult:
        """decode(ct, syndrome), tndecoder.jl:160-165."""
        cls = int(self.decode_batch(syndrome)[0])
        ep = self.error_pattern(cls, syndrome)
        return DecodingResult(ep is not None, ep)

    def close(self):
        self.program.close()


class CompiledDEMTNMMAP:
    """CompiledDEMTNMMAP (tndecoder.jl:176-182) with its GPU program."""

    def __init__(self, decoder: TNMMAP, dem: DetectorErrorModel):
        self.decoder = decoder
        self.dem = dem
        self.tanner = dem2tanner(dem)
        self.l2q = logical_map(dem)
        self.graph = tnmmap_dem_graph(self.tanner, self.l2q, dem.error_rates, len(dem.logical_list),
                                      decoder.factorize)
        self.steps = optimize_code(self.graph, decoder.optimizer)
        self.program = decoder._program(self.graph, self.steps)
        self._part = gf2.solve_particular(self.tanner.H)
        self._logical_fix = self._logical_corrections()

    def _logical_corrections(self):
        """For each logical i, a set of mechanisms that flips no detector and
        only logical i (None if the model has none)."""
        nq = self.tanner.nq
        L = np.zeros((len(self.l2q), nq), dtype=np.uint8)
        for i, l in enumerate(self.l2q):
            L[i, np.array(l, dtype=np.int64) - 1] = 1
        A = np.vstack([self.tanner.H, L]) if L.size else self.tanner.H
        solve = gf2.solve_particular(A)
        out = []
        for i in range(L.shape[0]):
            rhs = np.zeros(A.shape[0], dtype=np.uint8)
            rhs[self.tanner.ns + i] = 1
            out.append(solve(rhs))
        return out

    @property
    def n_syndrome(self):
        return self.tanner.ns

    @property
    def n_classes(self):
        return self.program.n_classes

    def decode_batch(self, syndromes, return_logp=False):
        bits = simple_rows(syndromes)
        packed = pack_syndromes(bits)
        n = packed.shape[0]
        logp = np.empty((n, self.n_classes), dtype=np.float64) if return_logp else None
        cls = self.program.decode_packed(packed, logp=logp)
        return (cls, logp) if return_logp else cls

    def class_logprobs(self, syndromes, precision=None):
        packed = pack_syndromes(simple_rows(syndromes))
        prec = self.decoder._native_precision() if precision is None else \
            {"f64": native.TQEC_F64, "f32": native.TQEC_F32, "f32x2": native.TQEC_F32X2,
             "bf16": native.TQEC_F32_BF16}[precision]
        return self.program.contract_packed(packed, prec)

    def error_pattern(self, cls: int, syndrome: SimpleSyndrome):
        """error_pattern(pos, ct, syndrome), tndecoder.jl:255-271: a
        syndrome-consistent error whose logical flips equal the decoded
        class.  Where the reference flips every mechanism of a logical, this
        applies a detector-neutral correction of that logical instead, so the
        pattern keeps reproducing the syndrome."""
        ep = self._part(np.asarray(syndrome.s))
        if ep is None:
            return None
        for i, l in enumerate(self.l2q):
            idx = np.array(l, dtype=np.int64) - 1
            par = int(ep[idx].sum()) % 2
            want = (cls >> i) & 1
            if par != want:
                fix = self._logical_fix[i]
                if fix is None:
                    ep[idx] ^= 1
                else:
                    ep = ep ^ fix
        return ep

    def decode(self, syndrome: SimpleSyndrome) -> DecodingResult:
        cls = int(self.decode_batch(np.asarray(syndrome.s)[None, :])[0])
        ep = self.error_pattern(cls, syndrome)
        return DecodingResult(ep is not None, ep)

    def close(self):
        self.program.close()


@dataclass
class TNMAP:
    """Most-probable-configuration decoder (tndecoder.jl:9-11): max-product
    contraction of the general decoding problem's factor graph on the GPU,
    then back-tracking of the maximising values from the root down.

    ``precision``: "f64" (default) or "f32" (power-of-two renormalised; the
    maximiser can differ from f64 only between configurations whose
    probabilities agree to float32 rounding)."""
    optimizer: object = field(default_factory=TreeSA)
    precision: str = "f64"
    device: int = 0
    group: int = 0
    threads: int = 0

    def _native_precision(self):
        return {"f64": native.TQEC_F64, "f32": native.TQEC_F32}[self.precision]


class CompiledTNMAP:
    """CompiledTNMAP (tndecoder.jl:16-19, compile at :46-50) for a
    GeneralDecodingProblem: a SimpleTannerGraph plus one prior tensor per
    ``prior_ixs`` entry (labels are 1-based bits)."""

    def __init__(self, decoder: TNMAP, tanner: SimpleTannerGraph, prior_ixs, prior_tensors):
        self.decoder = decoder
        self.tanner = tanner
        self.prior_ixs = [list(ix) for ix in prior_ixs]
        self.prior_tensors = [np.asarray(t, dtype=np.float64) for t in prior_tensors]
        self.graph = tnmap_graph(tanner, self.prior_ixs, self.prior_tensors)
        self.steps = optimize_code(self.graph, decoder.optimizer)
        self.program = native.Program(self.graph, self.steps, decoder._native_precision(), native.TQEC_FLAG_MAP,
                                      decoder.device, decoder.group, decoder.threads, -1.0)

    @property
    def n_syndrome(self):
        return self.tanner.ns

    @property
    def qubit_num(self):
        return self.tanner.nq

    def decode_batch(self, syndromes, return_logp=False):
        """Most probable bit configuration for each syndrome row: an
        (n, nq) 0/1 array (and the natural log of its probability)."""
        bits = simple_rows(syndromes)
        cfg, logp = self.program.map_decode_packed(pack_syndromes(bits), self.tanner.nq)
        return (cfg, logp) if return_logp else cfg

    def log_probability(self, config):
        """Natural log of the unnormalised probability of full bit
        configurations (rows of 0/1), from the prior tensors (host)."""
        config = np.atleast_2d(np.asarray(config, dtype=np.int64))
        out = np.zeros(config.shape[0])
        with np.errstate(divide="ignore"):
            for ix, t in zip(self.prior_ixs, self.prior_tensors):
                flat = t.ravel(order="F")
                idx = np.zeros(config.shape[0], dtype=np.int64)
                for j, v in enumerate(ix):
                    idx |= config[:, v - 1] << j
                out += np.log(flat[idx])
        return out

    def decode(self, syndrome: SimpleSyndrome) -> DecodingResult:
        """decode(ct::CompiledTNMAP, syndrome), tndecoder.jl:53-57."""
        cfg = self.decode_batch(np.asarray(syndrome.s)[None, :])[0]
        return DecodingResult(True, cfg.astype(np.uint8))

    def close(self):
        self.program.close()


class CompiledGeneralTNMAP:
    """CompiledGeneralDecoder (interfaces.jl:124-137): TNMAP on the CSS
    problem reduced by reduce2general; decode returns a CSSErrorPattern."""

    def __init__(self, decoder: TNMAP, tanner: CSSTannerGraph, em):
        self.css = tanner
        self.em = em
        general, ixs, ts = reduce2general(tanner, em)
        self.cd = CompiledTNMAP(decoder, general, ixs, ts)

    @property
    def program(self):
        return self.cd.program

    def decode_batch(self, syndromes, return_logp=False):
        """(ex, ez) rows for syndrome rows [sx..., sz...]."""
        if isinstance(syndromes, CSSSyndrome):
            syndromes = np.atleast_2d(syndromes.bits())
        cfg, logp = self.cd.decode_batch(syndromes, return_logp=True)
        nq = self.css.nq
        out = (cfg[:, :nq], cfg[:, nq:])
        return (out, logp) if return_logp else out

    def decode(self, syndrome: CSSSyndrome) -> DecodingResult:
        """extract_decoding (general_decoding.jl:9-12) of the general decode."""
        cfg = self.cd.decode_batch(syndrome.bits()[None, :])[0].astype(np.uint8)
        nq = self.css.nq
        return DecodingResult(True, CSSErrorPattern(cfg[:nq], cfg[nq:]))

    def close(self):
        self.cd.close()


def compile(decoder, problem, em=None):
    """compile(decoder, tanner[, em]) / compile(decoder, dem)
    (interfaces.jl:74-79, tndecoder.jl:97, :186).  Without ``em`` a CSS code
    gets the reference's default ``iid_error(0.05, tanner)``.  TNMAP takes a
    CSS code (reduced by reduce2general, interfaces.jl:129-133), a
    SimpleTannerGraph with an IndependentFlipError (:139-142) or a
    GeneralDecodingProblem given as (tanner, prior_ixs, prior_tensors)."""
    if isinstance(decoder, TNMAP):
        if isinstance(problem, CSSTannerGraph):
            if em is None:
                em = iid_error(0.05, problem)
            return CompiledGeneralTNMAP(decoder, problem, em)
        if isinstance(problem, SimpleTannerGraph):
            if em is None:
                em = iid_error(0.05, problem.nq)
            if isinstance(em, IndependentFlipError):
                p = em.p
            else:
                p = np.broadcast_to(np.asarray(em, dtype=np.float64), (problem.nq,))
            return CompiledTNMAP(decoder, problem, [[i + 1] for i in range(problem.nq)],
                                 [np.array([1 - q, q]) for q in p])
        if isinstance(problem, tuple) and len(problem) == 3:
            return CompiledTNMAP(decoder, *problem)
        raise TypeError(f"TNMAP cannot compile for {type(problem).__name__}")
    if not isinstance(decoder, TNMMAP):
        raise TypeError("compile supports TNMMAP and TNMAP")
    if isinstance(problem, DetectorErrorModel):
        return CompiledDEMTNMMAP(decoder, problem)
    if isinstance(problem, CSSTannerGraph):
        if em is None:
            em = iid_error(0.05, problem)
        return CompiledTNMMAP(decoder, problem, em)
    raise TypeError(f"cannot compile for {type(problem).__name__}")


def decode(ct_or_decoder, *args):
    """decode(ct, syndrome) or decode(decoder, tanner, syndrome[, em])
    (interfaces.jl:96-105)."""
    if isinstance(ct_or_decoder, (CompiledTNMMAP, CompiledDEMTNMMAP, CompiledTNMAP, CompiledGeneralTNMAP)):
        return ct_or_decoder.decode(*args)
    decoder, tanner, syndrome = ct_or_decoder, args[0], args[1]
    em = args[2] if len(args) > 2 else None
    ct = compile(decoder, tanner, em)
    try:
        return ct.decode(syndrome)
    finally:
        ct.close()


def multi_round_qec(tanner, decoder, em, tanner_check=None, rounds=10, rng=None, batch=1 << 16, prior=None):
    """multi_round_qec (threshold.jl:1-33): samples `rounds` errors from
    `em`, decodes their syndromes (in batches) and returns logical error
    rates.  Like the reference, the decoder is compiled with the default
    noise of ``compile(decoder, tanner)`` (interfaces.jl:74-76) unless
    `prior` gives another error model.

    CSS code: returns the rates of (X-type, Z-type, any) logical errors; a
    round counts for a type when the decoded class differs from the sampled
    error's class in that type's bits (lz . ex for X errors, lx . ez for Z
    errors, the CSS check_logical_error of error_model.jl:161-181; the
    reference's loop compares against the stabiliser matrices instead).
    TNMMAP decoders are judged by their classes, TNMAP decoders by the
    difference of their decoded error from the sampled one.
    Classical code (threshold.jl:21-33, a SimpleTannerGraph decoded by
    TNMAP): returns the rate of rounds whose decoded bits differ from the
    sampled ones by a vector with odd overlap with a row of
    ``tanner_check.H``."""
    rng = np.random.default_rng() if rng is None else rng
    ct = compile(decoder, tanner, prior)
    try:
        if isinstance(tanner, SimpleTannerGraph):
            if tanner_check is None:
                raise TypeError("a classical code needs tanner_check, the checks of a logical error")
            Hc = np.asarray(tanner_check.H, dtype=np.int64)
            bad = done = 0
            while done < rounds:
                n = min(batch, rounds - done)
                ex = random_error_pattern(em, rng, nsamples=n)
                syn = syndrome_extraction(ex, tanner)
                cfg = np.asarray(ct.decode_batch(syn), dtype=np.int64)
                bad += int((((ex.astype(np.int64) - cfg) % 2) @ Hc.T % 2).any(axis=1).sum())
                done += n
            return bad / rounds
        lx, lz = (m.astype(np.int64) for m in gf2.logical_operator(tanner))
        k = lx.shape[0]
        w = 1 << np.arange(k)
        nx = nz = nany = done = 0
        while done < rounds:
            n = min(batch, rounds - done)
            ep = random_error_pattern(em, rng, nsamples=n)
            ex = np.asarray(ep.xerror, dtype=np.int64)
            ez = np.asarray(ep.zerror, dtype=np.int64)
            out = ct.decode_batch(syndrome_extraction(ep, tanner))
            if isinstance(out, tuple):  # TNMAP: decoded (ex, ez) rows
                x_err = (((ex ^ np.asarray(out[0], dtype=np.int64)) @ lz.T) % 2).any(axis=1)
                z_err = (((ez ^ np.asarray(out[1], dtype=np.int64)) @ lx.T) % 2).any(axis=1)
            else:  # TNMMAP: decoded classes
                cls = np.asarray(out, dtype=np.int64)
                x_err = (cls >> k) != ((ex @ lz.T) % 2) @ w     # X-type class bits
                z_err = (cls & ((1 << k) - 1)) != ((ez @ lx.T) % 2) @ w   # Z-type class bits
            nx += int(x_err.sum())
            nz += int(z_err.sum())
            nany += int((x_err | z_err).sum())
            done += n
        return nx / rounds, nz / rounds, nany / rounds
    finally:
        ct.close()
