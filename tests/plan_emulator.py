"""A numpy executor of the compiled contraction program (test helper).

It runs the exact step records, permutation tables, constant tables and
arena offsets that the CUDA kernel receives, so a planner bug (wrong layout,
overlapping arena slots, wrong folding) shows up on the CPU.  Unwritten arena
memory is NaN, so reading a slot before it is written poisons the result.
"""
from __future__ import annotations

import numpy as np

OP_ARENA, OP_CONST, OP_PARITY = 0, 1, 2


def _popcount(x):
    x = np.asarray(x, dtype=np.int64)
    c = np.zeros_like(x)
    while np.any(x):
        c += x & 1
        x = x >> 1
    return c


def _perm_addr(perm, off, e, lw):
    addr = np.zeros_like(e)
    tab = off
    sh = 0
    while sh < lw:
        cb = min(8, lw - sh)
        addr |= perm[tab + ((e >> sh) & ((1 << cb) - 1))]
        tab += 1 << cb
        sh += 8
    return addr


def run_plan(plan, bits, dtype=np.float64, return_arena=False):
    """bits: (n, n_syndrome) 0/1.  Returns (n, n_classes) marginals (for a
    MAP-mode plan: the max-product value, shape (n, 1))."""
    maxp = plan.get("map_mode", False)
    bits = np.atleast_2d(np.asarray(bits, dtype=np.int64))
    n = bits.shape[0]
    steps = plan["steps"]
    consts = plan["consts"].astype(dtype)
    perm = plan["perm"].astype(np.int64)
    arena = np.full((n, plan["arena_elems"]), np.nan, dtype=dtype)
    rows = np.arange(n)[:, None, None]
    for d in steps:
        lh, lfa, lfb, lk = int(d["lh"]), int(d["lfa"]), int(d["lfb"]), int(d["lk"])
        lw = lh + lfa + lfb
        e = np.arange(1 << lw, dtype=np.int64)
        fb = e & ((1 << lfb) - 1)
        fa = (e >> lfb) & ((1 << lfa) - 1)
        h = e >> (lfb + lfa)
        k = np.arange(1 << lk, dtype=np.int64)
        aidx = (((h << lfa) | fa) << lk)[:, None] + k[None, :]
        if int(d["flags"]) & 8:  # GEMM-shaped step: B stored [h][fb][k]
            bidx = (((h << lfb) | fb) << lk)[:, None] + k[None, :]
        else:
            bidx = ((h << (lk + lfb)) | fb)[:, None] + (k[None, :] << lfb)

        def operand(kind, ref, sel, idx, obits):
            if kind == OP_PARITY:
                s = bits[:, ref][:, None, None]
                return ((((_popcount(idx)[None] ^ s) & 1) == 0)).astype(dtype)
            if kind == OP_ARENA:
                return arena[rows, ref + idx[None]]
            v = np.zeros(n, dtype=np.int64)
            for i, b in enumerate(sel):
                if b >= 0:
                    v |= bits[:, b] << i
            return consts[(ref + (v << obits))[:, None, None] + idx[None]]

        av = operand(int(d["a_kind"]), int(d["a_ref"]), d["a_sel"], aidx, lh + lfa + lk)
        bv = operand(int(d["b_kind"]), int(d["b_ref"]), d["b_sel"], bidx, lh + lk + lfb)
        acc = (av * bv).max(axis=2) if maxp else (av * bv).sum(axis=2)
        addr = e if int(d["perm_off"]) < 0 else _perm_addr(perm, int(d["perm_off"]), e, lw)
        arena[:, int(d["out_off"]) + addr] = acc
    root = steps[-1]
    out = arena[:, int(root["out_off"]): int(root["out_off"]) + plan["n_classes"]]
    return (out, arena) if return_arena else out


def map_backtrack(plan, bits, arena):
    """Most probable configuration from a MAP-mode plan's arena: walks the
    steps from the root down (as the kernel does) and returns the values of
    the reported variables, (n, n_report)."""
    bits = np.atleast_2d(np.asarray(bits, dtype=np.int64))
    n = bits.shape[0]
    consts = plan["consts"]
    vt = plan["vartab"]
    out = np.zeros((n, len(plan["report"])), dtype=np.uint8)
    for r in range(n):
        asg = np.where(plan["fixed"] == 1, 1, 0).astype(np.int64)
        for d in plan["steps"][::-1]:
            lh, lfa, lfb, lk = int(d["lh"]), int(d["lfa"]), int(d["lfb"]), int(d["lk"])
            o = int(d["var_off"])
            fb = sum(int(asg[vt[o + j]]) << j for j in range(lfb))
            fa = sum(int(asg[vt[o + lfb + j]]) << j for j in range(lfa))
            h = sum(int(asg[vt[o + lfb + lfa + j]]) << j for j in range(lh))
            abase = ((h << lfa) | fa) << lk
            bT = int(d["flags"]) & 8
            bbase = (((h << lfb) | fb) << lk) if bT else ((h << (lk + lfb)) | fb)
            bstep = 1 if bT else (1 << lfb)

            def val(kind, ref, sel, idx, obits):
                if kind == OP_PARITY:
                    return 1.0 if ((bin(idx).count("1") ^ int(bits[r, ref])) & 1) == 0 else 0.0
                if kind == OP_ARENA:
                    return arena[r, ref + idx]
                v = 0
                for i, b in enumerate(sel):
                    if b >= 0:
                        v |= int(bits[r, b]) << i
                return consts[ref + (v << obits) + idx]

            best, bk = -1.0, 0
            for k in range(1 << lk):
                v = (val(int(d["a_kind"]), int(d["a_ref"]), d["a_sel"], abase + k, lh + lfa + lk)
                     * val(int(d["b_kind"]), int(d["b_ref"]), d["b_sel"], bbase + k * bstep, lh + lk + lfb))
                if v > best:
                    best, bk = v, k
            for j in range(lk):
                asg[vt[o + lfb + lfa + lh + j]] = (bk >> j) & 1
        out[r] = asg[plan["report"]]
    return out


U32, U64, UX2 = 2.0 ** -24, 2.0 ** -53, 2.0 ** -43


class EmulatedProgram:
    """The calls the decoders make on ``native.Program``, answered by the
    numpy emulator of the compiled program (float32 or float64)."""

    instances = []

    def __init__(self, graph, steps, precision=1, flags=0, device=0, group=0, threads=0, margin=-1.0,
                 big_elems=0):
        import tensorqec_gb300.native as native

        self.plan = native.inspect_plan(graph, steps, flags & native.TQEC_FLAG_MAP)
        t = self.plan["err_terms"] * 1.01
        self.info = {"err_bound_f32": U32 * t, "err_bound_f64": U64 * t, "err_bound_f32x2": UX2 * t,
                     "flops_per_syndrome": self.plan["flops_per_syndrome"], "arena_elems": self.plan["arena_elems"],
                     "width": self.plan["width"], "n_classes": self.plan["n_classes"],
                     "syndrome_bytes": (self.plan["n_syndrome"] + 7) // 8}
        self.precision, self.flags = precision, flags
        self.calls = []
        EmulatedProgram.instances.append(self)

    @property
    def n_classes(self):
        return self.plan["n_classes"]

    @property
    def syndrome_bytes(self):
        return self.info["syndrome_bytes"]

    def contract_packed(self, packed, precision, logp=None):
        self.calls.append((precision, packed.shape[0]))
        bits = np.unpackbits(np.atleast_2d(packed), axis=1, count=self.plan["n_syndrome"], bitorder="little")
        m = run_plan(self.plan, bits, dtype=np.float32 if precision == 1 else np.float64).astype(np.float64)
        with np.errstate(divide="ignore"):
            out = np.log(m)
        if logp is not None:
            logp[...] = out
            return logp
        return out

    def decode_packed(self, packed, classes=None, logp=None, err=None, stream=None):
        """Argmax of the float64 emulation (the float32 recheck ends in a
        result within the float64 bound)."""
        lp = self.contract_packed(packed, 0)
        cls = np.argmax(lp, axis=1).astype(np.int32)
        if classes is not None:
            classes[...] = cls
        if logp is not None:
            logp[...] = lp
        return cls if classes is None else classes

    def map_decode_packed(self, packed, n_report):
        bits = np.unpackbits(np.atleast_2d(packed), axis=1, count=self.plan["n_syndrome"], bitorder="little")
        val, arena = run_plan(self.plan, bits, return_arena=True)
        with np.errstate(divide="ignore"):
            return map_backtrack(self.plan, bits, arena)[:, :n_report], np.log(val[:, 0])

    def last_recheck_count(self):
        return 0

    def close(self):
        pass
