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
