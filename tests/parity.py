"""Parity checks shared by the GPU tests.

The plain float64 form must give the reference's class log-probabilities
within 1e-10 relative, class by class: for every class whose oracle
probability p_ref is positive, |logp - log p_ref| <= 1e-10 * |log p_ref|, and
logp is -inf on exactly the classes whose p_ref is zero.  Reduced precision
is held to its own rounding bound the same way: the planner's bound is a
relative error of every class probability (all operands are non-negative),
so |logp - log p_ref| <= 2 * bound on every class that float32 can represent
relative to the row's largest (classes at least 1e-25 of it; float32
intermediates keep about 38 decades below their maximum).

Decisions: the class equals the oracle's first maximum, except on rows whose
top two oracle classes are within 1e-9 relative (a tie that summation order
decides), where the chosen class must be one of the tied maxima.
"""
import numpy as np

TIE = 1e-9
F32_FLOOR = 1e-25


def ties(want_p):
    want_p = np.asarray(want_p, dtype=np.float64)
    srt = np.sort(want_p, axis=1)
    top = srt[:, -1]
    return (top - srt[:, -2]) <= TIE * np.maximum(top, 1e-300)


def assert_decisions(cls, want_p):
    want_p = np.asarray(want_p, dtype=np.float64)
    cls = np.asarray(cls)
    tie = ties(want_p)
    best = want_p.argmax(axis=1)
    bad = (cls != best) & ~tie
    assert not bad.any(), f"{bad.sum()} decision mismatches outside ties, rows {np.flatnonzero(bad)[:10]}"
    top = want_p.max(axis=1)
    assert (want_p[np.arange(len(cls)), cls] >= top * (1 - TIE)).all()


def assert_class_logprobs(logp, want_p, rel=1e-10):
    """Per class: |logp - log p_ref| <= rel * |log p_ref| where p_ref > 0;
    -inf exactly where p_ref == 0."""
    logp = np.asarray(logp, dtype=np.float64)
    want_p = np.asarray(want_p, dtype=np.float64)
    assert logp.shape == want_p.shape
    zero = want_p == 0.0
    assert np.isneginf(logp[zero]).all(), "a class the oracle gives probability 0 is finite"
    assert np.isfinite(logp[~zero]).all(), "a class with positive oracle probability is -inf or nan"
    lw = np.log(want_p[~zero])
    err = np.abs(logp[~zero] - lw)
    lim = rel * np.abs(lw)
    worst = np.argmax(err / np.maximum(lim, 1e-300)) if err.size else 0
    assert (err <= lim).all(), (f"class log-probability error {err[worst]:.3e} > {rel:.0e} x |log p| "
                                f"= {lim[worst]:.3e} (log p_ref = {lw[worst]:.6f})")


def assert_class_logprobs_within(logp, want_p, bound, floor=F32_FLOOR):
    """Reduced precision: |logp - log p_ref| <= bound on every class with
    p_ref >= floor * (row maximum); classes the oracle gives 0 are -inf."""
    logp = np.asarray(logp, dtype=np.float64)
    want_p = np.asarray(want_p, dtype=np.float64)
    zero = want_p == 0.0
    assert np.isneginf(logp[zero]).all(), "a class the oracle gives probability 0 is finite"
    live = want_p >= floor * want_p.max(axis=1, keepdims=True)
    live &= ~zero
    err = np.abs(logp[live] - np.log(want_p[live]))
    assert err.size == 0 or err.max() <= bound, f"class log-probability error {err.max():.3e} > {bound:.3e}"
