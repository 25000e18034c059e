"""Detector error models (TensorQEC's src/decoding/dem.jl and
src/stim_parser/stim_parser.jl:337-375)."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .codes import SimpleTannerGraph


@dataclass
class DetectorErrorModel:
    """dem.jl:1-6.  ``flipped_detectors[i]`` lists the 1-based detectors and
    (renumbered after the last detector) logicals that mechanism i flips."""
    error_rates: list
    flipped_detectors: list
    detector_list: list
    logical_list: list


def parse_dem_string(content: str) -> DetectorErrorModel:
    """stim_parser.jl:342-375: only ``error(p) D.. L..`` lines are read;
    ``repeat`` blocks are rejected."""
    rates, dets, logs = [], [], []
    for line in content.split("\n"):
        if not line:
            continue
        s = line.split()
        if not s:
            continue
        if s[0].startswith("error("):
            rates.append(float(s[0][6:-1]))
            dets.append([int(t[1:]) + 1 for t in s[1:] if t.startswith("D")])
            logs.append([int(t[1:]) + 1 for t in s[1:] if t.startswith("L")])
        elif s[0].startswith("repeat"):
            raise ValueError("repeat is not supported; flatten the loops when exporting the model")
    if not rates:
        raise ValueError("no error mechanisms in the model")
    largest = max((max(d) for d in dets if d), default=0)
    logs = [[x + largest for x in lg] for lg in logs]
    largest_l = max((max(lg) for lg in logs if lg), default=0)
    flipped = []
    for d, lg in zip(dets, logs):
        seen = []
        for x in d + lg:
            if x not in seen:
                seen.append(x)
        flipped.append(seen)
    return DetectorErrorModel(rates, flipped, list(range(1, largest + 1)),
                              list(range(largest + 1, largest_l + 1)))


def parse_dem_file(path: str) -> DetectorErrorModel:
    with open(path) as f:
        return parse_dem_string(f.read())


def dem2tanner(dem: DetectorErrorModel) -> SimpleTannerGraph:
    """dem.jl:150-160: bits are error mechanisms, checks are detectors."""
    logical = set(dem.logical_list)
    q2s = [[v for v in f if v not in logical] for f in dem.flipped_detectors]
    ns = max(dem.detector_list) if dem.detector_list else 0
    s2q = [[j + 1 for j, q in enumerate(q2s) if i in q] for i in range(1, ns + 1)]
    return SimpleTannerGraph(len(dem.error_rates), s2q)


def logical_map(dem: DetectorErrorModel) -> list:
    """``l2q`` of compile(::TNMMAP, ::DetectorErrorModel) (tndecoder.jl:188):
    for each logical, the 1-based mechanisms that flip it."""
    return [[j + 1 for j, f in enumerate(dem.flipped_detectors) if i in f] for i in dem.logical_list]


def to_dem_string(dem: DetectorErrorModel) -> str:
    """Writes the model back in the text form ``parse_dem_string`` reads."""
    nd = len(dem.detector_list)
    lines = []
    for p, f in zip(dem.error_rates, dem.flipped_detectors):
        toks = [f"error({p!r})"]
        toks += [f"D{v - 1}" for v in f if v <= nd]
        toks += [f"L{v - nd - 1}" for v in f if v > nd]
        lines.append(" ".join(toks))
    return "\n".join(lines) + "\n"


def sample_dem(dem: DetectorErrorModel, nsamples: int, rng=None):
    """Independent mechanisms (random_error_pattern(dem), dem.jl:162-164),
    batched: returns (errors (n, nq) uint8, detectors (n, ns) uint8,
    logicals (n, nl) uint8)."""
    rng = np.random.default_rng() if rng is None else rng
    p = np.asarray(dem.error_rates)
    e = (rng.random((nsamples, p.size)) < p).astype(np.uint8)
    t = dem2tanner(dem)
    det = ((e.astype(np.int64) @ t.H.T.astype(np.int64)) % 2).astype(np.uint8)
    L = np.zeros((len(dem.logical_list), p.size), dtype=np.int64)
    for i, l in enumerate(logical_map(dem)):
        L[i, np.array(l, dtype=np.int64) - 1] = 1
    lg = ((e.astype(np.int64) @ L.T) % 2).astype(np.uint8)
    return e, det, lg
