"""Circuit-level noise: a rotated surface-code Z-memory circuit and its
detector error model.

``memory_z_circuit(d, rounds, p)`` lays out the standard rotated surface
code (d x d data qubits, d^2 - 1 measure qubits, CNOT order chosen so hook
errors run perpendicular to the Z logical) and runs ``rounds`` rounds of
syndrome extraction followed by a Z-basis readout of every data qubit.
Noise: after every 1-qubit gate a depolarising channel with total rate p
(X, Y, Z each p/3), after every CNOT a 2-qubit depolarising channel (each of
the 15 non-identity Paulis with p/15), after every reset an X flip with
rate p, and before every measurement an X flip with rate p.

Detectors are the Z-type stabiliser outcomes compared across consecutive
rounds (the first round against the deterministic +1 of |0...0>, the last
against the data readout); the observable is the Z logical on the first
row of data qubits.  ``detector_error_model`` propagates every Pauli
component of every channel through the Clifford circuit as a Pauli frame
(all components in parallel, bit-packed), and merges components with equal
(detector, observable) signatures by XOR-ing independent probabilities
(as dem.jl:134-145 does: p = p1 (1 - p2) + p2 (1 - p1)).  Components that
flip nothing are dropped.

This replaces TensorQEC's Yao-based circuit -> DEM path (dem.jl:22-145),
which asserts single-qubit depolarising noise only (dem.jl:42-43).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .dem import DetectorErrorModel


@dataclass
class Op:
    name: str            # "R", "H", "CX", "M", "DEP1", "DEP2", "XERR"
    targets: tuple       # qubit ids (pairs for CX / DEP2)
    p: float = 0.0


@dataclass
class Circuit:
    n_qubits: int
    ops: list = field(default_factory=list)
    detectors: list = field(default_factory=list)   # lists of measurement indices
    observable: list = field(default_factory=list)  # measurement indices
    n_measurements: int = 0

    def to_stim_text(self) -> str:
        """The circuit in stim's text format (for inspection and export)."""
        lines = []
        names = {"R": "R", "H": "H", "CX": "CX", "M": "M", "DEP1": "DEPOLARIZE1", "DEP2": "DEPOLARIZE2",
                 "XERR": "X_ERROR"}
        m = 0
        for op in self.ops:
            arg = f"({op.p!r})" if op.name in ("DEP1", "DEP2", "XERR") else ""
            lines.append(f"{names[op.name]}{arg} " + " ".join(str(q) for q in op.targets))
            if op.name == "M":
                m += len(op.targets)
        for det in self.detectors:
            lines.append("DETECTOR " + " ".join(f"rec[{i - self.n_measurements}]" for i in det))
        lines.append("OBSERVABLE_INCLUDE(0) " + " ".join(f"rec[{i - self.n_measurements}]" for i in self.observable))
        return "\n".join(lines) + "\n"


def _layout(d):
    """Coordinates: data qubit (r, c) for 0 <= r, c < d at (2r+1, 2c+1);
    measure qubits at even coordinates on plaquette corners."""
    data = {(2 * r + 1, 2 * c + 1): r * d + c for r in range(d) for c in range(d)}
    xs, zs = [], []
    for r in range(d + 1):
        for c in range(d + 1):
            pos = (2 * r, 2 * c)
            # plaquette type alternates; boundary plaquettes only on two sides each
            is_x = (r + c) % 2 == 1
            inside_r = 0 < r < d
            inside_c = 0 < c < d
            if inside_r and inside_c:
                (xs if is_x else zs).append(pos)
            elif is_x and (r == 0 or r == d) and inside_c:
                xs.append(pos)          # X boundary plaquettes on top/bottom
            elif (not is_x) and (c == 0 or c == d) and inside_r:
                zs.append(pos)          # Z boundary plaquettes on left/right
    return data, xs, zs


def _neighbours(pos, data):
    r, c = pos
    out = {}
    for key, (dr, dc) in {"nw": (-1, -1), "ne": (-1, 1), "sw": (1, -1), "se": (1, 1)}.items():
        q = data.get((r + dr, c + dc))
        if q is not None:
            out[key] = q
    return out


def memory_z_circuit(d: int, rounds: int, p: float) -> Circuit:
    data, xs, zs = _layout(d)
    nd = d * d
    anc = {}
    for pos in xs + zs:
        anc[pos] = nd + len(anc)
    nq = nd + len(anc)
    circ = Circuit(nq)
    ops = circ.ops
    all_data = tuple(range(nd))
    x_anc = tuple(anc[pos] for pos in xs)
    z_anc = tuple(anc[pos] for pos in zs)
    all_anc = x_anc + z_anc
    # CNOT schedule: X plaquettes nw, ne, sw, se; Z plaquettes nw, sw, ne, se
    order_x = ("nw", "ne", "sw", "se")
    order_z = ("nw", "sw", "ne", "se")

    ops.append(Op("R", all_data + all_anc))
    if p > 0:
        ops.append(Op("XERR", all_data + all_anc, p))
    meas = 0
    last_z = {}
    for rnd in range(rounds):
        if rnd > 0:
            ops.append(Op("R", all_anc))
            if p > 0:
                ops.append(Op("XERR", all_anc, p))
        ops.append(Op("H", x_anc))
        if p > 0:
            ops.append(Op("DEP1", x_anc, p))
        for layer in range(4):
            pairs = []
            for pos in xs:
                nb = _neighbours(pos, data)
                q = nb.get(order_x[layer])
                if q is not None:
                    pairs.append((anc[pos], q))        # X check: ancilla controls data
            for pos in zs:
                nb = _neighbours(pos, data)
                q = nb.get(order_z[layer])
                if q is not None:
                    pairs.append((q, anc[pos]))        # Z check: data controls ancilla
            flat = tuple(x for pr in pairs for x in pr)
            ops.append(Op("CX", flat))
            if p > 0:
                ops.append(Op("DEP2", flat, p))
        ops.append(Op("H", x_anc))
        if p > 0:
            ops.append(Op("DEP1", x_anc, p))
            ops.append(Op("XERR", all_anc, p))
        ops.append(Op("M", all_anc))
        idx = {q: meas + i for i, q in enumerate(all_anc)}
        meas += len(all_anc)
        for pos in zs:
            cur = idx[anc[pos]]
            circ.detectors.append([cur] if rnd == 0 else [last_z[pos], cur])
            last_z[pos] = cur
    if p > 0:
        ops.append(Op("XERR", all_data, p))
    ops.append(Op("M", all_data))
    didx = {q: meas + i for i, q in enumerate(all_data)}
    meas += nd
    for pos in zs:
        nb = _neighbours(pos, data)
        circ.detectors.append([last_z[pos]] + [didx[q] for q in nb.values()])
    # Z logical: the first row of data qubits (even overlap with every X check)
    circ.observable = [didx[data[(1, 2 * c + 1)]] for c in range(d)]
    circ.n_measurements = meas
    return circ


def _components(op):
    """(probability, [(qubit, pauli)]) of every Pauli component of a channel;
    pauli in {1: X, 2: Y, 3: Z}."""
    out = []
    if op.name == "DEP1":
        for q in op.targets:
            for pa in (1, 2, 3):
                out.append((op.p / 3, [(q, pa)]))
    elif op.name == "DEP2":
        t = op.targets
        for i in range(0, len(t), 2):
            a, b = t[i], t[i + 1]
            for pa in range(4):
                for pb in range(4):
                    if pa == 0 and pb == 0:
                        continue
                    comp = [(q, pp) for q, pp in ((a, pa), (b, pb)) if pp]
                    out.append((op.p / 15, comp))
    elif op.name == "XERR":
        for q in op.targets:
            out.append((op.p, [(q, 1)]))
    return out


def detector_error_model(circ: Circuit) -> DetectorErrorModel:
    """Pauli-frame propagation of every noise component (bit-packed over
    components) through the circuit; returns the merged model in the
    reference's DetectorErrorModel form (detectors 1..n_det, the observable
    n_det + 1)."""
    comps = []   # (op index, probability, paulis)
    for oi, op in enumerate(circ.ops):
        for pr, paulis in _components(op):
            comps.append((oi, pr, paulis))
    F = len(comps)
    nw = (F + 63) // 64
    X = np.zeros((circ.n_qubits, nw), dtype=np.uint64)
    Z = np.zeros((circ.n_qubits, nw), dtype=np.uint64)
    mflip = np.zeros((circ.n_measurements, nw), dtype=np.uint64)
    by_op = {}
    for f, (oi, pr, paulis) in enumerate(comps):
        by_op.setdefault(oi, []).append((f, paulis))
    m = 0
    one = np.uint64(1)
    for oi, op in enumerate(circ.ops):
        if op.name == "R":
            for q in op.targets:
                X[q] = 0
                Z[q] = 0
        elif op.name == "H":
            for q in op.targets:
                X[q], Z[q] = Z[q].copy(), X[q].copy()
        elif op.name == "CX":
            t = op.targets
            for i in range(0, len(t), 2):
                c, tg = t[i], t[i + 1]
                X[tg] ^= X[c]
                Z[c] ^= Z[tg]
        elif op.name == "M":
            for q in op.targets:
                mflip[m] = X[q]
                m += 1
        # a channel injects its components after the gate it follows
        for f, paulis in by_op.get(oi, []):
            w, b = divmod(f, 64)
            bit = one << np.uint64(b)
            for q, pa in paulis:
                if pa in (1, 2):
                    X[q, w] ^= bit
                if pa in (2, 3):
                    Z[q, w] ^= bit
    # detector and observable signatures per component
    def bits_of(rows):
        acc = np.zeros(nw, dtype=np.uint64)
        for r in rows:
            acc ^= mflip[r]
        return np.unpackbits(acc.view(np.uint8), bitorder="little")[:F].astype(bool)

    det = np.stack([bits_of(dt) for dt in circ.detectors], axis=0)    # (n_det, F)
    obs = bits_of(circ.observable)
    merged = {}
    for f, (oi, pr, paulis) in enumerate(comps):
        ds = tuple(int(i) + 1 for i in np.flatnonzero(det[:, f]))
        key = (ds, bool(obs[f]))
        if not ds and not key[1]:
            continue
        q = merged.get(key, 0.0)
        merged[key] = q * (1 - pr) + pr * (1 - q)
    n_det = len(circ.detectors)
    rates, flipped = [], []
    for (ds, o), pr in sorted(merged.items(), key=lambda kv: (kv[0][0], kv[0][1])):
        rates.append(pr)
        flipped.append(list(ds) + ([n_det + 1] if o else []))
    return DetectorErrorModel(rates, flipped, list(range(1, n_det + 1)), [n_det + 1])


def detectors_deterministic(circ: Circuit) -> bool:
    """True when every detector and the observable of the noiseless circuit
    are deterministic: each, propagated backwards (Heisenberg picture)
    through the Clifford gates, meets resets only with Z support and every
    measurement it does not include only with Z support."""
    meas_at = []  # (op index, qubit) per measurement index
    for oi, op in enumerate(circ.ops):
        if op.name == "M":
            for q in op.targets:
                meas_at.append((oi, q))
    checks = [set(dt) for dt in circ.detectors] + [set(circ.observable)]
    for members in checks:
        x = np.zeros(circ.n_qubits, dtype=bool)
        z = np.zeros(circ.n_qubits, dtype=bool)
        mi = len(meas_at)
        for oi in range(len(circ.ops) - 1, -1, -1):
            op = circ.ops[oi]
            if op.name == "M":
                for q in reversed(op.targets):
                    mi -= 1
                    if x[q]:
                        return False        # anticommutes with a measurement
                    if mi in members:
                        z[q] ^= True
            elif op.name == "R":
                for q in op.targets:
                    if x[q]:
                        return False
                    z[q] = False
            elif op.name == "H":
                for q in op.targets:
                    x[q], z[q] = z[q], x[q]
            elif op.name == "CX":
                t = op.targets
                for i in range(len(t) - 2, -1, -2):
                    c, tg = t[i], t[i + 1]
                    # CX conjugation is its own inverse on Pauli frames
                    x[tg] ^= x[c]
                    z[c] ^= z[tg]
        if x.any() or z.any():
            return False
    return True
