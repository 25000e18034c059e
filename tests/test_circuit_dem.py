"""The circuit-level noise model behind the detector-sample workload: the
rotated surface-code Z-memory circuit and its detector error model
(tensorqec.jl_gb300/circuit.py, in place of dem.jl:22-145).

``detector_error_model`` propagates every noise component at once, bit-packed
64 per word.  Here every component is propagated on its own through the
circuit by a plain per-qubit Pauli frame, the signatures are merged the way
dem.jl:134-145 merges equal mechanisms (p = p1 (1 - p2) + p2 (1 - p1)), and
the two models must agree mechanism for mechanism.  Structural checks at the
workload's size (d=5, 5 rounds) follow: 72 deterministic detectors, 301
mechanisms of at most two detectors each, the data-qubit readout errors'
signatures, and the sizes the decoder relies on.
"""
import numpy as np
import pytest


def _components(op):
    """(probability, {qubit: (x, z)}) of every Pauli component of a channel."""
    paulis = {1: (1, 0), 2: (1, 1), 3: (0, 1)}
    if op.name == "DEP1":
        return [(op.p / 3, {q: paulis[a]}) for q in op.targets for a in (1, 2, 3)]
    if op.name == "DEP2":
        out = []
        for a, b in zip(op.targets[0::2], op.targets[1::2]):
            for pa in range(4):
                for pb in range(4):
                    if pa or pb:
                        out.append((op.p / 15, {q: paulis[x] for q, x in ((a, pa), (b, pb)) if x}))
        return out
    if op.name == "XERR":
        return [(op.p, {q: (1, 0)}) for q in op.targets]
    return []


def _signature(circ, start, frame):
    """Measurements flipped by a Pauli frame injected after op `start - 1`."""
    x = np.zeros(circ.n_qubits, dtype=bool)
    z = np.zeros(circ.n_qubits, dtype=bool)
    for q, (px, pz) in frame.items():
        x[q] ^= bool(px)
        z[q] ^= bool(pz)
    m = sum(len(op.targets) for op in circ.ops[:start] if op.name == "M")
    flips = set()
    for op in circ.ops[start:]:
        if op.name == "R":
            x[list(op.targets)] = False
            z[list(op.targets)] = False
        elif op.name == "H":
            t = list(op.targets)
            x[t], z[t] = z[t].copy(), x[t].copy()
        elif op.name == "CX":
            for c, tg in zip(op.targets[0::2], op.targets[1::2]):
                x[tg] ^= x[c]
                z[c] ^= z[tg]
        elif op.name == "M":
            for q in op.targets:
                if x[q]:
                    flips.add(m)
                m += 1
    return flips


def _per_fault_model(circ):
    merged = {}
    n_det = len(circ.detectors)
    for oi, op in enumerate(circ.ops):
        for pr, frame in _components(op):
            flips = _signature(circ, oi + 1, frame)
            ds = tuple(i + 1 for i, dt in enumerate(circ.detectors) if len(flips & set(dt)) % 2)
            obs = len(flips & set(circ.observable)) % 2 == 1
            if not ds and not obs:
                continue
            key = ds + ((n_det + 1,) if obs else ())
            q = merged.get(key, 0.0)
            merged[key] = q * (1 - pr) + pr * (1 - q)
    return merged


@pytest.mark.parametrize("d,rounds,p", [(3, 1, 0.01), (3, 3, 0.002), (5, 5, 0.001)])
def test_model_matches_per_fault_propagation(pkg, d, rounds, p):
    from tensorqec_gb300 import circuit

    circ = circuit.memory_z_circuit(d, rounds, p)
    dm = circuit.detector_error_model(circ)
    got = {tuple(f): r for f, r in zip(dm.flipped_detectors, dm.error_rates)}
    assert len(got) == len(dm.error_rates), "two mechanisms with one signature"
    want = _per_fault_model(circ)
    assert got.keys() == want.keys()
    for k in want:
        assert abs(got[k] - want[k]) <= 1e-15 * want[k], k
    assert dm.detector_list == list(range(1, len(circ.detectors) + 1))
    assert dm.logical_list == [len(circ.detectors) + 1]


def test_workload_circuit_structure(pkg):
    """d=5, 5 rounds, p=0.001: 12 Z checks per round plus the readout
    comparison give 72 detectors, all deterministic without noise; a readout
    X error on a data qubit flips the final detectors of the Z checks holding
    it, and the observable exactly for the first row."""
    from tensorqec_gb300 import circuit

    d, rounds = 5, 5
    circ = circuit.memory_z_circuit(d, rounds, 0.001)
    assert len(circ.detectors) == rounds * (d * d - 1) // 2 + (d * d - 1) // 2 == 72
    assert circuit.detectors_deterministic(circ)
    dm = circuit.detector_error_model(circ)
    n_det = 72
    assert all(0 < r < 0.01 for r in dm.error_rates)
    assert all(1 <= f <= n_det + 1 for fl in dm.flipped_detectors for f in fl)
    # 301 independent mechanisms, each flipping at most two detectors (and
    # possibly the observable)
    assert len(dm.error_rates) == 301
    assert max(sum(f <= n_det for f in fl) for fl in dm.flipped_detectors) == 2
    # the readout X_ERROR channel on the data qubits is the last noise op
    last = max(i for i, op in enumerate(circ.ops) if op.name == "XERR")
    assert set(circ.ops[last].targets) == set(range(d * d))
    final = circ.detectors[-(d * d - 1) // 2:]
    meas_base = circ.n_measurements - d * d
    for q in range(d * d):
        flips = _signature(circ, last + 1, {q: (1, 0)})
        assert flips == {meas_base + q}
        hit = [i for i, dt in enumerate(final) if meas_base + q in dt]
        assert 1 <= len(hit) <= 2
        assert (meas_base + q in circ.observable) == (q < d)
    # the decoder's DEM graph of this model: one variable per mechanism and
    # per detector, one output (the observable)
    t = pkg.dem2tanner(dm)
    assert t.ns == n_det and t.nq == len(dm.error_rates)


def test_noiseless_circuit_has_no_mechanisms(pkg):
    from tensorqec_gb300 import circuit

    circ = circuit.memory_z_circuit(3, 2, 0.0)
    assert not any(op.name in ("DEP1", "DEP2", "XERR") for op in circ.ops)
    assert circuit.detectors_deterministic(circ)
    dm = circuit.detector_error_model(circ)
    assert dm.error_rates == [] and dm.flipped_detectors == []
    with pytest.raises(ValueError):
        pkg.parse_dem_string("")
