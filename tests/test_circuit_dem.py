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
    """(probability, {qubit: (x, z)}) of the independent Pauli channels of a
    noise op: a depolarising channel is the composition of one channel per
    non-identity Pauli, each of rate q with (1 - 2q)^2 = 1 - 4p/3 on one qubit
    (dem.jl:44-63) and (1 - 2q)^8 = 1 - 16p/15 on two."""
    paulis = {1: (1, 0), 2: (1, 1), 3: (0, 1)}
    if op.name == "DEP1":
        q1 = 0.5 * (1 - np.sqrt(1 - 4 * op.p / 3))
        return [(q1, {q: paulis[a]}) for q in op.targets for a in (1, 2, 3)]
    if op.name == "DEP2":
        q2 = 0.5 * (1 - (1 - 16 * op.p / 15) ** 0.125)
        out = []
        for a, b in zip(op.targets[0::2], op.targets[1::2]):
            for pa in range(4):
                for pb in range(4):
                    if pa or pb:
                        out.append((q2, {q: paulis[x] for q, x in ((a, pa), (b, pb)) if x}))
        return out
    if op.name in ("XERR", "YERR", "ZERR"):
        pa = paulis[{"XERR": 1, "YERR": 2, "ZERR": 3}[op.name]]
        return [(op.p, {q: pa}) for q in op.targets]
    return []


def _signature(circ, start, frame):
    """Measurements flipped by a Pauli frame injected after op `start - 1`."""
    x = np.zeros(circ.n_qubits, dtype=bool)
    z = np.zeros(circ.n_qubits, dtype=bool)
    for q, (px, pz) in frame.items():
        x[q] ^= bool(px)
        z[q] ^= bool(pz)
    m = sum(len(op.targets) for op in circ.ops[:start] if op.name in ("M", "MX", "MR"))
    flips = set()
    for op in circ.ops[start:]:
        if op.name in ("R", "RX"):
            x[list(op.targets)] = False
            z[list(op.targets)] = False
        elif op.name == "H":
            t = list(op.targets)
            x[t], z[t] = z[t].copy(), x[t].copy()
        elif op.name == "S":
            for q in op.targets:
                z[q] ^= x[q]
        elif op.name in ("CXYZ", "CZYX"):
            # conjugation by C_XYZ sends X to Y, Y to Z, Z to X
            cyc = {(1, 0): (1, 1), (1, 1): (0, 1), (0, 1): (1, 0), (0, 0): (0, 0)}
            if op.name == "CZYX":
                cyc = {v: k for k, v in cyc.items()}
            for q in op.targets:
                x[q], z[q] = cyc[(int(x[q]), int(z[q]))]
        elif op.name == "CX":
            for c, tg in zip(op.targets[0::2], op.targets[1::2]):
                x[tg] ^= x[c]
                z[c] ^= z[tg]
        elif op.name == "CZ":
            for a, b in zip(op.targets[0::2], op.targets[1::2]):
                z[a] ^= x[b]
                z[b] ^= x[a]
        elif op.name in ("M", "MX", "MR"):
            for q in op.targets:
                if (z[q] if op.name == "MX" else x[q]):
                    flips.add(m)
                m += 1
                if op.name == "MR":
                    x[q] = z[q] = False
    return flips


def _per_fault_model(circ):
    merged = {}
    n_det = len(circ.detectors)
    for oi, op in enumerate(circ.ops):
        for pr, frame in _components(op):
            flips = _signature(circ, oi + 1, frame)
            ds = tuple(i + 1 for i, dt in enumerate(circ.detectors) if len(flips & set(dt)) % 2)
            obs = tuple(n_det + 1 + k for k, o in enumerate(circ.observables) if len(flips & set(o)) % 2)
            if not ds and not obs:
                continue
            key = ds + obs
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


def _kat():
    import json
    import os

    with open(os.path.join(os.path.dirname(__file__), "golden", "reference_kat.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("case", range(4))
def test_reference_dem_known_answers(pkg, case):
    """test/decoding/dem.jl:5-86: the reference's circuit -> DEM answers
    (merged X_ERROR and DEPOLARIZE1 rates, resets, propagation through H
    and CX), through the stim text parser."""
    from tensorqec_gb300 import circuit

    k = _kat()["dem_from_circuit"]["cases"][case]
    circ = circuit.parse_stim_string(k["circuit"], k["n_qubits"])
    assert circ.n_qubits == k["n_qubits"]
    dm = circuit.detector_error_model(circ)
    got = {tuple(f): r for f, r in zip(dm.flipped_detectors, dm.error_rates)}
    want = {tuple(f): r for f, r in zip(k["flipped_detectors"], k["error_rates"])}
    assert got.keys() == want.keys()
    for key in want:
        assert abs(got[key] - want[key]) <= 1e-10, (key, got[key], want[key])


def test_reference_stim_parse_known_answers(pkg):
    """test/stim_parser/stim_parser.jl:5-48: nested REPEAT blocks and a
    noisy measurement parse; an unknown instruction is an error."""
    from tensorqec_gb300 import circuit

    k = _kat()["stim_parse"]
    circ = circuit.parse_stim_string(k["circuit"], k["n_qubits"])
    assert circ.n_qubits == 7
    assert circ.n_measurements == 3 + 2 * 3 + 4
    assert len(circ.detectors) == 3 + 2 * 3 + 3
    assert circ.observables == [[circ.n_measurements - 1]]
    # the second round's first detector compares its first MR with the first round's
    assert circ.detectors[3] == [3, 0]
    # M(0.1) puts a 0.1 X flip in front of the readout of qubits 0, 2, 4, 6
    flip = [op for op in circ.ops if op.name == "XERR"]
    assert len(flip) == 1 and flip[0].targets == (0, 2, 4, 6) and flip[0].p == 0.1
    with pytest.raises(ValueError):
        circuit.parse_stim_string(k["bad_circuit"], 5)


def test_stim_text_round_trip_of_the_workload_circuit(pkg):
    """The d=5, 5-round Z-memory circuit written as stim text and read back
    gives the same detector error model."""
    from tensorqec_gb300 import circuit

    circ = circuit.memory_z_circuit(5, 5, 0.001)
    back = circuit.parse_stim_string(circ.to_stim_text())
    assert back.n_qubits == circ.n_qubits and back.n_measurements == circ.n_measurements
    assert back.detectors == circ.detectors and back.observables == circ.observables
    a, b = circuit.detector_error_model(circ), circuit.detector_error_model(back)
    assert a.flipped_detectors == b.flipped_detectors and a.error_rates == b.error_rates


def test_parsed_circuit_with_x_basis_and_cz(pkg):
    """X-basis reset and measurement, S and CZ: an X-basis Bell-pair check
    is deterministic, Z errors on the pair flip it, X errors do not, and the
    per-fault propagation agrees with the bit-packed model."""
    from tensorqec_gb300 import circuit

    text = """
    RX 0 1
    H 1
    CZ 0 1
    H 1
    S 2
    Z_ERROR(0.05) 0
    X_ERROR(0.07) 1
    DEPOLARIZE1(0.03) 0
    MX 0 1
    DETECTOR rec[-1] rec[-2]
    """
    circ = circuit.parse_stim_string(text)
    assert circ.n_qubits == 3
    assert circuit.detectors_deterministic(circ)
    dm = circuit.detector_error_model(circ)
    want = _per_fault_model(circ)
    got = {tuple(f): r for f, r in zip(dm.flipped_detectors, dm.error_rates)}
    assert got.keys() == want.keys() == {(1,)}
    q = 0.5 * (1 - np.sqrt(1 - 4 * 0.03 / 3))
    z = 2 * q * (1 - q)  # the Z and Y components of the depolarising channel
    assert abs(got[(1,)] - (0.05 * (1 - z) + z * (1 - 0.05))) < 1e-15


def test_insert_errors_rebuilds_the_workload_noise(pkg):
    """insert_errors (dem.jl:166-207) on the noiseless Z-memory circuit with
    p everywhere gives the noisy circuit's model mechanism for mechanism."""
    from tensorqec_gb300 import circuit

    for d, rounds, p in ((3, 2, 0.004), (5, 5, 0.001)):
        clean = circuit.memory_z_circuit(d, rounds, 0.0)
        noisy = circuit.insert_errors(clean, p, p, p)
        a = circuit.detector_error_model(circuit.memory_z_circuit(d, rounds, p))
        b = circuit.detector_error_model(noisy)
        assert a.flipped_detectors == b.flipped_detectors
        np.testing.assert_allclose(a.error_rates, b.error_rates, rtol=1e-14)


def test_reference_insert_errors_circuit(pkg):
    """The circuit of test/decoding/dem.jl:88-128 (with MR and C_XYZ): noise
    lands where insert_errors puts it, the model matches per-fault
    propagation, and C_XYZ followed by C_ZYX is the identity."""
    from tensorqec_gb300 import circuit

    text = """
    H 0 1
    CX 0 1
    M 0
    MR 1
    DETECTOR rec[-1] rec[-2]
    R 1
    CX 1 0
    M 0 1
    DETECTOR rec[-1] rec[-2]
    C_XYZ 1
    """
    circ = circuit.parse_stim_string(text, 2)
    noisy = circuit.insert_errors(circ, after_clifford_depolarization=0.01, after_reset_flip_probability=0.02,
                                  before_measure_flip_probability=0.03)
    names = [op.name for op in noisy.ops]
    assert names == ["H", "DEP1", "CX", "DEP2", "XERR", "M", "XERR", "MR", "XERR", "R", "XERR", "CX", "DEP2",
                     "XERR", "M", "CXYZ", "DEP1"]
    dm = circuit.detector_error_model(noisy)
    got = {tuple(f): r for f, r in zip(dm.flipped_detectors, dm.error_rates)}
    want = _per_fault_model(noisy)
    assert got.keys() == want.keys() and got
    for k in want:
        assert abs(got[k] - want[k]) <= 1e-15 * want[k]
    # C_XYZ then C_ZYX leaves every frame as it was
    twice = circuit.parse_stim_string("RX 0\nR 1\nC_XYZ 0 1\nC_ZYX 0 1\nMX 0\nM 1\nDETECTOR rec[-2]\n"
                                      "DETECTOR rec[-1]\n")
    assert circuit.detectors_deterministic(twice)
    once = circuit.parse_stim_string("RX 0\nC_XYZ 0\nMX 0\nDETECTOR rec[-1]\n")
    assert not circuit.detectors_deterministic(once)


def test_mechanism_order(pkg):
    """Mechanisms are listed by their detectors, then by their observables,
    so a model's factor graph (and the contraction order searched for it)
    does not move when rates change."""
    from tensorqec_gb300 import circuit

    dm = circuit.detector_error_model(circuit.memory_z_circuit(5, 5, 0.001))
    n_det = len(dm.detector_list)
    keys = [(tuple(v for v in f if v <= n_det), tuple(v for v in f if v > n_det)) for f in dm.flipped_detectors]
    assert keys == sorted(keys) and len(set(keys)) == len(keys)
    other = circuit.detector_error_model(circuit.memory_z_circuit(5, 5, 0.003))
    assert other.flipped_detectors == dm.flipped_detectors
