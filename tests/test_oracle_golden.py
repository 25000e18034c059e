"""The oracle against the reference's own known answers, and against a
brute-force enumeration that does not depend on any contraction order."""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_kat.json")


@pytest.fixture(scope="module")
def kat():
    with open(GOLD) as f:
        return json.load(f)


def test_parity_tensor_kat(oracle, kat):
    pc = oracle.parity_check_matrix(4)
    for idx, want in kat["parity_check_matrix_4"]["entries"]:
        assert pc[tuple(idx)] == want


def test_zero_syndrome_marginal_kat(oracle, kat):
    k = kat["surface3_zero_syndrome_marginal"]
    st, nq = oracle.surface_code_stabilizers(3, 3)
    t = oracle.css_tanner(st, nq)
    lx, lz = oracle.logical_operator(t)
    net = oracle.tnmmap_network(t, k["px"], k["py"], k["pz"], lx, lz)
    mar = oracle.contract(net.ixs, net.tensors, net.iy)
    np.testing.assert_allclose(mar, np.array(k["marginal_julia"]), atol=k["atol"], rtol=0)


def test_logical_operator_kat(oracle, kat):
    k = kat["surface3_logical_operators"]
    st, nq = oracle.surface_code_stabilizers(3, 3)
    lx, lz = oracle.logical_operator(oracle.css_tanner(st, nq))
    assert lx.tolist() == k["lx"]
    assert lz.tolist() == k["lz"]


def test_row_echelon_kat(oracle, kat):
    k = kat["row_echelon_form"]
    R = oracle.row_echelon_form(np.array(k["H"], dtype=bool)).astype(int)
    assert R.tolist() == k["R"]


def test_null_space_property(oracle, kat):
    k = kat["null_space_hamming"]
    H = np.array(k["H"], dtype=bool)
    ns = oracle.null_space(H)
    assert list(ns.shape) == k["shape"]
    assert not ((H.astype(int) @ ns.T.astype(int)) % 2).any()


def test_toric_stabilizers_kat(oracle, kat):
    st, nq = oracle.toric_code_stabilizers(2, 3)
    code = {"X": 2, "Z": 4}
    got = []
    for t, s in st:
        ops = [1] * nq
        for q in s:
            ops[q - 1] = code[t]
        got.append(ops)
    assert got == kat["toric_2x3_stabilizers"]["ops"]


def test_brute_force_matches_contraction_d3(oracle):
    """Every one of the 256 syndromes at d=3, depolarising p=0.05."""
    st, nq = oracle.surface_code_stabilizers(3, 3)
    t = oracle.css_tanner(st, nq)
    lx, lz = oracle.logical_operator(t)
    p = 0.05 / 3
    brute = oracle.brute_force_marginals(t, p, p, p, lx, lz)
    dec = oracle.OracleDecoder(t, p, p, p)
    for sidx in range(0, 256, 5):
        bits = [(sidx >> j) & 1 for j in range(8)]
        np.testing.assert_allclose(dec.marginal(bits), brute[sidx], rtol=1e-12, atol=1e-300)


def test_brute_force_zero_syndrome_kat(oracle, kat):
    k = kat["surface3_zero_syndrome_marginal"]
    st, nq = oracle.surface_code_stabilizers(3, 3)
    t = oracle.css_tanner(st, nq)
    lx, lz = oracle.logical_operator(t)
    brute = oracle.brute_force_marginals(t, k["px"], k["py"], k["pz"], lx, lz)
    want = np.array(k["marginal_julia"]).flatten(order="F")
    np.testing.assert_allclose(brute[0], want, atol=k["atol"], rtol=0)


def test_decision_kat_x1(oracle, kat):
    """tndecoder.jl:60-73: X on qubit 1 with px=0.1 decodes without a
    logical error (class of X1 is the argmax class)."""
    k = kat["surface3_decision_x1"]
    st, nq = oracle.surface_code_stabilizers(3, 3)
    t = oracle.css_tanner(st, nq)
    dec = oracle.OracleDecoder(t, k["px"], 0.0, 0.0)
    ex = np.array(k["error_x"], dtype=np.uint8)
    ez = np.zeros(9, dtype=np.uint8)
    sx, sz = oracle.syndrome_extraction(ex, ez, t)
    mar = dec.marginal(np.concatenate([sx[0], sz[0]]))
    cls = int(np.argmax(mar))
    b_true = int(dec.lz[0] @ ex) % 2   # class bit of X1 (logical-z parity)
    assert cls == 2 * b_true  # a = 0 (no Z error), b = lz.ex
    assert (cls != 2 * b_true) == k["logical_error"]


def test_dem_parse_kat(oracle, kat):
    dem = oracle.parse_dem_string(kat["dem_small"]["text"])
    assert len(dem.error_rates) == 21
    assert dem.detector_list == [1, 2, 3, 4, 5, 6]
    assert dem.logical_list == [7]
    assert dem.flipped[3] == [1, 2, 7]


def test_dem_marginal_brute_force(oracle, kat):
    """DEM TNMMAP (tndecoder.jl:186-253) on the reference's dem.dem: the
    contraction equals enumeration over all 2^21 mechanism subsets (chunked)."""
    dem = oracle.parse_dem_string(kat["dem_small"]["text"])
    dec = oracle.OracleDEMDecoder(dem, factorize=True)
    t = dec.tanner
    p = np.array(dem.error_rates)
    nq = len(p)
    L = np.zeros(nq, dtype=np.int64)
    for j in dec.l2q[0]:
        L[j - 1] = 1
    tot = np.zeros((64, 2))
    H = t.H.astype(np.int64)
    for hi in range(1 << (nq - 14)):
        idx = (hi << 14) + np.arange(1 << 14)
        e = ((idx[:, None] >> np.arange(nq)[None, :]) & 1)
        pr = np.prod(np.where(e == 1, p, 1 - p), axis=1)
        s = (e @ H.T) % 2
        sid = (s << np.arange(6)).sum(axis=1)
        lg = (e @ L) % 2
        np.add.at(tot, (sid, lg), pr)
    for sid in (0, 1, 5, 17, 42, 63):
        bits = [(sid >> j) & 1 for j in range(6)]
        np.testing.assert_allclose(dec.marginal(bits), tot[sid], rtol=1e-11, atol=1e-300)
