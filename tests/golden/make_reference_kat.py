"""Writes reference_kat.json: known answers from TensorQEC.jl's own tests.

Each entry cites the reference test it comes from (paths relative to the
TensorQEC.jl project root).  The detector error model fixture is the one the
reference's DEM decoder test reads; when the reference tree is mounted the
script copies it from there, otherwise it keeps the committed copy.
Run:  python tests/golden/make_reference_kat.py [path-to-TensorQEC.jl]
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "reference_kat.json")


def main(ref_root=None):
    kat = {
        "parity_check_matrix_4": {
            "source": "test/decoding/tndecoder.jl:8-14",
            "entries": [[[0, 0, 0, 0, 0], 1], [[0, 0, 0, 0, 1], 0], [[0, 1, 0, 1, 0], 1], [[1, 0, 1, 1, 0], 0]],
            "note": "0-based indices of mat[1,1,1,1,1], mat[1,1,1,1,2], mat[1,2,1,2,1], mat[2,1,2,2,1]",
        },
        "surface3_zero_syndrome_marginal": {
            "source": "test/decoding/tndecoder.jl:101-110",
            "code": "SurfaceCode(3,3)",
            "px": 0.1, "py": 0.0, "pz": 0.0,
            "marginal_julia": [[0.3972875040000002, 0.004284496000000001], [0.0, 0.0]],
            "atol": 1e-10,
            "note": "ct.code(ct.tensors...) right after compile: every syndrome leaf is [1,0]",
        },
        "surface3_logical_operators": {
            "source": "test/codes/code_distance.jl:54-59",
            "lx": [[0, 0, 0, 0, 0, 0, 1, 1, 1]],
            "lz": [[1, 0, 0, 0, 1, 0, 0, 0, 1]],
        },
        "row_echelon_form": {
            "source": "test/codes/code_distance.jl:18-39",
            "H": [[1, 1, 0, 1, 0, 0, 1, 0, 1, 0], [1, 1, 0, 1, 1, 0, 0, 1, 1, 1], [1, 0, 0, 1, 1, 1, 1, 1, 1, 1],
                  [0, 1, 0, 0, 1, 0, 0, 0, 0, 0], [0, 0, 1, 1, 1, 1, 1, 1, 0, 1], [1, 1, 0, 1, 1, 0, 0, 1, 1, 0],
                  [0, 0, 1, 0, 1, 0, 0, 0, 0, 1], [1, 0, 0, 1, 0, 0, 1, 0, 1, 0], [1, 0, 1, 0, 0, 0, 0, 1, 0, 1],
                  [0, 1, 0, 1, 1, 1, 0, 1, 1, 0]],
            "R": [[1, 0, 0, 0, 0, 0, 0, 0, 1, 0], [0, 1, 0, 0, 0, 0, 0, 0, 0, 0], [0, 0, 1, 0, 0, 0, 0, 0, 0, 0],
                  [0, 0, 0, 1, 0, 0, 0, 0, 1, 0], [0, 0, 0, 0, 1, 0, 0, 0, 0, 0], [0, 0, 0, 0, 0, 1, 0, 0, 1, 0],
                  [0, 0, 0, 0, 0, 0, 1, 0, 1, 0], [0, 0, 0, 0, 0, 0, 0, 1, 1, 0], [0, 0, 0, 0, 0, 0, 0, 0, 0, 1],
                  [0, 0, 0, 0, 0, 0, 0, 0, 0, 0]],
        },
        "null_space_hamming": {
            "source": "test/codes/code_distance.jl:41-53",
            "H": [[0, 0, 0, 1, 1, 1, 1], [0, 1, 1, 0, 0, 1, 1], [1, 0, 1, 0, 1, 0, 1]],
            "shape": [4, 7],
        },
        "toric_2x3_stabilizers": {
            "source": "test/codes/codes.jl:5-22",
            "note": "Pauli(x-1) codes: 1=I, 2=X, 4=Z",
            "ops": [[2, 1, 2, 1, 1, 1, 2, 2, 1, 1, 1, 1], [1, 2, 1, 2, 1, 1, 2, 2, 1, 1, 1, 1],
                    [1, 1, 2, 1, 2, 1, 1, 1, 2, 2, 1, 1], [1, 1, 1, 2, 1, 2, 1, 1, 2, 2, 1, 1],
                    [2, 1, 1, 1, 2, 1, 1, 1, 1, 1, 2, 2], [4, 4, 1, 1, 1, 1, 4, 1, 1, 1, 4, 1],
                    [4, 4, 1, 1, 1, 1, 1, 4, 1, 1, 1, 4], [1, 1, 4, 4, 1, 1, 4, 1, 4, 1, 1, 1],
                    [1, 1, 4, 4, 1, 1, 1, 4, 1, 4, 1, 1], [1, 1, 1, 1, 4, 4, 1, 1, 4, 1, 4, 1]],
        },
        "surface3_decision_x1": {
            "source": "test/decoding/tndecoder.jl:60-73",
            "note": "X error on qubit 1, px=0.1 (py=pz=0): TNMMAP's pattern has no logical error vs X1",
            "error_x": [1, 0, 0, 0, 0, 0, 0, 0, 0],
            "px": 0.1,
            "logical_error": False,
        },
        "surface3_map_decision_flip": {
            "source": "test/decoding/tndecoder.jl:75-82",
            "note": "TNMAP (most probable error): with px[2]=px[3]=0.26 the decoded pattern differs "
                    "from X1 by a logical operator",
            "error_x": [1, 0, 0, 0, 0, 0, 0, 0, 0],
            "px": [0.1, 0.26, 0.26, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1],
            "logical_error": True,
        },
    }
    dem_path = None
    if ref_root:
        dem_path = os.path.join(ref_root, "test", "decoding", "test_circuits", "dem.dem")
    if dem_path and os.path.exists(dem_path):
        with open(dem_path) as f:
            dem_text = f.read()
    else:
        with open(OUT) as f:
            dem_text = json.load(f)["dem_small"]["text"]
    kat["dem_from_circuit"] = {
        "source": "test/decoding/dem.jl:5-86",
        "note": "detector_error_model(parse_stim_string(circuit)): mechanism rates (atol 1e-10) and the "
                "detectors (then logicals, numbered after the detectors) each flips; the reference lists "
                "them in dictionary order, so they compare as a set",
        "cases": [
            {"circuit": "X_ERROR(0.2) 0 1\nDEPOLARIZE1(0.03) 0 1\n\nCX 0 1\n\nM 0 1\nDETECTOR rec[-1]\n"
                        "DETECTOR rec[-2]\nDETECTOR rec[-1] rec[-2]\nOBSERVABLE_INCLUDE(0) rec[-1] rec[-2]\n",
             "n_qubits": 2, "error_rates": [0.212, 0.212], "flipped_detectors": [[1, 3, 4], [1, 2]],
             "source": "test/decoding/dem.jl:5-22"},
            {"circuit": "DEPOLARIZE1(0.3) 0\nM 0\nDETECTOR rec[-1]\n",
             "n_qubits": 1, "error_rates": [0.2], "flipped_detectors": [[1]],
             "source": "test/decoding/dem.jl:24-35"},
            {"circuit": "H 0\nCX 0 1\nDEPOLARIZE1(0.0297) 0\nH 3\nCX 0 2 1 2 3 0 3 1\nH 3\nM 2 3\n"
                        "DETECTOR rec[-2]\nDETECTOR rec[-1]\n",
             "n_qubits": 4, "error_rates": [0.01, 0.01, 0.01], "flipped_detectors": [[1], [1, 2], [2]],
             "source": "test/decoding/dem.jl:37-53"},
            {"circuit": "X_ERROR(0.2) 0 1\n\nCX 0 1\n\nM 0 1\nDETECTOR rec[-1] rec[-2]\n\nR 1\n\n"
                        "X_ERROR(0.2) 0 1\nCX 1 0\n\nM 0 1\nDETECTOR rec[-1] rec[-2]\n",
             "n_qubits": 2, "error_rates": [0.2, 0.32], "flipped_detectors": [[1], [2]],
             "source": "test/decoding/dem.jl:56-78"},
        ],
    }
    kat["stim_parse"] = {
        "source": "test/stim_parser/stim_parser.jl:5-48",
        "note": "the nested-REPEAT circuit parses (7 qubits); an unknown instruction is an error",
        "circuit": "CNOT 0 1 2 3 4 5 # A CNOT gate\nCNOT 2 1 4 3 6 5\nMR 1 3 5\n\nDETECTOR rec[-3]\n"
                   "DETECTOR rec[-2]\nDETECTOR rec[-1]\n\nREPEAT 2 {\n    CNOT 0 1 2 3 4 5 # A CNOT gate\n"
                   "    CNOT 2 1 4 3 6 5\n    MR 1 3 5\n\n    DETECTOR rec[-3] rec[-6]\n"
                   "    DETECTOR rec[-2] rec[-5]\n    DETECTOR rec[-1] rec[-4]\n    REPEAT 2 \n    {\n"
                   "    X 0 1 2 3 4 5 6\n    }\n}\n\nM(0.1) 0 2 4 6\n\nDETECTOR rec[-3] rec[-4] rec[-7]\n"
                   "DETECTOR rec[-2] rec[-3] rec[-6]\nDETECTOR rec[-1] rec[-2] rec[-5]\n\n"
                   "OBSERVABLE_INCLUDE(0) rec[-1]\n",
        "n_qubits": 7,
        "bad_circuit": "WRONG_INSTRUCTION 1\n",
    }
    kat["dem_small"] = {
        "source": "test/decoding/test_circuits/dem.dem (read by test/decoding/tndecoder.jl:112-121)",
        "text": dem_text,
    }
    with open(OUT, "w") as f:
        json.dump(kat, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
