"""Writes circuit_d5_r7.json: oracle marginals of seeded detector samples of
the rotated Z-memory circuit d=5, 7 rounds, p=0.001 (width-25 contraction tree
orders/circuit_d5_r7.tree), the fixture of the sliced-contraction GPU test.

The oracle builds its own factor graph from the detector error model text
(oracle.tnmmap_oracle.dem_network, the restatement of tndecoder.jl:186-212),
checks that it equals the package's graph tensor for tensor, and contracts
each sample in float64 with the C oracle.  About a minute of CPU per sample
and thread.
Run:  python tests/golden/make_circuit_d5_r7.py [samples]
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "circuit_d5_r7.json")
SEED = 0x7E5A0007


def main(n=6):
    sys.path.insert(0, ROOT)
    import __graft_entry__ as G
    from oracle import tnmmap_oracle as oracle
    from oracle.c_oracle import CContractor, host_cores

    pkg = G.load_package()
    from tensorqec_gb300 import circuit as cz
    from tensorqec_gb300.dem import sample_dem, to_dem_string

    dm = cz.detector_error_model(cz.memory_z_circuit(5, 7, 0.001))
    g = pkg.tnmmap_dem_graph(pkg.dem2tanner(dm), pkg.logical_map(dm), dm.error_rates, len(dm.logical_list), True)
    net, _, _ = oracle.dem_network(oracle.parse_dem_string(to_dem_string(dm)), True)
    assert g.ixs == [list(x) for x in net.ixs] and list(g.iy) == list(net.iy)
    assert list(g.syndrome_positions) == list(net.syndrome_positions)
    assert all(np.array_equal(np.asarray(a).ravel(), np.asarray(b).flatten(order="F"))
               for a, b in zip(g.tensors, net.tensors))
    steps = pkg.load_order(os.path.join(ROOT, "tensorqec.jl_gb300", "orders", "circuit_d5_r7.tree"))
    _, det, _ = sample_dem(dm, n, np.random.default_rng(SEED))
    cc = CContractor(net.ixs, [np.asarray(t) for t in net.tensors], net.iy, net.syndrome_positions, steps)
    mar, cls = cc.contract(pkg.pack_syndromes(det), threads=host_cores())
    out = {"circuit": "memory_z_circuit(5, 7, 0.001)", "seed": SEED, "samples": n,
           "note": "detector bits from sample_dem(dm, samples, default_rng(seed)); marginals of the oracle's "
                   "float64 contraction (Julia linear class order)",
           "detectors": det.astype(int).tolist(), "marginals": mar.tolist(), "classes": cls.tolist()}
    with open(OUT, "w") as f:
        json.dump(out, f)
    print(OUT, mar.shape)


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 6)
