"""GB300-native tensor-network decoder for TensorQEC.jl's TNMMAP path.

Host side of the drop-in: codes, Tanner graphs, logical operators, the
TNMMAP factor graph and its contraction order are built here; the contraction
itself runs in ``libtqec_gb300.so`` (hand-written sm_103a CUDA kernels behind
the C ABI of include/tqec_gb300.h).
"""
from .circuit import (Circuit, detector_error_model, insert_errors, memory_z_circuit, parse_stim_file,
                      parse_stim_string)
from .codes import (BivariateBicycleCode, Code422, Code832, Code1573, Color488, Color666, CSSTannerGraph,
                    PauliString, ShorCode, SimpleTannerGraph, SteaneCode, SurfaceCode, ToricCode,
                    remove_linear_dependency, stabilizers, tanner_graph)
from .decoder import (CompiledDEMTNMMAP, CompiledGeneralTNMAP, CompiledTNMAP, CompiledTNMMAP, FixedOrder,
                      GreedyMethod, NoOptimizer, TNMAP, TNMMAP, TreeSA, compile, decode, load_order,
                      multi_round_qec, optimize_code, save_order)
from .dem import DetectorErrorModel, dem2tanner, logical_map, parse_dem_file, parse_dem_string, sample_dem
from .error_model import (CSSErrorPattern, CSSSyndrome, DecodingResult, IndependentDepolarizingError,
                          IndependentFlipError, SimpleSyndrome, check_logical_error, depolarizing, iid_error,
                          pack_syndromes, random_error_pattern, syndrome_extraction, unpack_syndromes)
from .gf2 import logical_operator, null_space, row_echelon_form
from .network import (FactorGraph, parity_check_matrix, reduce2general, tnmap_graph, tnmmap_css_graph,
                      tnmmap_dem_graph)

__version__ = "0.1.0"
