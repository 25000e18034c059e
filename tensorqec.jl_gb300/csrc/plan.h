// plan.h -- the contraction program a network + tree compiles into.
//
// A program is a list of runtime steps over one syndrome's "arena" (its
// working set).  Every step is a batched product with binary dimensions
//     C[h, fa, fb] = sum_k A[h, fa, k] * B[h, k, fb]
// where h are labels shared by both operands and still needed later, k are
// labels shared and summed here, fa / fb are labels of only one operand.
// Operand layouts are chosen top-down so that every operand is stored in
// exactly the order its consumer reads ([h][fa][k] for A, [h][k][fb] for B);
// a step writes its output through a bit-permutation table into the layout
// its own consumer wants.  Leaves that do not depend on the syndrome are
// folded on the host; leaves that depend on a few syndrome bits are kept as
// small lookup tables ("select" operands) or, for parity checks, evaluated
// from the index bits.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace tqec {

enum OperandKind : int32_t {
  OP_ARENA = 0,   // a runtime intermediate in the syndrome's arena
  OP_CONST = 1,   // constant data, optionally one of 2^m variants chosen by
                  // m syndrome bits (sel[])
  OP_PARITY = 2,  // 1 where popcount(index) has the parity of syndrome bit ref
};

constexpr int kMaxSel = 4;

// StepDesc::flags
constexpr int32_t kStepSync = 1;     // block barrier after this step (end of a barrier group)
constexpr int32_t kStepRotate4 = 2;  // permuted stores of 4-output items are lane-rotated
constexpr int32_t kStepRotate8 = 4;  // the same for 8-output items
constexpr int32_t kStepTensor = 8;   // GEMM-shaped step: B stored [h][fb][k] (K-major);
                                     // float32 blocks may run it on the tensor cores

struct StepDesc {
  int32_t a_kind, b_kind;
  int32_t a_ref, b_ref;      // arena offset | const offset | syndrome bit
  int32_t a_prod, b_prod;    // runtime step producing an arena operand, else -1
  int8_t a_sel[kMaxSel];     // syndrome bits choosing the const variant (-1: unused)
  int8_t b_sel[kMaxSel];
  int32_t lh, lfa, lfb, lk;  // log2 sizes of the index groups
  int32_t out_off;           // arena offset of the output
  int32_t perm_off;          // output permutation tables, -1 = identity
  int32_t flags;             // kStepSync | kStepRotate4 | kStepRotate8
  int32_t var_off;           // MAP mode: offset of the step's labels in Plan::vartab
};
static_assert(sizeof(StepDesc) == 64, "StepDesc is 64 bytes");

struct Plan {
  int32_t n_syndrome = 0;
  int32_t syndrome_bytes = 0;
  int32_t n_out = 0;
  int32_t n_classes = 1;
  int32_t n_tree_steps = 0;
  int32_t width = 0;               // log2 of the widest runtime intermediate
  int64_t arena_elems = 0;         // per syndrome
  int64_t arena_small = 0;         // elements of the small-tensor pool at the arena's start (0: one pool)
  int32_t tensor_steps = 0;        // steps marked kStepTensor
  int32_t root_step = -1;          // the last runtime step
  double macs_runtime = 0.0;       // multiply-adds per syndrome, runtime steps
  double macs_tree = 0.0;          // multiply-adds of the tree as given
  double err_terms = 0.0;          // sum over runtime steps of (K + 1) plus leaves
  // MAP mode (most probable configuration): every runtime step keeps its
  // output; vartab lists, per step, the variable ids of its fb, fa, h and k
  // index bits (lowest first); report lists the variables whose values are
  // returned; fixed holds values decided on the host (-1: from the search).
  bool map_mode = false;
  int32_t n_vars = 0;
  std::vector<int32_t> vartab;
  std::vector<int32_t> report;
  std::vector<int8_t> fixed;
  std::vector<StepDesc> steps;
  std::vector<int32_t> perm;       // concatenated permutation tables
  std::vector<double> consts;      // constant operand data (all variants)
};

struct NetworkView {
  int32_t n_tensors;
  const int32_t* ix_offsets;
  const int32_t* ix_labels;
  const int64_t* data_offsets;
  const double* data;
  int32_t n_out;
  const int32_t* out_labels;
  int32_t n_syndrome;
  const int32_t* syndrome_tensors;
};

struct PlanLimits {
  int max_sel_bits = 2;       // fold syndrome-dependent leaves up to this many bits
  int max_sel_rank = 8;       // ... and up to this many labels
  int max_width = 30;         // refuse intermediates wider than 2^max_width
  bool map_mode = false;      // max-product contraction + back-tracking (TNMAP)
  int64_t big_elems = 1024;   // intermediates above this size go to the big pool
  bool tensor_steps = true;   // mark GEMM-shaped steps (kStepTensor)
  // ... when they hold at least this share of the program's multiply-adds
  double tensor_min_share = 0.25;
  // run the runtime steps level by level (each after everything it reads,
  // the shallowest first), so independent chains of the tree share barrier
  // groups, and group wide steps too: fewer barriers for the single-syndrome
  // launches whose time is one syndrome's latency, more live intermediates
  bool level_order = false;
};

// A step is GEMM-shaped when, per h, it multiplies a 2^lfa x 2^lk block by a
// 2^lk x 2^lfb block with lfa >= 7 (one 128-row tile), lfb >= 5 (whole
// 32-column tensor-memory reads) and lk >= 5 (whole 32-element k chunks), and
// both operands are arena tensors or constant tables without syndrome
// selection.
constexpr int kTensorMinFa = 7, kTensorMinFb = 5, kTensorMinK = 5;

// Builds the program; returns "" on success or an error message.
// *unsupported is set when the network is valid but outside the kernels' scope.
std::string build_plan(const NetworkView& net, int32_t n_steps, const int32_t* steps,
                       const PlanLimits& lim, Plan* out, bool* unsupported);

}  // namespace tqec
