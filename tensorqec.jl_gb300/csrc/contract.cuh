// contract.cuh -- launch interface of the batched tensor-network contraction.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "plan.h"

namespace tqec {

// Everything one launch of the contraction kernel needs.  Rows are syndromes;
// with `list` set, the kernel decodes rows list[0..*list_count) instead of
// rows row_offset .. row_offset + n.
struct KArgs {
  const StepDesc* steps;
  int32_t n_steps;
  const int32_t* perm;
  const void* consts;  // float or double, matching the kernel
  // tables staged in shared memory at kernel start: the constants (n_consts,
  // a multiple of 4) and the permutation tables (n_perm entries, a multiple
  // of 8), the latter from perm16 (uint16 entries) when it is set
  int32_t tables_smem;
  int32_t n_consts;
  int32_t n_perm;
  const uint16_t* perm16;
  const uint8_t* syn;
  int32_t syn_bytes;
  int32_t syn_words;  // 32-bit words per syndrome in shared memory (>= 1)
  int64_t n;
  int64_t row_offset;
  const int32_t* list;
  const int32_t* list_count;
  int32_t G, lg;  // syndromes per block and log2(G)
  int64_t arena_elems;
  void* arena_global;  // NULL: arena in shared memory
  // > 0: the first arena_small elements of each arena (the small tensors)
  // are in shared memory and the rest in arena_global
  int64_t arena_small;
  int32_t n_classes;
  int32_t* class_out;
  double* logp_out;
  float* err_out;
  float err_bound;
  double recheck_margin;  // < 0: never flag
  int32_t* recheck_list;
  int32_t* recheck_count;
  // most probable configuration (max-product contraction + back-tracking)
  int32_t map_mode;
  const int32_t* vartab;  // per step: variable ids of fb, fa, h, k bits
  int32_t n_vars;
  int32_t var_words;      // ceil(n_vars / 32)
  const int8_t* fixed;    // per variable: -1, or the value decided on the host
  const int32_t* report;  // variables whose values are returned
  int32_t n_report;
  uint8_t* assign_out;    // n x ceil(n_report / 8) bit-packed values
  // tensor-core steps: 1 when the block allocates tensor memory and runs
  // kStepTensor steps on tcgen05 (float32 only); tc_err is set when a wait
  // for the tensor cores gave up
  int32_t tc;
  int32_t vsplit;  // block launches: lanes may share four-output items (SK_VSPLIT)
  int32_t* tc_err;
  // per step, options the autotuner chose (kOpt*; nullptr: all 0), read
  // while the kernel plans its steps
  const int8_t* step_opts;
  // float32 launches: round every stored intermediate to bfloat16 (a study
  // of bf16 intermediates, TQEC_F32_BF16)
  int32_t round_bf16;
  int32_t opts_pad;
};
// step options: no shared work items; (cluster form) the step's barrier
// group never runs on the first block alone; runs there whenever its items
// fit, whatever the lanes' runs of k
constexpr int8_t kOptNoShare = 1;
constexpr int8_t kOptNoSolo = 2;
constexpr int8_t kOptSoloAlways = 4;
static_assert(sizeof(KArgs) % 16 == 0, "KArgs is copied in 16-byte units");

// Threads per block of the multi-program kernel (128 registers each).
constexpr int kMultiThreads = 512;

// A work unit of a multi-program launch: up to G rows of one program.
struct MultiUnit {
  int32_t prog;
  int32_t pad;
  int64_t first_row;
};

// One persistent launch over several programs (each a KArgs in device memory
// with its own syndromes and outputs).  Batch b owns units
// [unit_offsets[b], unit_offsets[b+1]); its rows of program i end at
// batch_rows[b * n_progs + i].  A program whose KArgs.arena_global is set
// uses the block's slice of arena_global (arena_per_block elements).
struct MultiArgs {
  const KArgs* progs;
  int32_t n_progs;
  int32_t list_mode;  // 1: each program contracts the rows of its list (recheck)
  const MultiUnit* units;
  const int64_t* unit_offsets;
  const int64_t* batch_rows;
  int32_t n_batches;   // a launch past the last batch does nothing
  int32_t* batch;      // device: the current batch
  int32_t* next_unit;  // device: units claimed in the current batch
  void* arena_global;
  int64_t arena_per_block;
};

// Shared memory a launch needs (bytes).
size_t contract_smem_bytes(int precision, int32_t n_steps, int32_t syn_words, int G,
                           int64_t arena_elems, bool arena_in_smem, int32_t var_words = 0,
                           size_t table_bytes = 0, bool tensor = false);

// Shared-memory bytes of the staged constant and permutation tables.
size_t contract_table_bytes(int precision, int64_t n_consts, int64_t n_perm, bool perm16);

// Largest dynamic shared memory a block may use on this device.
size_t contract_smem_limit(int device);

// Precisions: 0 float64, 1 float32 (normalised), 2 double-float (pairs of
// float32, normalised; the re-contraction of low-margin rows).
// Most threads a block of the given precision may have (blocks running
// tensor-core steps: 512).
constexpr int contract_max_threads(int precision, bool tensor = false) {
  return precision == 1 && !tensor ? 1024 : 512;
}

// Resident blocks per SM for a launch shape (0 if it cannot launch).
int contract_occupancy(int precision, int threads, size_t smem, bool map_mode = false, bool tensor = false);

cudaError_t contract_launch(int precision, const KArgs& a, int grid, int threads, size_t smem,
                            cudaStream_t stream);

// The cluster form (one syndrome per thread-block cluster of csize blocks,
// G = 1; arena in global memory, a.arena_global holding clusters *
// arena_elems elements, or with a.arena_small > 0 the small pool in the first
// block's shared memory and clusters * (arena_elems - arena_small) elements
// in a.arena_global): float64 (precision 0) and double-float (precision 2).  Returns
// the clusters that can be resident at once (0: the shape cannot launch).
// `configure` sets the kernel's shared-memory and cluster-size attributes
// first; a launch being captured into a CUDA graph passes false after an
// earlier contract_cluster_configure of the same shape.
int contract_cluster_capacity(int precision, int csize, int threads, size_t smem);
cudaError_t contract_cluster_launch(int precision, const KArgs& a, int clusters, int csize, int threads, size_t smem,
                                    cudaStream_t stream, bool configure = true);
cudaError_t contract_cluster_configure(int precision, int csize, int threads, size_t smem);

// The multi-program kernel (float32 normalised, or float64), and the
// per-batch advance (batch + 1, unit counter and recheck counts to zero).
cudaError_t contract_multi_launch(int precision, const MultiArgs& m, int grid, int threads, size_t smem,
                                  cudaStream_t stream);
int contract_multi_occupancy(int precision, int threads, size_t smem);
cudaError_t contract_multi_advance(int32_t* batch, int32_t* next_unit, int32_t* counts, int32_t n_progs,
                                   cudaStream_t stream);

}  // namespace tqec
