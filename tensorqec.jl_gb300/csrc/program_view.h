// program_view.h -- read-only launch description of a program's float64
// contraction, for entry points that launch the kernel themselves.
#pragma once

#include <mutex>

#include "../../include/tqec_gb300.h"
#include "contract.cuh"

namespace tqec {

struct ProgramF64View {
  KArgs args;  // steps, tables, constants and sizes; no buffers
  int device;
  int sm_count;
  int threads;
  int group;
  std::mutex* mu;
};

int program_f64_view(tqec_program* p, ProgramF64View* v);

// What a multi-program launch needs of one program: its float32 and recheck
// launch descriptions (global tables, no buffers) and its sizes.
struct ProgramMultiView {
  KArgs args32, args_recheck;
  int recheck_precision;  // TQEC_F32X2 or TQEC_F64
  int device;
  int sm_count;
  int64_t arena_elems;
  int width;
  int n_steps;
  int syn_words;
  int syndrome_bytes;
  int n_classes;
  bool map_mode;
  double flops_per_syndrome;
  double recheck_margin;  // float32 log-margin below which a row is re-contracted
  // the recheck's cluster form (cluster_blocks 0: none): args_cluster is the
  // recheck launch description for it (tables and small pool as the shape
  // places them; no buffers), cluster_arena_elems the global arena elements
  // one cluster needs
  int cluster_blocks = 0, cluster_threads = 0, cluster_cap = 0;
  size_t cluster_smem = 0;
  int64_t cluster_arena_elems = 0;
  KArgs args_cluster;
};

int program_multi_view(tqec_program* p, ProgramMultiView* v);

}  // namespace tqec
