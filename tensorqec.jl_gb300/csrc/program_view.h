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

}  // namespace tqec
