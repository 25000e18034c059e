// abi.cu -- the C ABI (include/tqec_gb300.h): program lifetime and decode
// orchestration.  The Julia side binds these with ccall in place of
// `decode(ct::CompiledTNMMAP, syndrome)` (src/decoding/tndecoder.jl:160-165)
// and `decode(ct::CompiledDEMTNMMAP, syndrome)` (:248-253).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/tqec_gb300.h"
#include "contract.cuh"
#include "plan.h"
#include "program_view.h"

namespace tqec {
std::string& last_error_ref() {
  thread_local std::string msg;
  return msg;
}
}  // namespace tqec

namespace {

#define g_last_error (tqec::last_error_ref())

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

#define TQ_CUDA(call)                                                                     \
  do {                                                                                    \
    cudaError_t e__ = (call);                                                             \
    if (e__ != cudaSuccess) {                                                             \
      return fail(e__ == cudaErrorMemoryAllocation ? TQEC_ERR_OOM : TQEC_ERR_CUDA,        \
                  std::string(#call) + ": " + cudaGetErrorString(e__));                   \
    }                                                                                     \
  } while (0)

struct Shape {
  int G = 1;
  int threads = 256;
  bool smem_arena = true;
  bool smem_tables = false;  // constants and permutation tables staged in shared memory
  bool split = false;        // small-tensor pool in shared memory, big-tensor pool in global memory
  bool tensor = false;       // GEMM-shaped steps on the tensor cores (float32 programs that have them)
  bool vsplit = false;       // lanes may share the four-output items of steps that leave threads idle
  size_t smem = 0;
  int grid_cap = 1;  // blocks resident on the whole device
};

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t want) {
    if (want <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) bytes = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

// The inputs a program was compiled from, kept for tqec_program_save: the
// network repacked densely (tensor i's labels and entries start at offsets
// i, the one-hot syndrome leaves stored as [1, 0], which the planner never
// reads), the tree and the options.
struct ProgramInputs {
  tqec_options opts;
  int32_t n_tensors = 0;
  std::vector<int32_t> ix_offsets, ix_labels, out_labels, syndrome_tensors, steps;
  std::vector<int64_t> data_offsets;
  std::vector<double> data;
};

}  // namespace

// The cluster form of a precision: `size` blocks of `threads` threads per
// syndrome, `cap` clusters resident at once, the tables staged in each
// block's shared memory when `tables`.
struct ClusterShape {
  int size = 0;
  int threads = 0;
  int cap = 0;
  size_t smem = 0;
  bool tables = false;
  bool split = false;  // the small pool in the first block's shared memory
};

struct tqec_program {
  tqec::Plan plan;
  int device = 0;
  int sm_count = 1;
  int precision = TQEC_F32;
  uint32_t flags = 0;
  double margin = -1.0;
  cudaStream_t stream = nullptr;
  tqec::StepDesc* d_steps = nullptr;
  int32_t* d_perm = nullptr;
  uint16_t* d_perm16 = nullptr;  // the same tables as uint16 (programs of width <= 16)
  int32_t* h_wait_err = nullptr;  // pinned, mapped: set by a bounded device wait that gave up
  int32_t* d_tc_err = nullptr;    // its device address
  int64_t n_perm_padded = 0;     // entries, a multiple of 8
  int32_t* d_vartab = nullptr;   // MAP mode tables
  int32_t* d_report = nullptr;
  int8_t* d_fixed = nullptr;
  double* d_c64 = nullptr;
  float* d_c32 = nullptr;
  float* d_cx2 = nullptr;  // the constants as double-float pairs (hi, lo)
  Shape shape[3];  // indexed by precision: the shape of large batches
  // shapes tuned for smaller batches: (rows they were tuned at, shape),
  // ascending; a launch takes the one nearest its row count (log scale)
  std::vector<std::pair<int64_t, Shape>> sized[3];
  // re-contraction of the few flagged rows (double-float, or float64):
  // latency matters, so one syndrome per block with the most threads and the
  // tables staged
  Shape recheck_shape;
  // single-syndrome launches (the plain form, the recheck) as one syndrome
  // per thread-block cluster, per precision (size 0: one block per syndrome)
  ClusterShape cluster[3];
  // per-step options of the cluster form found by tqec_program_autotune
  // (kOpt*, per precision; empty: none) and their device copies
  std::vector<int8_t> copts[3];
  DevBuf d_copts[3];
  DevBuf arena[3], carena[3];
  DevBuf syn, cls, logp, err, list, count;
  int32_t* h_count = nullptr;  // pinned
  // a wide float32 program's recheck twin: the same network compiled as a
  // plain program, its steps level by level (fewer barrier groups for one
  // syndrome's latency); the recheck runs on the twin's cluster form
  tqec_program* twin = nullptr;
  int64_t last_recheck = 0;
  // the last call's count is still being copied to h_count on its stream
  // (a call on a caller's stream with device outputs returns before it ends)
  bool recheck_async = false;
  ProgramInputs inputs;
  std::mutex mu;
};

namespace {

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Arithmetic of the recheck of low-margin float32 rows.
int recheck_precision(const tqec_program* p) {
  return (p->flags & TQEC_FLAG_RECHECK_F64) ? TQEC_F64 : TQEC_F32X2;
}

double err_bound(const tqec_program* p, int precision) {
  // per operation: float32 rounding, the double-float multiply-add's bound
  // (below 2^-44, taken as 2^-43), float64 rounding
  const double u = precision == TQEC_F32     ? std::ldexp(1.0, -24)
                   : precision == TQEC_F32X2 ? std::ldexp(1.0, -43)
                                             : std::ldexp(1.0, -53);
  const double b = u * p->plan.err_terms * 1.01;
  return b / (1.0 - std::min(b, 0.5));
}

int syn_words(const tqec_program* p) { return std::max(1, (p->plan.n_syndrome + 31) / 32); }

int var_words(const tqec_program* p) { return p->plan.map_mode ? (p->plan.n_vars + 31) / 32 : 0; }

size_t table_bytes(const tqec_program* p, int precision) {
  return tqec::contract_table_bytes(precision == TQEC_F32 ? 1 : 0, (int64_t)p->plan.consts.size(), p->n_perm_padded,
                                    p->d_perm16 != nullptr);
}

// Picks (G, threads) for one precision: the largest group whose arena fits
// about half of the shared memory (two blocks per SM), else a global arena.
// tables_req: 1 stages the constant and permutation tables in shared memory
// (unless that would push a one-syndrome arena out of it), 0 keeps them in
// global memory, -1 stages them only next to a shared-memory arena (a
// global-arena shape wants small blocks, many per SM).
bool tensor_program(const tqec_program* p, int precision) {
  return precision == TQEC_F32 && p->plan.tensor_steps > 0 && !p->plan.map_mode;
}

// Tensor-core shapes: at most 512 threads (at least 128: four warps read the
// 128 tensor-memory lanes) and at most four blocks per SM (128 of the 512
// tensor-memory columns each).
void finish_tensor_shape(const tqec_program* p, Shape* s) {
  s->grid_cap = std::min(s->grid_cap, 4 * p->sm_count);
}

int choose_shape(tqec_program* p, int precision, int G_req, int threads_req, int tables_req, Shape* out,
                 bool tensor_req = true) {
  const size_t limit = tqec::contract_smem_limit(p->device);
  const int64_t arena = p->plan.arena_elems;
  const int nsteps = (int)p->plan.steps.size();
  const int sw = syn_words(p);
  const int vw = var_words(p);
  const size_t tb_all = table_bytes(p, precision);
  const bool tensor = tensor_req && tensor_program(p, precision);
  auto bytes = [&](int G, bool arena_smem, size_t tb) {
    return tqec::contract_smem_bytes(precision, nsteps, sw, G, arena, arena_smem, vw, tb, tensor);
  };
  Shape s;
  s.threads = threads_req > 0 ? threads_req : 256;
  size_t tb = tb_all;
  if (G_req > 0) {
    s.G = G_req;
    s.smem_arena = bytes(s.G, true, tb) <= limit;
    if (!s.smem_arena && bytes(s.G, true, 0) <= limit) {
      tb = 0;
      s.smem_arena = true;
    }
  } else {
    const size_t target = limit / 2 - 1024;
    if (bytes(1, true, tb) > limit && bytes(1, true, 0) <= limit) tb = 0;
    int G = 1;
    while (G < 256 && bytes(G * 2, true, tb) <= target && (int64_t(G) * 2 << p->plan.width) <= 16 * 4096) G *= 2;
    s.G = G;
    s.smem_arena = bytes(G, true, tb) <= limit;
    // one syndrome per block with a wide arena: use more threads per block
    if (G == 1 && (!s.smem_arena || bytes(1, true, tb) > target))
      s.threads = threads_req > 0 ? threads_req : 1024;
  }
  s.threads = std::min(s.threads, tqec::contract_max_threads(precision, tensor));
  // the kernel's thread rotation needs a power-of-two block (at least a warp)
  while (s.threads & (s.threads - 1)) s.threads &= s.threads - 1;
  s.threads = std::max(s.threads, tensor ? 128 : 32);
  s.tensor = tensor;
  if (bytes(s.G, s.smem_arena, tb) > limit) tb = 0;
  if (tables_req == 0 || (tables_req < 0 && !s.smem_arena)) tb = 0;
  s.smem_tables = tb > 0;
  s.smem = bytes(s.G, s.smem_arena, tb);
  if (s.smem > limit) return fail(TQEC_ERR_UNSUPPORTED, "program does not fit shared memory even with a global arena");
  int occ = tqec::contract_occupancy(precision, s.threads, s.smem, p->plan.map_mode, tensor);
  if (occ < 1) return fail(TQEC_ERR_UNSUPPORTED, "launch shape cannot be resident on this device");
  s.grid_cap = occ * p->sm_count;
  if (tensor) finish_tensor_shape(p, &s);
  *out = s;
  return TQEC_OK;
}

// A split shape: G syndromes per block with their small-tensor pools in
// shared memory and their big-tensor pools in global memory (programs that
// have both pools).
int choose_split_shape(tqec_program* p, int precision, int G, int threads, int tables, Shape* out,
                       bool tensor_req = true) {
  if (p->plan.arena_small <= 0 || p->plan.map_mode) return fail(TQEC_ERR_UNSUPPORTED, "program has one pool");
  const size_t limit = tqec::contract_smem_limit(p->device);
  const int nsteps = (int)p->plan.steps.size();
  const bool tensor = tensor_req && tensor_program(p, precision);
  Shape s;
  s.G = G;
  s.threads = std::min(threads, tqec::contract_max_threads(precision, tensor));
  while (s.threads & (s.threads - 1)) s.threads &= s.threads - 1;
  s.threads = std::max(s.threads, tensor ? 128 : 32);
  s.smem_arena = false;
  s.split = true;
  s.tensor = tensor;
  const size_t tb = tables ? table_bytes(p, precision) : 0;
  s.smem_tables = tb > 0;
  s.smem = tqec::contract_smem_bytes(precision, nsteps, syn_words(p), G, p->plan.arena_small, true, 0, tb, tensor);
  if (s.smem > limit) return fail(TQEC_ERR_UNSUPPORTED, "program does not fit shared memory even with a global arena");
  int occ = tqec::contract_occupancy(precision, s.threads, s.smem, p->plan.map_mode, tensor);
  if (occ < 1) return fail(TQEC_ERR_UNSUPPORTED, "launch shape cannot be resident on this device");
  s.grid_cap = occ * p->sm_count;
  if (tensor) finish_tensor_shape(p, &s);
  *out = s;
  return TQEC_OK;
}

// The launch shape for a batch of n rows.
const Shape& pick_shape(const tqec_program* p, int precision, int64_t n) {
  const auto& v = p->sized[precision];
  for (size_t i = 0; i < v.size(); ++i) {
    // boundary: geometric mean of this size and the next larger one
    const double next = i + 1 < v.size() ? double(v[i + 1].first) : double(v[i].first) * 4.0;
    if (double(n) * double(n) <= double(v[i].first) * next) return v[i].second;
  }
  return p->shape[precision];
}

int ensure_arena(tqec_program* p, int precision, const Shape& s, int grid) {
  if (s.smem_arena) return TQEC_OK;
  const size_t esz = precision == TQEC_F32 ? 4 : 8;
  const int64_t per = s.split ? p->plan.arena_elems - p->plan.arena_small : p->plan.arena_elems;
  const size_t want = size_t(grid) * s.G * size_t(per) * esz;
  TQ_CUDA(p->arena[precision].ensure(want));
  return TQEC_OK;
}

tqec::KArgs base_args(tqec_program* p, int precision) {
  tqec::KArgs a;
  std::memset(&a, 0, sizeof(a));
  a.steps = p->d_steps;
  a.n_steps = (int32_t)p->plan.steps.size();
  a.perm = p->d_perm;
  a.consts = precision == TQEC_F32     ? (const void*)p->d_c32
             : precision == TQEC_F32X2 ? (const void*)p->d_cx2
                                       : (const void*)p->d_c64;
  a.syn_bytes = p->plan.syndrome_bytes;
  a.syn_words = syn_words(p);
  const Shape& s = p->shape[precision];
  a.tables_smem = s.smem_tables ? 1 : 0;
  a.n_consts = (int32_t)p->plan.consts.size();
  a.n_perm = (int32_t)p->n_perm_padded;
  a.perm16 = s.smem_tables ? p->d_perm16 : nullptr;
  a.G = s.G;
  a.lg = 0;
  while ((1 << a.lg) < s.G) a.lg++;
  a.arena_elems = p->plan.arena_elems;
  a.arena_global = s.smem_arena ? nullptr : p->arena[precision].p;
  a.n_classes = p->plan.n_classes;
  a.err_bound = (float)err_bound(p, precision);
  a.recheck_margin = -1.0;
  if (p->plan.map_mode) {
    a.map_mode = 1;
    a.vartab = p->d_vartab;
    a.n_vars = p->plan.n_vars;
    a.var_words = var_words(p);
    a.fixed = p->d_fixed;
    a.report = p->d_report;
    a.n_report = (int32_t)p->plan.report.size();
  }
  return a;
}

// Launches the batched kernel over up to n_rows_max rows with the shape
// tuned for that many rows (`forced`: that shape instead).
// Global-memory arenas of one launch stay within this many bytes: a wide
// program (a circuit-level tree of width 25 holds 62 million elements per
// syndrome) gets fewer blocks, which stride over the rows.
constexpr size_t kArenaBudget = size_t(16) << 30;

int launch_rows(tqec_program* p, int precision, tqec::KArgs a, int64_t n_rows_max, cudaStream_t st,
                const Shape* forced = nullptr) {
  const Shape& s = forced ? *forced : pick_shape(p, precision, n_rows_max);
  int64_t want = (n_rows_max + s.G - 1) / s.G;
  if (!s.smem_arena) {
    const int64_t per = s.split ? p->plan.arena_elems - p->plan.arena_small : p->plan.arena_elems;
    const size_t block_bytes = size_t(s.G) * size_t(std::max<int64_t>(per, 1)) * (precision == TQEC_F32 ? 4 : 8);
    want = std::min<int64_t>(want, std::max<int64_t>(1, int64_t(kArenaBudget / block_bytes)));
  }
  int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, s.grid_cap));
  int rc = ensure_arena(p, precision, s, grid);
  if (rc) return rc;
  a.G = s.G;
  a.lg = 0;
  while ((1 << a.lg) < s.G) a.lg++;
  a.tables_smem = s.smem_tables ? 1 : 0;
  a.perm16 = s.smem_tables ? p->d_perm16 : nullptr;
  a.arena_global = s.smem_arena ? nullptr : p->arena[precision].p;
  a.arena_small = s.split ? p->plan.arena_small : 0;
  a.tc = s.tensor ? 1 : 0;
  a.vsplit = s.vsplit ? 1 : 0;
  a.tc_err = p->d_tc_err;
  TQ_CUDA(tqec::contract_launch(precision, a, grid, s.threads, s.smem, st));
  return TQEC_OK;
}

// The cluster form of `precision` with csize blocks of `threads` threads
// (the tables staged when they fit); false if it cannot launch here.
// small_in_smem: 1 the small tensors in the first block's shared memory
// (read by the other blocks through distributed shared memory), 0 every
// intermediate in the cluster's slice of global memory, -1 the first when it
// fits.
bool choose_cluster(tqec_program* p, int precision, int csize, int threads, ClusterShape* out,
                    int small_in_smem = -1) {
  if (p->plan.map_mode || (precision != TQEC_F64 && precision != TQEC_F32X2) || csize < 2) return false;
  const size_t limit = tqec::contract_smem_limit(p->device);
  const int nsteps = (int)p->plan.steps.size();
  ClusterShape c;
  c.size = csize;
  c.threads = threads;
  const size_t tb = table_bytes(p, precision);
  // the small pool in shared memory when the program has one and it fits
  // with the tables, else beside global tables, else everything global
  const int sw = syn_words(p);
  const int64_t small = p->plan.arena_small;
  bool found = false;
  for (int split : {1, 0})
    for (int tables : {1, 0}) {
      if (found || (split && small <= 0) || (small_in_smem >= 0 && split != small_in_smem)) continue;
      const size_t b = tqec::contract_smem_bytes(precision, nsteps, sw, 1, split ? small : p->plan.arena_elems,
                                                 split != 0, 0, tables ? tb : 0);
      if (b > limit) continue;
      c.smem = b;
      c.tables = tables != 0;
      c.split = split != 0;
      found = true;
    }
  if (!found) return false;
  c.cap = tqec::contract_cluster_capacity(precision, csize, threads, c.smem);
  if (c.cap < 1) return false;
  *out = c;
  return true;
}

// One syndrome per cluster over up to n_rows_max rows (a.list / a.n), at
// most one wave of resident clusters striding over the rows.
int launch_cluster_rows(tqec_program* p, int precision, tqec::KArgs a, int64_t n_rows_max, cudaStream_t st) {
  const ClusterShape& c = p->cluster[precision];
  const int clusters = (int)std::max<int64_t>(1, std::min<int64_t>(n_rows_max, c.cap));
  const size_t esz = precision == TQEC_F32 ? 4 : 8;
  const int64_t per = c.split ? p->plan.arena_elems - p->plan.arena_small : p->plan.arena_elems;
  TQ_CUDA(p->carena[precision].ensure(size_t(clusters) * size_t(std::max<int64_t>(per, 1)) * esz));
  a.G = 1;
  a.lg = 0;
  a.tables_smem = c.tables ? 1 : 0;
  a.perm16 = c.tables ? p->d_perm16 : nullptr;
  a.arena_global = p->carena[precision].p;
  a.arena_small = c.split ? p->plan.arena_small : 0;
  a.tc = 0;
  a.step_opts = p->copts[precision].empty() ? nullptr : static_cast<const int8_t*>(p->d_copts[precision].p);
  TQ_CUDA(tqec::contract_cluster_launch(precision, a, clusters, c.size, c.threads, c.smem, st));
  return TQEC_OK;
}

// After a synchronisation: a bounded device wait that gave up (a tensor-core
// step waiting for its MMAs, or a block waiting for its table copies) makes
// the call fail (its results are not valid); the flag, in pinned host memory
// the device writes through its mapping, is cleared for the next call.
int check_tensor_error(tqec_program* p) {
  if (!p->h_wait_err) return TQEC_OK;
  const int32_t e = *static_cast<volatile int32_t*>(p->h_wait_err);
  if (e) {
    *static_cast<volatile int32_t*>(p->h_wait_err) = 0;
    return fail(TQEC_ERR_TIMEOUT, e == 2 ? "a block timed out waiting for its table copies"
                                         : "a tensor-core step timed out waiting for its MMAs");
  }
  return TQEC_OK;
}

// Runs the plain form: one launch (one block, one syndrome) per row, or the
// cluster form.
int launch_plain(tqec_program* p, int precision, tqec::KArgs a, int64_t n, cudaStream_t st) {
  // the cluster form: one launch, each syndrome on its own cluster
  if (p->cluster[precision].size > 0) return launch_cluster_rows(p, precision, a, n, st);
  Shape s = p->shape[precision];
  const size_t limit = tqec::contract_smem_limit(p->device);
  const int nsteps = (int)p->plan.steps.size();
  Shape one;
  one.G = 1;
  one.threads = s.threads;
  const size_t tb = table_bytes(p, precision);
  auto bytes = [&](bool arena_smem, size_t t) {
    return tqec::contract_smem_bytes(precision, nsteps, syn_words(p), 1, p->plan.arena_elems, arena_smem,
                                     var_words(p), t);
  };
  one.smem_arena = bytes(true, 0) <= limit;
  one.smem_tables = bytes(one.smem_arena, tb) <= limit;
  one.smem = bytes(one.smem_arena, one.smem_tables ? tb : 0);
  a.tables_smem = one.smem_tables ? 1 : 0;
  a.perm16 = one.smem_tables ? p->d_perm16 : nullptr;
  a.G = 1;
  a.lg = 0;
  if (!one.smem_arena) {
    const size_t esz = precision == TQEC_F32 ? 4 : 8;
    TQ_CUDA(p->arena[precision].ensure(size_t(p->plan.arena_elems) * esz));
    a.arena_global = p->arena[precision].p;
  } else {
    a.arena_global = nullptr;
  }
  a.n = 1;
  for (int64_t i = 0; i < n; ++i) {
    a.row_offset = i;
    TQ_CUDA(tqec::contract_launch(precision, a, 1, one.threads, one.smem, st));
  }
  return TQEC_OK;
}

// The re-contraction of the rows a float32 launch listed (b.list,
// b.list_count on the device; at most n_max of them).
// Programs at least this wide (log2 of the largest intermediate) run their
// single-syndrome launches on clusters by default: 16 blocks of 128 threads
// (at surface d=7 the fastest single-row form in float64 and double-float,
// about half the one-block latency), else 8 of 256.
constexpr int kClusterMinWidth = 12;

void default_clusters(tqec_program* p) {
  for (auto& c : p->cluster) c = ClusterShape{};
  if (p->plan.map_mode || p->plan.width < kClusterMinWidth) return;
  const bool plain = (p->flags & TQEC_FLAG_PLAIN) != 0;
  for (int prec : {recheck_precision(p), plain ? p->precision : -1}) {
    if (prec < 0) continue;
    ClusterShape c;
    if (choose_cluster(p, prec, 16, 128, &c) || choose_cluster(p, prec, 8, 256, &c)) p->cluster[prec] = c;
  }
  cudaGetLastError();
}

// The program whose cluster form contracts single rows of `precision`: the
// recheck twin for the recheck's arithmetic where the program has one.
tqec_program* cluster_program(tqec_program* p, int precision) {
  return p->twin && precision == recheck_precision(p) && p->twin->cluster[precision].size > 0 ? p->twin : p;
}

// Rows on clusters (cluster_program's form), `a` built for p.
int launch_cluster_rows_of(tqec_program* p, int precision, const tqec::KArgs& a, int64_t n_max, cudaStream_t st) {
  tqec_program* cp = cluster_program(p, precision);
  if (cp == p) return launch_cluster_rows(p, precision, a, n_max, st);
  // the twin's program (steps, tables, constants), these rows and outputs
  tqec::KArgs t = base_args(cp, precision);
  t.syn = a.syn;
  t.n = a.n;
  t.row_offset = a.row_offset;
  t.list = a.list;
  t.list_count = a.list_count;
  t.class_out = a.class_out;
  t.logp_out = a.logp_out;
  t.err_out = a.err_out;
  t.recheck_margin = a.recheck_margin;
  t.recheck_list = a.recheck_list;
  t.recheck_count = a.recheck_count;
  t.round_bf16 = a.round_bf16;
  t.tc_err = a.tc_err;  // a wait that gave up fails this program's call
  return launch_cluster_rows(cp, precision, t, n_max, st);
}

int launch_recheck(tqec_program* p, const tqec::KArgs& b, int64_t n_max, cudaStream_t st) {
  const int rp = recheck_precision(p);
  if (cluster_program(p, rp)->cluster[rp].size > 0) return launch_cluster_rows_of(p, rp, b, n_max, st);
  if (p->cluster[rp].size > 0) return launch_cluster_rows(p, rp, b, n_max, st);
  return launch_rows(p, rp, b, n_max, st, &p->recheck_shape);
}

struct Staged {
  const uint8_t* d_syn;
  int32_t* d_cls;
  double* d_logp;
  float* d_err;
  bool host_cls, host_logp, host_err;
};

int stage_inputs(tqec_program* p, const uint8_t* syn, int64_t n, int32_t* cls, double* logp, float* err,
                 cudaStream_t st, Staged* s) {
  const size_t sb = size_t(p->plan.syndrome_bytes) * size_t(n);
  if (sb > 0 && is_device_ptr(syn)) {
    s->d_syn = syn;
  } else {
    TQ_CUDA(p->syn.ensure(std::max<size_t>(sb, 16)));
    if (sb) TQ_CUDA(cudaMemcpyAsync(p->syn.p, syn, sb, cudaMemcpyHostToDevice, st));
    s->d_syn = (const uint8_t*)p->syn.p;
  }
  s->host_cls = cls && !is_device_ptr(cls);
  s->host_logp = logp && !is_device_ptr(logp);
  s->host_err = err && !is_device_ptr(err);
  if (s->host_cls) {
    TQ_CUDA(p->cls.ensure(sizeof(int32_t) * std::max<int64_t>(n, 1)));
    s->d_cls = (int32_t*)p->cls.p;
  } else {
    s->d_cls = cls;
  }
  if (s->host_logp) {
    TQ_CUDA(p->logp.ensure(sizeof(double) * std::max<int64_t>(n, 1) * p->plan.n_classes));
    s->d_logp = (double*)p->logp.p;
  } else {
    s->d_logp = logp;
  }
  if (s->host_err) {
    TQ_CUDA(p->err.ensure(sizeof(float) * std::max<int64_t>(n, 1)));
    s->d_err = (float*)p->err.p;
  } else {
    s->d_err = err;
  }
  return TQEC_OK;
}

int unstage_outputs(tqec_program* p, int64_t n, int32_t* cls, double* logp, float* err, cudaStream_t st,
                    const Staged& s) {
  if (s.host_cls && n) TQ_CUDA(cudaMemcpyAsync(cls, s.d_cls, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
  if (s.host_logp && n)
    TQ_CUDA(cudaMemcpyAsync(logp, s.d_logp, sizeof(double) * n * p->plan.n_classes, cudaMemcpyDeviceToHost, st));
  if (s.host_err && n) TQ_CUDA(cudaMemcpyAsync(err, s.d_err, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
  return TQEC_OK;
}

int decode_locked(tqec_program* p, const uint8_t* syn, int64_t n, int32_t* cls, double* logp, float* err,
                  int precision, bool recheck, bool plain, cudaStream_t st, bool round_bf16 = false) {
  Staged s;
  int rc = stage_inputs(p, syn, n, cls, logp, err, st, &s);
  if (rc) return rc;
  if (n > 0) {
    tqec::KArgs a = base_args(p, precision);
    a.syn = s.d_syn;
    a.n = n;
    a.class_out = s.d_cls;
    a.logp_out = s.d_logp;
    a.err_out = s.d_err;
    a.round_bf16 = round_bf16 ? 1 : 0;
    if (recheck && precision == TQEC_F32) {
      if (n > INT32_MAX) return fail(TQEC_ERR_INVALID, "batch above 2^31 rows");
      TQ_CUDA(p->list.ensure(sizeof(int32_t) * n));
      TQ_CUDA(p->count.ensure(sizeof(int32_t)));
      TQ_CUDA(cudaMemsetAsync(p->count.p, 0, sizeof(int32_t), st));
      a.recheck_margin = p->margin >= 0.0 ? p->margin : 2.0 * err_bound(p, TQEC_F32);
      a.recheck_list = (int32_t*)p->list.p;
      a.recheck_count = (int32_t*)p->count.p;
      // the float64 pass needs class/err outputs even if the caller did not ask
      if (!a.class_out) {
        TQ_CUDA(p->cls.ensure(sizeof(int32_t) * n));
        a.class_out = (int32_t*)p->cls.p;
      }
    }
    // a batch no larger than one wave of clusters takes the cluster form
    // of its precision (float64, double-float) where the program has one
    const ClusterShape& fc = cluster_program(p, precision)->cluster[precision];
    const bool few = precision != TQEC_F32 && fc.size > 0 && n <= fc.cap;
    rc = plain ? launch_plain(p, precision, a, n, st)
               : few ? launch_cluster_rows_of(p, precision, a, n, st) : launch_rows(p, precision, a, n, st);
    if (rc) return rc;
    if (recheck && precision == TQEC_F32) {
      tqec::KArgs b = base_args(p, recheck_precision(p));
      b.syn = s.d_syn;
      b.list = (const int32_t*)p->list.p;
      b.list_count = (const int32_t*)p->count.p;
      b.class_out = a.class_out;
      b.logp_out = s.d_logp;
      b.err_out = s.d_err;
      rc = launch_recheck(p, b, n, st);
      if (rc) return rc;
      TQ_CUDA(cudaMemcpyAsync(p->h_count, p->count.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    }
  }
  rc = unstage_outputs(p, n, cls, logp, err, st, s);
  if (rc) return rc;
  return TQEC_OK;
}

}  // namespace

namespace tqec {

int program_f64_view(tqec_program* p, ProgramF64View* v) {
  if (!p || !v) return TQEC_ERR_INVALID;
  v->args = base_args(p, TQEC_F64);
  v->args.arena_global = nullptr;
  // the view's launches size their own shared memory: tables stay global
  v->args.tables_smem = 0;
  v->args.perm16 = nullptr;
  v->device = p->device;
  v->sm_count = p->sm_count;
  v->threads = p->shape[TQEC_F64].threads;
  v->group = p->shape[TQEC_F64].G;
  v->mu = &p->mu;
  return TQEC_OK;
}

int program_multi_view(tqec_program* p, ProgramMultiView* v) {
  if (!p || !v) return TQEC_ERR_INVALID;
  v->recheck_precision = recheck_precision(p);
  for (int prec : {TQEC_F32, v->recheck_precision}) {
    KArgs a = base_args(p, prec);
    a.arena_global = nullptr;
    a.tables_smem = 0;
    a.perm16 = nullptr;
    (prec == TQEC_F32 ? v->args32 : v->args_recheck) = a;
  }
  v->device = p->device;
  v->sm_count = p->sm_count;
  v->arena_elems = p->plan.arena_elems;
  v->width = p->plan.width;
  v->n_steps = (int)p->plan.steps.size();
  v->syn_words = syn_words(p);
  v->syndrome_bytes = p->plan.syndrome_bytes;
  v->n_classes = p->plan.n_classes;
  v->map_mode = p->plan.map_mode;
  v->flops_per_syndrome = 2.0 * p->plan.macs_runtime;
  v->recheck_margin = p->margin >= 0.0 ? p->margin : 2.0 * err_bound(p, TQEC_F32);
  // the recheck's cluster form: the twin's where the program has one
  tqec_program* cp = p->twin ? p->twin : p;
  const ClusterShape& c = cp->cluster[v->recheck_precision];
  v->cluster_blocks = c.size;
  if (c.size > 0) {
    v->cluster_threads = c.threads;
    v->cluster_cap = c.cap;
    v->cluster_smem = c.smem;
    v->cluster_arena_elems = c.split ? cp->plan.arena_elems - cp->plan.arena_small : cp->plan.arena_elems;
    KArgs a = base_args(cp, v->recheck_precision);
    a.G = 1;
    a.lg = 0;
    a.tables_smem = c.tables ? 1 : 0;
    a.perm16 = c.tables ? cp->d_perm16 : nullptr;
    a.arena_global = nullptr;
    a.arena_small = c.split ? cp->plan.arena_small : 0;
    a.tc = 0;
    a.tc_err = p->d_tc_err;
    const auto& o = cp->copts[v->recheck_precision];
    a.step_opts = o.empty() ? nullptr : static_cast<const int8_t*>(cp->d_copts[v->recheck_precision].p);
    v->args_cluster = a;
  }
  return TQEC_OK;
}

}  // namespace tqec

namespace {

// The plan of a program.  A TQEC_FLAG_PLAIN program at least
// kClusterMinWidth wide decodes each syndrome on a thread-block cluster,
// whose time is one syndrome's latency: its steps run level by level
// (PlanLimits::level_order), so independent chains of the tree share barrier
// groups.
std::string plan_program(const tqec::NetworkView& v, const tqec_tree& tree, uint32_t flags, tqec::PlanLimits lim,
                         tqec::Plan* out, bool* unsupported) {
  std::string err = tqec::build_plan(v, tree.n_steps, tree.steps, lim, out, unsupported);
  if (!err.empty() || !(flags & TQEC_FLAG_PLAIN) || lim.map_mode || out->width < kClusterMinWidth) return err;
  lim.level_order = true;
  tqec::Plan lp;
  bool u2 = false;
  if (tqec::build_plan(v, tree.n_steps, tree.steps, lim, &lp, &u2).empty()) *out = std::move(lp);
  return err;
}

// Copies a network and tree that build_plan accepted (so every offset, size
// and position in them has been checked) into `in`.
void keep_inputs(const tqec_network& net, const tqec_tree& tree, const tqec_options& o, ProgramInputs* in) {
  const int T = net.n_tensors;
  in->opts = o;
  in->n_tensors = T;
  std::vector<char> leaf(T, 0);
  for (int j = 0; j < net.n_syndrome; ++j) leaf[net.syndrome_tensors[j]] = 1;
  in->ix_offsets.assign(1, 0);
  in->data_offsets.assign(1, 0);
  in->ix_labels.clear();
  in->data.clear();
  for (int i = 0; i < T; ++i) {
    in->ix_labels.insert(in->ix_labels.end(), net.ix_labels + net.ix_offsets[i], net.ix_labels + net.ix_offsets[i + 1]);
    in->ix_offsets.push_back((int32_t)in->ix_labels.size());
    if (leaf[i]) {
      in->data.push_back(1.0);
      in->data.push_back(0.0);
    } else {
      in->data.insert(in->data.end(), net.data + net.data_offsets[i], net.data + net.data_offsets[i + 1]);
    }
    in->data_offsets.push_back((int64_t)in->data.size());
  }
  in->out_labels.assign(net.out_labels, net.out_labels + std::max(net.n_out, 0));
  in->syndrome_tensors.assign(net.syndrome_tensors, net.syndrome_tensors + std::max(net.n_syndrome, 0));
  in->steps.assign(tree.steps, tree.steps + 2 * std::max(tree.n_steps, 0));
}

}  // namespace

extern "C" {

const char* tqec_version(void) { return "tqec-gb300 0.1.0 sm_103a"; }

int tqec_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return TQEC_ERR_INVALID;
  size_t n = std::min(len - 1, g_last_error.size());
  std::memcpy(buf, g_last_error.data(), n);
  buf[n] = '\0';
  return TQEC_OK;
}

int tqec_program_create(const tqec_network* net, const tqec_tree* tree, const tqec_options* opts,
                        tqec_program** out) {
  if (!net || !tree || !out) return fail(TQEC_ERR_INVALID, "NULL argument");
  *out = nullptr;
  tqec_options o;
  std::memset(&o, 0, sizeof(o));
  o.precision = TQEC_F32;
  o.margin = -1.0;
  if (opts) o = *opts;
  if (o.precision != TQEC_F32 && o.precision != TQEC_F64) return fail(TQEC_ERR_INVALID, "unknown precision");
  if (o.group < 0 || (o.group & (o.group - 1)) || o.group > 1024) return fail(TQEC_ERR_INVALID, "group must be 0 or a power of two <= 1024");
  if (o.threads < 0 || (o.threads % 32) || o.threads > 1024) return fail(TQEC_ERR_INVALID, "threads must be 0 or a multiple of 32 up to 1024");
  tqec::NetworkView v{net->n_tensors, net->ix_offsets, net->ix_labels, net->data_offsets, net->data,
                      net->n_out, net->out_labels, net->n_syndrome, net->syndrome_tensors};
  tqec::PlanLimits lim;
  lim.map_mode = (o.flags & TQEC_FLAG_MAP) != 0;
  lim.tensor_steps = (o.flags & TQEC_FLAG_NO_TENSOR_CORES) == 0;
  if (o.big_elems < 0) return fail(TQEC_ERR_INVALID, "big_elems must be >= 0");
  if (o.big_elems > 0) lim.big_elems = o.big_elems;
  auto* p = new tqec_program();
  bool unsupported = false;
  std::string err = plan_program(v, *tree, o.flags, lim, &p->plan, &unsupported);
  if (!err.empty()) {
    delete p;
    return fail(unsupported ? TQEC_ERR_UNSUPPORTED : TQEC_ERR_INVALID, err);
  }
  keep_inputs(*net, *tree, o, &p->inputs);
  p->device = o.device;
  p->precision = o.precision;
  p->flags = o.flags;
  p->margin = o.margin;
  auto bail = [&](int code, const std::string& m) {
    tqec_program_destroy(p);
    return fail(code, m);
  };
  cudaError_t e = cudaSetDevice(o.device);
  if (e != cudaSuccess) return bail(TQEC_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  cudaDeviceGetAttribute(&p->sm_count, cudaDevAttrMultiProcessorCount, o.device);
  if ((e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return bail(TQEC_ERR_CUDA, cudaGetErrorString(e));
  for (const tqec::StepDesc& d : p->plan.steps)
    if (d.a_kind == tqec::OP_PARITY || d.b_kind == tqec::OP_PARITY)
      return bail(TQEC_ERR_INVALID, "internal: the kernel reads no parity operands");
  const tqec::Plan& P = p->plan;
  size_t nst = P.steps.size();
  if ((e = cudaMalloc(&p->d_steps, nst * sizeof(tqec::StepDesc))) != cudaSuccess) return bail(TQEC_ERR_OOM, "steps");
  cudaMemcpy(p->d_steps, P.steps.data(), nst * sizeof(tqec::StepDesc), cudaMemcpyHostToDevice);
  {
    // both copies padded to a multiple of 8 entries (16-byte staging copies)
    std::vector<int32_t> perm(P.perm);
    while (perm.size() % 8) perm.push_back(0);
    p->n_perm_padded = (int64_t)perm.size();
    const size_t np = std::max<size_t>(perm.size(), 8);
    if ((e = cudaMalloc(&p->d_perm, np * sizeof(int32_t))) != cudaSuccess) return bail(TQEC_ERR_OOM, "perm");
    if (!perm.empty()) cudaMemcpy(p->d_perm, perm.data(), perm.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    bool fits16 = true;
    for (int32_t v : perm) fits16 = fits16 && v >= 0 && v < 65536;
    if (fits16) {
      std::vector<uint16_t> p16(perm.begin(), perm.end());
      if ((e = cudaMalloc(&p->d_perm16, np * sizeof(uint16_t))) != cudaSuccess) return bail(TQEC_ERR_OOM, "perm");
      if (!p16.empty()) cudaMemcpy(p->d_perm16, p16.data(), p16.size() * sizeof(uint16_t), cudaMemcpyHostToDevice);
    }
  }
  size_t nc = std::max<size_t>(P.consts.size(), 4);
  if ((e = cudaMalloc(&p->d_c64, nc * sizeof(double))) != cudaSuccess) return bail(TQEC_ERR_OOM, "consts");
  if ((e = cudaMalloc(&p->d_c32, nc * sizeof(float))) != cudaSuccess) return bail(TQEC_ERR_OOM, "consts");
  if ((e = cudaMalloc(&p->d_cx2, nc * 2 * sizeof(float))) != cudaSuccess) return bail(TQEC_ERR_OOM, "consts");
  if (!P.consts.empty()) {
    std::vector<float> c32(P.consts.begin(), P.consts.end());
    std::vector<float> cx2(2 * P.consts.size());
    for (size_t i = 0; i < P.consts.size(); ++i) {
      const float hi = float(P.consts[i]);
      cx2[2 * i] = hi;
      cx2[2 * i + 1] = float(P.consts[i] - double(hi));
    }
    cudaMemcpy(p->d_c64, P.consts.data(), P.consts.size() * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(p->d_c32, c32.data(), c32.size() * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(p->d_cx2, cx2.data(), cx2.size() * sizeof(float), cudaMemcpyHostToDevice);
  }
  if (P.map_mode) {
    const size_t nv = std::max<size_t>(P.vartab.size(), 1), nr = std::max<size_t>(P.report.size(), 1);
    if (cudaMalloc(&p->d_vartab, nv * 4) != cudaSuccess || cudaMalloc(&p->d_report, nr * 4) != cudaSuccess ||
        cudaMalloc(&p->d_fixed, std::max<size_t>(P.fixed.size(), 1)) != cudaSuccess)
      return bail(TQEC_ERR_OOM, "MAP tables");
    if (!P.vartab.empty()) cudaMemcpy(p->d_vartab, P.vartab.data(), P.vartab.size() * 4, cudaMemcpyHostToDevice);
    if (!P.report.empty()) cudaMemcpy(p->d_report, P.report.data(), P.report.size() * 4, cudaMemcpyHostToDevice);
    if (!P.fixed.empty()) cudaMemcpy(p->d_fixed, P.fixed.data(), P.fixed.size(), cudaMemcpyHostToDevice);
  }
  if ((e = cudaMallocHost(&p->h_count, sizeof(int32_t))) != cudaSuccess) return bail(TQEC_ERR_OOM, "pinned count");
  if ((e = cudaHostAlloc(&p->h_wait_err, sizeof(int32_t), cudaHostAllocMapped)) != cudaSuccess)
    return bail(TQEC_ERR_OOM, "error flag");
  *p->h_wait_err = 0;
  if ((e = cudaHostGetDevicePointer(&p->d_tc_err, p->h_wait_err, 0)) != cudaSuccess)
    return bail(TQEC_ERR_CUDA, "error flag mapping");
  *p->h_count = 0;
  if ((e = cudaGetLastError()) != cudaSuccess) return bail(TQEC_ERR_CUDA, cudaGetErrorString(e));
  int rc;
  for (int prec : {TQEC_F32, TQEC_F64, TQEC_F32X2}) {
    if (prec == TQEC_F32X2 && P.map_mode) continue;  // max-product runs in float32 or float64
    Shape sp;
    if ((o.flags & TQEC_FLAG_SPLIT_ARENA) && p->plan.arena_small > 0 &&
        choose_split_shape(p, prec, std::max(1, o.group), o.threads > 0 ? o.threads : 256, 0, &sp) == TQEC_OK) {
      p->shape[prec] = sp;
    } else if ((rc = choose_shape(p, prec, o.group, o.threads, -1, &p->shape[prec])) != TQEC_OK) {
      std::string m = g_last_error;
      return bail(rc, m);
    }
    Shape& sh = p->shape[prec];
    sh.vsplit = (o.flags & TQEC_FLAG_SHARED_ITEMS) && sh.G == 1 && !sh.tensor && !P.map_mode;
  }
  // the recheck keeps the small intermediates and the tables in shared
  // memory when the program has both pools and they fit
  const int rp = P.map_mode ? TQEC_F64 : recheck_precision(p);
  if (p->plan.arena_small <= 0 ||
      choose_split_shape(p, rp, 1, tqec::contract_max_threads(rp), 1, &p->recheck_shape) != TQEC_OK) {
    if ((rc = choose_shape(p, rp, 1, tqec::contract_max_threads(rp), 1, &p->recheck_shape)) != TQEC_OK) {
      std::string m = g_last_error;
      return bail(rc, m);
    }
  }
  // wide programs take their single-syndrome launches (the recheck; the
  // plain form) on 8-block clusters until tqec_program_autotune measures
  default_clusters(p);
  if (!(o.flags & (TQEC_FLAG_PLAIN | TQEC_FLAG_NORECHECK | TQEC_FLAG_MAP)) && o.precision == TQEC_F32 &&
      p->plan.width >= kClusterMinWidth) {
    tqec_options o2 = o;
    o2.flags |= TQEC_FLAG_PLAIN;
    tqec_program* tw = nullptr;
    if (tqec_program_create(net, tree, &o2, &tw) == TQEC_OK) {
      if (tw->cluster[recheck_precision(p)].size > 0) p->twin = tw;
      else tqec_program_destroy(tw);
    }
  }
  g_last_error.clear();
  *out = p;
  return TQEC_OK;
}

int tqec_program_destroy(tqec_program* p) {
  if (!p) return TQEC_OK;
  if (p->twin) tqec_program_destroy(p->twin);
  cudaSetDevice(p->device);
  if (p->stream) cudaStreamSynchronize(p->stream);
  cudaFree(p->d_steps);
  cudaFree(p->d_perm);
  cudaFree(p->d_perm16);
  if (p->h_wait_err) cudaFreeHost(p->h_wait_err);
  cudaFree(p->d_c64);
  cudaFree(p->d_c32);
  cudaFree(p->d_cx2);
  cudaFree(p->d_vartab);
  cudaFree(p->d_report);
  cudaFree(p->d_fixed);
  if (p->h_count) cudaFreeHost(p->h_count);
  for (auto* b : {&p->arena[0], &p->arena[1], &p->arena[2], &p->syn, &p->cls, &p->logp, &p->err, &p->list, &p->count}) b->release();
  if (p->stream) cudaStreamDestroy(p->stream);
  delete p;
  return TQEC_OK;
}

int tqec_program_info(const tqec_program* p, tqec_program_info_t* info) {
  if (!p || !info) return fail(TQEC_ERR_INVALID, "NULL argument");
  std::memset(info, 0, sizeof(*info));
  const tqec::Plan& P = p->plan;
  info->n_syndrome = P.n_syndrome;
  info->syndrome_bytes = P.syndrome_bytes;
  info->n_classes = P.n_classes;
  info->n_steps = (int32_t)P.steps.size();
  info->n_tree_steps = P.n_tree_steps;
  info->width = P.width;
  info->arena_elems = P.arena_elems;
  info->flops_per_syndrome = 2.0 * P.macs_runtime;
  info->flops_tree = 2.0 * P.macs_tree;
  info->err_bound_f32 = err_bound(p, TQEC_F32);
  info->err_bound_f64 = err_bound(p, TQEC_F64);
  info->group_f32 = p->shape[TQEC_F32].G;
  info->threads_f32 = p->shape[TQEC_F32].threads;
  info->smem_f32 = (int32_t)p->shape[TQEC_F32].smem;
  info->group_f64 = p->shape[TQEC_F64].G;
  info->threads_f64 = p->shape[TQEC_F64].threads;
  info->smem_f64 = (int32_t)p->shape[TQEC_F64].smem;
  info->resident_f32 = p->shape[TQEC_F32].grid_cap;
  info->resident_f64 = p->shape[TQEC_F64].grid_cap;
  info->tables_smem_f32 = p->shape[TQEC_F32].smem_tables ? 1 : 0;
  info->tables_smem_f64 = p->shape[TQEC_F64].smem_tables ? 1 : 0;
  info->arena_small = p->plan.arena_small;
  info->tensor_steps = p->plan.tensor_steps;
  info->tensor_f32 = p->shape[TQEC_F32].tensor ? 1 : 0;
  info->split_f32 = p->shape[TQEC_F32].split ? 1 : 0;
  info->split_f64 = p->shape[TQEC_F64].split ? 1 : 0;
  info->recheck_precision = P.map_mode ? TQEC_F64 : recheck_precision(p);
  // the form of single-syndrome launches: the plain form's, else the
  // recheck's (on the twin where the program has one)
  const tqec_program* cp = (p->flags & TQEC_FLAG_PLAIN) || !p->twin ? p : p->twin;
  info->cluster_blocks = cp->cluster[(p->flags & TQEC_FLAG_PLAIN) ? p->precision : info->recheck_precision].size;
  info->shared_items_f32 = p->shape[TQEC_F32].vsplit ? 1 : 0;
  info->shared_items_f64 = p->shape[TQEC_F64].vsplit ? 1 : 0;
  {
    const auto& o = cp->copts[(p->flags & TQEC_FLAG_PLAIN) ? p->precision : info->recheck_precision];
    info->cluster_tuned_steps = int32_t(std::count_if(o.begin(), o.end(), [](int8_t v) { return v != 0; }));
  }
  info->err_bound_f32x2 = err_bound(p, TQEC_F32X2);
  return TQEC_OK;
}

int tqec_decode_batch(tqec_program* p, const uint8_t* syndromes, int64_t n, int32_t* class_out, double* logp_out,
                      float* err_bound_out, void* stream) {
  if (!p || n < 0 || (n > 0 && !syndromes)) return fail(TQEC_ERR_INVALID, "bad argument");
  if (p->plan.map_mode) return fail(TQEC_ERR_INVALID, "a TQEC_FLAG_MAP program decodes with tqec_map_decode_batch");
  std::lock_guard<std::mutex> lk(p->mu);
  TQ_CUDA(cudaSetDevice(p->device));
  cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
  const bool plain = (p->flags & TQEC_FLAG_PLAIN) != 0;
  const bool recheck = p->precision == TQEC_F32 && !(p->flags & TQEC_FLAG_NORECHECK);
  int rc = decode_locked(p, syndromes, n, class_out, logp_out, err_bound_out, p->precision, recheck, plain, st);
  if (rc) return rc;
  if (!stream || (class_out && !is_device_ptr(class_out)) || (logp_out && !is_device_ptr(logp_out)) ||
      (err_bound_out && !is_device_ptr(err_bound_out))) {
    TQ_CUDA(cudaStreamSynchronize(st));
    p->last_recheck = recheck ? *p->h_count : 0;
    p->recheck_async = false;
    return check_tensor_error(p);
  }
  p->last_recheck = 0;
  p->recheck_async = recheck && n > 0;
  return TQEC_OK;
}

int tqec_decode_rows(tqec_program* p, const uint8_t* syndromes, const int32_t* rows, const int32_t* n_rows,
                     int64_t n_max, int64_t n_hint, int32_t* class_out, void* stream) {
  if (!p || n_max < 0 || (n_max > 0 && (!syndromes || !rows || !n_rows || !class_out)))
    return fail(TQEC_ERR_INVALID, "bad argument");
  if (p->plan.map_mode) return fail(TQEC_ERR_INVALID, "a TQEC_FLAG_MAP program decodes with tqec_map_decode_batch");
  if (n_max > INT32_MAX) return fail(TQEC_ERR_INVALID, "n_max above 2^31 rows");
  if ((p->flags & TQEC_FLAG_PLAIN) != 0) return fail(TQEC_ERR_UNSUPPORTED, "the plain form decodes with tqec_decode_batch");
  std::lock_guard<std::mutex> lk(p->mu);
  TQ_CUDA(cudaSetDevice(p->device));
  if (n_max == 0) return TQEC_OK;
  if (!is_device_ptr(syndromes) || !is_device_ptr(rows) || !is_device_ptr(n_rows) || !is_device_ptr(class_out))
    return fail(TQEC_ERR_INVALID, "tqec_decode_rows takes device pointers only");
  cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
  const bool recheck = p->precision == TQEC_F32 && !(p->flags & TQEC_FLAG_NORECHECK);
  tqec::KArgs a = base_args(p, p->precision);
  a.syn = syndromes;
  a.n = n_max;
  a.list = rows;
  a.list_count = n_rows;
  a.class_out = class_out;
  if (recheck) {
    TQ_CUDA(p->list.ensure(sizeof(int32_t) * n_max));
    TQ_CUDA(p->count.ensure(sizeof(int32_t)));
    TQ_CUDA(cudaMemsetAsync(p->count.p, 0, sizeof(int32_t), st));
    a.recheck_margin = p->margin >= 0.0 ? p->margin : 2.0 * err_bound(p, TQEC_F32);
    a.recheck_list = (int32_t*)p->list.p;
    a.recheck_count = (int32_t*)p->count.p;
  }
  // the shape tuned for about n_hint rows; the grid is at most one wave of
  // resident blocks, whose blocks stride over however many rows there are
  const Shape& s = pick_shape(p, p->precision, std::max<int64_t>(1, std::min(n_hint, n_max)));
  int rc = launch_rows(p, p->precision, a, n_max, st, &s);
  if (rc) return rc;
  if (recheck) {
    tqec::KArgs b = base_args(p, recheck_precision(p));
    b.syn = syndromes;
    b.list = (const int32_t*)p->list.p;
    b.list_count = (const int32_t*)p->count.p;
    b.n = n_max;
    b.class_out = class_out;
    if ((rc = launch_recheck(p, b, n_max, st))) return rc;
    TQ_CUDA(cudaMemcpyAsync(p->h_count, p->count.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  }
  p->last_recheck = 0;
  p->recheck_async = recheck;
  return TQEC_OK;
}

int tqec_contract_batch(tqec_program* p, const uint8_t* syndromes, int64_t n, int32_t precision, double* logp_out,
                        void* stream) {
  if (!p || n < 0 || (n > 0 && (!syndromes || !logp_out))) return fail(TQEC_ERR_INVALID, "bad argument");
  if (precision != TQEC_F32 && precision != TQEC_F64 && precision != TQEC_F32X2 && precision != TQEC_F32_BF16)
    return fail(TQEC_ERR_INVALID, "unknown precision");
  if (precision == TQEC_F32_BF16 && p->plan.map_mode)
    return fail(TQEC_ERR_INVALID, "a TQEC_FLAG_MAP program contracts in TQEC_F32 or TQEC_F64");
  // the bf16 study runs the float32 program with its stored intermediates rounded
  const bool bf16 = precision == TQEC_F32_BF16;
  if (bf16) precision = TQEC_F32;
  if (precision == TQEC_F32X2 && p->plan.map_mode)
    return fail(TQEC_ERR_INVALID, "a TQEC_FLAG_MAP program contracts in TQEC_F32 or TQEC_F64");
  std::lock_guard<std::mutex> lk(p->mu);
  TQ_CUDA(cudaSetDevice(p->device));
  cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
  const bool plain = (p->flags & TQEC_FLAG_PLAIN) != 0;
  int rc = decode_locked(p, syndromes, n, nullptr, logp_out, nullptr, precision, false, plain, st, bf16);
  if (rc) return rc;
  if (!stream || !is_device_ptr(logp_out)) {
    TQ_CUDA(cudaStreamSynchronize(st));
    return check_tensor_error(p);
  }
  return TQEC_OK;
}

int tqec_map_decode_batch(tqec_program* p, const uint8_t* syndromes, int64_t n, uint8_t* assignment_out,
                          double* logp_out, void* stream) {
  if (!p || n < 0 || (n > 0 && (!syndromes || !assignment_out))) return fail(TQEC_ERR_INVALID, "bad argument");
  if (!p->plan.map_mode) return fail(TQEC_ERR_INVALID, "program was not created with TQEC_FLAG_MAP");
  std::lock_guard<std::mutex> lk(p->mu);
  TQ_CUDA(cudaSetDevice(p->device));
  cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
  Staged s;
  int rc = stage_inputs(p, syndromes, n, nullptr, logp_out, nullptr, st, &s);
  if (rc) return rc;
  const size_t rb = (p->plan.report.size() + 7) / 8;
  const bool host_asg = !is_device_ptr(assignment_out);
  uint8_t* d_asg = assignment_out;
  if (host_asg) {
    TQ_CUDA(p->err.ensure(std::max<size_t>(rb * size_t(n), 16)));
    d_asg = static_cast<uint8_t*>(p->err.p);
  }
  if (n > 0) {
    tqec::KArgs a = base_args(p, p->precision);
    a.syn = s.d_syn;
    a.n = n;
    a.logp_out = s.d_logp;
    a.assign_out = d_asg;
    const bool plain = (p->flags & TQEC_FLAG_PLAIN) != 0;
    rc = plain ? launch_plain(p, p->precision, a, n, st) : launch_rows(p, p->precision, a, n, st);
    if (rc) return rc;
    if (host_asg) TQ_CUDA(cudaMemcpyAsync(assignment_out, d_asg, rb * size_t(n), cudaMemcpyDeviceToHost, st));
    if (s.host_logp) TQ_CUDA(cudaMemcpyAsync(logp_out, s.d_logp, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  }
  if (!stream || host_asg || s.host_logp) TQ_CUDA(cudaStreamSynchronize(st));
  return TQEC_OK;
}

int tqec_last_recheck_count(const tqec_program* p, int64_t* count) {
  if (!p || !count) return fail(TQEC_ERR_INVALID, "NULL argument");
  // after an asynchronous call the count is in the pinned word once the
  // caller's stream has passed the call (the caller synchronises first)
  *count = p->recheck_async ? int64_t(*p->h_count) : p->last_recheck;
  return TQEC_OK;
}

namespace {

// The fastest launch shape for batches of n rows (the probe syndromes are
// already on the device).  Returns false if a launch failed.
bool tune_shape(tqec_program* p, int prec, int64_t n, cudaEvent_t e0, cudaEvent_t e1, Shape* out) {
  Shape best = p->shape[prec];
  float best_ms = 1e30f;
  for (int G : {1, 2, 4, 8, 16, 32, 64, 128}) {
    if (G > 1 && G > n) break;
    for (int th : {128, 256, 512, 1024}) {
      if (th > tqec::contract_max_threads(prec)) continue;
      for (int tables : {0, 1}) {
        // global-arena shapes also try fewer resident blocks per SM, so that
        // the arenas in flight can stay in L2
        for (int resident : {0, 8, 4, 2, 1}) {
         for (int split : {0, 1}) {
          // programs with GEMM-shaped steps also try them on the SIMT path
          for (int tensor : {1, 0}) {
          if (!tensor && !tensor_program(p, prec)) continue;
          // one syndrome per block: also with lanes sharing the items of
          // steps that would leave threads idle
          for (int vs : {0, 1}) {
          if (vs && (G > 1 || tensor || p->plan.map_mode)) continue;
          Shape s;
          if (split) {
            if (choose_split_shape(p, prec, G, th, tables, &s, tensor) != TQEC_OK) continue;
          } else if (choose_shape(p, prec, G, th, tables, &s, tensor) != TQEC_OK) {
            continue;
          }
          if (tables && !s.smem_tables) continue;
          s.vsplit = vs != 0;
          if (resident) {
            if (s.smem_arena || tables || resident * p->sm_count >= s.grid_cap) continue;
            s.grid_cap = resident * p->sm_count;
          }
          // a global arena bigger than 4 GB is not worth probing on a shared GPU
          const size_t esz = prec == TQEC_F32 ? 4 : 8;
          if (!s.smem_arena &&
              (G > 8 || size_t(s.grid_cap) * G * size_t(p->plan.arena_elems) * esz > (size_t(4) << 30)))
            continue;
          tqec::KArgs a = base_args(p, prec);
          a.syn = (const uint8_t*)p->syn.p;
          a.n = n;
          a.logp_out = (double*)p->logp.p;
          if (launch_rows(p, prec, a, n, p->stream, &s) != TQEC_OK) continue;  // warm-up
          cudaEventRecord(e0, p->stream);
          launch_rows(p, prec, a, n, p->stream, &s);
          cudaEventRecord(e1, p->stream);
          if (cudaEventSynchronize(e1) != cudaSuccess) return false;
          float ms = 0.f;
          cudaEventElapsedTime(&ms, e0, e1);
          if (ms < best_ms) {
            best_ms = ms;
            best = s;
          }
          }
          }
         }
        }
      }
    }
  }
  *out = best;
  return true;
}

}  // namespace

namespace {

// The cluster form's plan, barrier group by barrier group: whether the group
// runs on the first block alone (never; whenever its items fit) and whether
// its steps share work items, each kept when it shortens the single-row
// latency by more than 1 % (the fastest of five calls per setting).
bool tune_cluster_steps(tqec_program* p, int prec, bool plain, cudaEvent_t e0, cudaEvent_t e1) {
  const int n = (int)p->plan.steps.size();
  std::vector<int8_t>& o = p->copts[prec];
  o.assign(n, 0);
  auto time_row = [&](float* ms_out) {
    if (p->d_copts[prec].ensure(size_t(n)) != cudaSuccess) return false;
    if (cudaMemcpy(p->d_copts[prec].p, o.data(), size_t(n), cudaMemcpyHostToDevice) != cudaSuccess) return false;
    tqec::KArgs a = base_args(p, prec);
    a.syn = (const uint8_t*)p->syn.p;
    a.n = 1;
    a.logp_out = (double*)p->logp.p;
    auto run = [&]() { return plain ? launch_plain(p, prec, a, 1, p->stream) : launch_cluster_rows(p, prec, a, 1, p->stream); };
    if (run() != TQEC_OK) return false;
    float best = 1e30f;
    for (int r = 0; r < 5; ++r) {
      cudaEventRecord(e0, p->stream);
      if (run() != TQEC_OK) return false;
      cudaEventRecord(e1, p->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) return false;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      best = std::min(best, ms);
    }
    *ms_out = best;
    return true;
  };
  float cur = 0.f;
  if (!time_row(&cur)) return false;
  if (cur > 2.f) {  // a row of milliseconds: per-group tuning would take minutes; keep the plan as is
    o.clear();
    return true;
  }
  for (int s0 = 0; s0 < n;) {
    int s1 = s0;
    while (s1 + 1 < n && !(p->plan.steps[s1].flags & tqec::kStepSync)) ++s1;
    for (int8_t bit : {tqec::kOptNoSolo, tqec::kOptSoloAlways, tqec::kOptNoShare}) {
      for (int s = s0; s <= s1; ++s) o[s] ^= bit;
      float t = 0.f;
      if (!time_row(&t)) return false;
      if (t < 0.99f * cur) {
        cur = t;
      } else {
        for (int s = s0; s <= s1; ++s) o[s] ^= bit;
      }
    }
    s0 = s1 + 1;
  }
  // keep the device copy in step with the options kept
  if (cudaMemcpy(p->d_copts[prec].p, o.data(), size_t(n), cudaMemcpyHostToDevice) != cudaSuccess) return false;
  if (std::all_of(o.begin(), o.end(), [](int8_t v) { return v == 0; })) o.clear();
  return true;
}

// Single-syndrome launches of one precision: the block form (the recheck
// shape, or one launch per row in the plain form) against clusters of 2-16
// blocks of 128, 256 or 512 threads, timed on one row (the plain form: the
// drop-in decodes one syndrome a call) or on one and on four rows (the
// recheck: a few rows a batch; the sum decides).
bool tune_cluster(tqec_program* p, int prec, bool plain, cudaEvent_t e0, cudaEvent_t e1) {
  // the largest clusters first and the block form last: a program so wide
  // that one row takes milliseconds stops trying shapes once the tuning has
  // spent about two seconds of GPU time, keeping the best so far
  std::vector<ClusterShape> cands;
  for (int cs : {16, 8, 4, 2})
    for (int th : {128, 256, 512})
      for (int split : {1, 0}) {
        ClusterShape c;
        if (choose_cluster(p, prec, cs, th, &c, split)) cands.push_back(c);
      }
  cands.push_back(ClusterShape{});  // the block form
  cudaGetLastError();
  ClusterShape best;
  float best_ms = 1e30f, spent_ms = 0.f;
  for (const ClusterShape& c : cands) {
    if (spent_ms > 2000.f && best_ms < 1e30f) break;
    p->cluster[prec] = c;
    float total = 0.f;
    bool ok = true;
    for (int64_t rows : {int64_t(1), int64_t(plain ? 0 : 4)}) {
      if (rows == 0) continue;
      tqec::KArgs a = base_args(p, prec);
      a.syn = (const uint8_t*)p->syn.p;
      a.n = rows;
      a.logp_out = (double*)p->logp.p;
      auto run = [&]() {
        if (plain) return launch_plain(p, prec, a, rows, p->stream);
        if (c.size > 0) return launch_cluster_rows(p, prec, a, rows, p->stream);
        return launch_rows(p, prec, a, rows, p->stream, &p->recheck_shape);
      };
      if (run() != TQEC_OK) {  // warm-up
        ok = false;
        break;
      }
      cudaEventRecord(e0, p->stream);
      for (int r = 0; r < 3; ++r) run();
      cudaEventRecord(e1, p->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) return false;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      total += ms;
      spent_ms += ms * 4.f / 3.f;  // the warm-up call and the three timed ones
    }
    if (ok && total < best_ms) {
      best_ms = total;
      best = c;
    }
    cudaGetLastError();
  }
  p->cluster[prec] = best;
  p->copts[prec].clear();
  if (best.size > 0) return tune_cluster_steps(p, prec, plain, e0, e1);
  return true;
}

}  // namespace

int tqec_program_trim(tqec_program* p) {
  if (!p) return fail(TQEC_ERR_INVALID, "NULL program");
  std::lock_guard<std::mutex> lk(p->mu);
  TQ_CUDA(cudaSetDevice(p->device));
  TQ_CUDA(cudaStreamSynchronize(p->stream));
  for (int i = 0; i < 3; ++i) {
    p->arena[i].release();
    p->carena[i].release();
  }
  return TQEC_OK;
}

int tqec_program_set_cluster(tqec_program* p, int32_t precision, int32_t blocks, int32_t threads,
                             int32_t small_in_smem) {
  if (!p) return fail(TQEC_ERR_INVALID, "NULL program");
  if (precision != TQEC_F64 && precision != TQEC_F32X2)
    return fail(TQEC_ERR_INVALID, "clusters serve TQEC_F64 and TQEC_F32X2 launches");
  if (p->twin && precision == recheck_precision(p)) {
    // the recheck runs on the twin's cluster form
    const int rc = tqec_program_set_cluster(p->twin, precision, blocks, threads, small_in_smem);
    if (rc) return rc;
  }
  std::lock_guard<std::mutex> lk(p->mu);
  TQ_CUDA(cudaSetDevice(p->device));
  p->copts[precision].clear();  // tuned for the previous form
  if (blocks == 0) {
    p->cluster[precision] = ClusterShape{};
    return TQEC_OK;
  }
  if (blocks < 2 || blocks > 16 || (blocks & (blocks - 1)) || threads < 32 || threads > 512 ||
      (threads & (threads - 1)) || small_in_smem < -1 || small_in_smem > 1)
    return fail(TQEC_ERR_INVALID,
                "blocks must be 0 or 2, 4, 8, 16; threads a power of two from 32 to 512; small_in_smem -1, 0 or 1");
  ClusterShape c;
  if (!choose_cluster(p, precision, blocks, threads, &c, small_in_smem)) {
    cudaGetLastError();
    return fail(TQEC_ERR_UNSUPPORTED, "this cluster shape cannot launch for this program on this device");
  }
  p->cluster[precision] = c;
  return TQEC_OK;
}

int tqec_program_autotune(tqec_program* p, int64_t n_probe) {
  if (!p || n_probe <= 0) return fail(TQEC_ERR_INVALID, "bad argument");
  std::lock_guard<std::mutex> lk(p->mu);
  TQ_CUDA(cudaSetDevice(p->device));
  const int64_t n = n_probe;
  std::vector<uint8_t> h((size_t)n * p->plan.syndrome_bytes);
  uint64_t x = 0x9E3779B97F4A7C15ull;
  for (auto& b : h) {
    x ^= x << 13; x ^= x >> 7; x ^= x << 17;
    b = uint8_t(x & 0x11);  // sparse bits, like low-noise syndromes
  }
  TQ_CUDA(p->syn.ensure(std::max<size_t>(h.size(), 16)));
  TQ_CUDA(cudaMemcpy(p->syn.p, h.data(), h.size(), cudaMemcpyHostToDevice));
  TQ_CUDA(p->logp.ensure(sizeof(double) * n * p->plan.n_classes));
  cudaEvent_t e0, e1;
  TQ_CUDA(cudaEventCreate(&e0));
  TQ_CUDA(cudaEventCreate(&e1));
  bool ok = true;
  for (int prec : {TQEC_F32, TQEC_F64}) {
    // large batches at n rows; smaller batches (down to 1/64 of it, at
    // least 256 rows) get shapes of their own
    Shape big;
    ok = ok && tune_shape(p, prec, n, e0, e1, &big);
    std::vector<std::pair<int64_t, Shape>> sized;
    for (int64_t m = n / 4; ok && m >= 256 && m >= n / 64; m /= 4) {
      Shape sm;
      ok = ok && tune_shape(p, prec, m, e0, e1, &sm);
      sized.insert(sized.begin(), {m, sm});
    }
    if (!ok) break;
    p->shape[prec] = big;
    p->sized[prec] = sized;
  }
  // single-syndrome launches: the recheck's arithmetic, and the plain form
  if (ok && !p->plan.map_mode) {
    const bool plain = (p->flags & TQEC_FLAG_PLAIN) != 0;
    ok = tune_cluster(p, recheck_precision(p), false, e0, e1);
    if (ok && plain && p->precision != TQEC_F32) ok = tune_cluster(p, p->precision, true, e0, e1);
    if (ok && p->twin) {
      // the recheck runs on the twin's cluster form: tune that one on the same probes
      tqec_program* tw = p->twin;
      const size_t sb = size_t(n) * p->plan.syndrome_bytes;
      ok = tw->syn.ensure(std::max<size_t>(sb, 16)) == cudaSuccess &&
           cudaMemcpy(tw->syn.p, p->syn.p, sb, cudaMemcpyDeviceToDevice) == cudaSuccess &&
           tw->logp.ensure(sizeof(double) * n * p->plan.n_classes) == cudaSuccess &&
           tune_cluster(tw, recheck_precision(p), false, e0, e1);
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!ok) return fail(TQEC_ERR_CUDA, "autotune launch failed");
  const int te = check_tensor_error(p);
  if (te) return te;
  g_last_error.clear();
  return TQEC_OK;
}

int tqec_plan_inspect(const tqec_network* net, const tqec_tree* tree, tqec_plan_view* view, void** handle) {
  return tqec_plan_inspect_flags(net, tree, 0u, view, handle);
}

int tqec_plan_inspect_flags(const tqec_network* net, const tqec_tree* tree, uint32_t flags, tqec_plan_view* view,
                            void** handle) {
  if (!net || !tree || !view || !handle) return fail(TQEC_ERR_INVALID, "NULL argument");
  *handle = nullptr;
  tqec::NetworkView v{net->n_tensors, net->ix_offsets, net->ix_labels, net->data_offsets, net->data,
                      net->n_out, net->out_labels, net->n_syndrome, net->syndrome_tensors};
  auto* P = new tqec::Plan();
  bool unsupported = false;
  tqec::PlanLimits lim;
  lim.map_mode = (flags & TQEC_FLAG_MAP) != 0;
  lim.tensor_steps = (flags & TQEC_FLAG_NO_TENSOR_CORES) == 0;
  std::string err = plan_program(v, *tree, flags, lim, P, &unsupported);
  if (!err.empty()) {
    delete P;
    return fail(unsupported ? TQEC_ERR_UNSUPPORTED : TQEC_ERR_INVALID, err);
  }
  std::memset(view, 0, sizeof(*view));
  view->n_steps = (int32_t)P->steps.size();
  view->steps = P->steps.data();
  view->n_perm = (int64_t)P->perm.size();
  view->perm = P->perm.data();
  view->n_consts = (int64_t)P->consts.size();
  view->consts = P->consts.data();
  view->arena_elems = P->arena_elems;
  view->width = P->width;
  view->n_classes = P->n_classes;
  view->n_syndrome = P->n_syndrome;
  view->flops_per_syndrome = 2.0 * P->macs_runtime;
  view->flops_tree = 2.0 * P->macs_tree;
  view->err_terms = P->err_terms;
  view->map_mode = P->map_mode ? 1 : 0;
  view->n_vars = P->n_vars;
  view->n_vartab = (int64_t)P->vartab.size();
  view->vartab = P->vartab.data();
  view->n_report = (int32_t)P->report.size();
  view->report = P->report.data();
  view->fixed = P->fixed.data();
  *handle = P;
  return TQEC_OK;
}

int tqec_plan_release(void* handle) {
  delete static_cast<tqec::Plan*>(handle);
  return TQEC_OK;
}

}  // extern "C"

// ---- program files -------------------------------------------------------
// A program file holds what a program was compiled from (network, tree,
// options) and the launch shapes chosen for it (by tqec_program_autotune or
// at creation), so a process can skip the order search and the autotuning
// that produced them.  Loading compiles the network again with the stored
// tree, requires the same program as when it was saved (a fingerprint of the
// step records and tables) and takes the stored shapes when the device has
// the same SM count and shared-memory limit and each shape is consistent with
// the program.  Layout: "TQECPROG", version, byte-order mark, the fields in
// the order written below (arrays as a uint64 count and the elements), and a
// 64-bit FNV-1a checksum of everything before it.

namespace {

constexpr char kFileMagic[8] = {'T', 'Q', 'E', 'C', 'P', 'R', 'O', 'G'};
constexpr uint32_t kFileVersion = 1;
constexpr uint32_t kByteOrderMark = 0x01020304u;
constexpr size_t kMaxFileBytes = size_t(1) << 31;

uint64_t fnv1a(const void* data, size_t n, uint64_t h = 0xcbf29ce484222325ull) {
  const unsigned char* b = static_cast<const unsigned char*>(data);
  for (size_t i = 0; i < n; ++i) {
    h ^= b[i];
    h *= 0x100000001b3ull;
  }
  return h;
}

// Identifies a compiled program: its step records, tables and sizes.
uint64_t plan_fingerprint(const tqec::Plan& P) {
  uint64_t h = fnv1a(P.steps.data(), P.steps.size() * sizeof(tqec::StepDesc));
  h = fnv1a(P.perm.data(), P.perm.size() * sizeof(int32_t), h);
  h = fnv1a(P.consts.data(), P.consts.size() * sizeof(double), h);
  h = fnv1a(P.vartab.data(), P.vartab.size() * sizeof(int32_t), h);
  const int64_t sizes[] = {P.arena_elems, P.arena_small, P.n_classes, P.n_syndrome, P.width, P.map_mode ? 1 : 0};
  return fnv1a(sizes, sizeof(sizes), h);
}

struct Writer {
  std::string buf;
  template <class T>
  void put(const T& v) {
    buf.append(reinterpret_cast<const char*>(&v), sizeof(T));
  }
  template <class T>
  void put_vec(const std::vector<T>& v) {
    put<uint64_t>(v.size());
    if (!v.empty()) buf.append(reinterpret_cast<const char*>(v.data()), v.size() * sizeof(T));
  }
  void put_shape(const Shape& s) {
    put<int32_t>(s.G);
    put<int32_t>(s.threads);
    put<uint8_t>(s.smem_arena);
    put<uint8_t>(s.smem_tables);
    put<uint8_t>(s.split);
    put<uint8_t>(uint8_t(s.tensor ? 1 : 0) | uint8_t(s.vsplit ? 2 : 0));
    put<uint64_t>(s.smem);
    put<int32_t>(s.grid_cap);
  }
};

struct Reader {
  const char* p;
  size_t left;
  bool ok = true;
  template <class T>
  T get() {
    T v{};
    if (!ok || left < sizeof(T)) {
      ok = false;
      return v;
    }
    std::memcpy(&v, p, sizeof(T));
    p += sizeof(T);
    left -= sizeof(T);
    return v;
  }
  template <class T>
  std::vector<T> get_vec(uint64_t max_count) {
    const uint64_t n = get<uint64_t>();
    std::vector<T> v;
    if (!ok || n > max_count || n > left / sizeof(T)) {
      ok = false;
      return v;
    }
    v.resize(n);
    if (n) std::memcpy(v.data(), p, n * sizeof(T));
    p += n * sizeof(T);
    left -= n * sizeof(T);
    return v;
  }
  Shape get_shape() {
    Shape s;
    s.G = get<int32_t>();
    s.threads = get<int32_t>();
    s.smem_arena = get<uint8_t>() != 0;
    s.smem_tables = get<uint8_t>() != 0;
    s.split = get<uint8_t>() != 0;
    const uint8_t flags = get<uint8_t>();
    s.tensor = (flags & 1) != 0;
    s.vsplit = (flags & 2) != 0;
    s.smem = (size_t)get<uint64_t>();
    s.grid_cap = get<int32_t>();
    return s;
  }
};

// True when a stored shape is one this program can launch on its device: the
// field values are in range and its shared memory, occupancy and grid cap are
// what the shape choosers would compute for them.
bool shape_consistent(const tqec_program* p, int prec, const Shape& s) {
  if (s.G < 1 || s.G > 1024 || (s.G & (s.G - 1))) return false;
  if (s.tensor && !tensor_program(p, prec)) return false;
  if (s.vsplit && s.G != 1) return false;
  if (s.threads < (s.tensor ? 128 : 32) || s.threads > tqec::contract_max_threads(prec, s.tensor) ||
      (s.threads & (s.threads - 1)))
    return false;
  if (s.split && (s.smem_arena || p->plan.arena_small <= 0 || p->plan.map_mode)) return false;
  const int nsteps = (int)p->plan.steps.size();
  const size_t tb = s.smem_tables ? table_bytes(p, prec) : 0;
  const size_t want =
      s.split ? tqec::contract_smem_bytes(prec, nsteps, syn_words(p), s.G, p->plan.arena_small, true, 0, tb, s.tensor)
              : tqec::contract_smem_bytes(prec, nsteps, syn_words(p), s.G, p->plan.arena_elems, s.smem_arena,
                                          var_words(p), tb, s.tensor);
  if (s.smem != want || s.smem > tqec::contract_smem_limit(p->device)) return false;
  const int occ = tqec::contract_occupancy(prec, s.threads, s.smem, p->plan.map_mode, s.tensor);
  return occ >= 1 && s.grid_cap >= 1 && int64_t(s.grid_cap) <= int64_t(occ) * p->sm_count;
}

}  // namespace

extern "C" {

int tqec_program_save(tqec_program* p, const char* path) {
  if (!p || !path) return fail(TQEC_ERR_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lk(p->mu);
  const ProgramInputs& in = p->inputs;
  Writer w;
  w.buf.append(kFileMagic, sizeof(kFileMagic));
  w.put<uint32_t>(kFileVersion);
  w.put<uint32_t>(kByteOrderMark);
  w.put<int32_t>(in.opts.precision);
  w.put<uint32_t>(in.opts.flags);
  w.put<int32_t>(in.opts.device);
  w.put<int32_t>(in.opts.group);
  w.put<int32_t>(in.opts.threads);
  w.put<double>(in.opts.margin);
  w.put<int32_t>(in.opts.big_elems);
  w.put<int32_t>(in.n_tensors);
  w.put_vec(in.ix_offsets);
  w.put_vec(in.ix_labels);
  w.put_vec(in.data_offsets);
  w.put_vec(in.data);
  w.put_vec(in.out_labels);
  w.put_vec(in.syndrome_tensors);
  w.put_vec(in.steps);
  w.put<uint64_t>(plan_fingerprint(p->plan));
  w.put<int32_t>(p->sm_count);
  w.put<uint64_t>(tqec::contract_smem_limit(p->device));
  for (int prec = 0; prec < 3; ++prec) {
    w.put_shape(p->shape[prec]);
    w.put<int32_t>((int32_t)p->sized[prec].size());
    for (const auto& [rows, s] : p->sized[prec]) {
      w.put<int64_t>(rows);
      w.put_shape(s);
    }
  }
  w.put_shape(p->recheck_shape);
  w.put<uint64_t>(fnv1a(w.buf.data(), w.buf.size()));
  const std::string tmp = std::string(path) + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) return fail(TQEC_ERR_IO, std::string("cannot write ") + tmp);
  const bool wrote = std::fwrite(w.buf.data(), 1, w.buf.size(), f) == w.buf.size();
  const bool closed = std::fclose(f) == 0;
  if (!wrote || !closed || std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    return fail(TQEC_ERR_IO, std::string("cannot write ") + path);
  }
  g_last_error.clear();
  return TQEC_OK;
}

int tqec_program_load(const char* path, int32_t device, tqec_program** out) {
  if (!path || !out) return fail(TQEC_ERR_INVALID, "NULL argument");
  *out = nullptr;
  std::string buf;
  {
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(TQEC_ERR_IO, std::string("cannot open ") + path);
    char chunk[1 << 16];
    size_t n;
    while ((n = std::fread(chunk, 1, sizeof(chunk), f)) > 0 && buf.size() <= kMaxFileBytes) buf.append(chunk, n);
    std::fclose(f);
  }
  const size_t head = sizeof(kFileMagic) + 2 * sizeof(uint32_t);
  if (buf.size() > kMaxFileBytes || buf.size() < head + sizeof(uint64_t) ||
      std::memcmp(buf.data(), kFileMagic, sizeof(kFileMagic)) != 0)
    return fail(TQEC_ERR_INVALID, "not a program file");
  uint64_t stored_sum;
  std::memcpy(&stored_sum, buf.data() + buf.size() - sizeof(uint64_t), sizeof(uint64_t));
  if (fnv1a(buf.data(), buf.size() - sizeof(uint64_t)) != stored_sum)
    return fail(TQEC_ERR_INVALID, "program file checksum mismatch (truncated or corrupted)");
  Reader r{buf.data() + sizeof(kFileMagic), buf.size() - sizeof(kFileMagic) - sizeof(uint64_t)};
  if (r.get<uint32_t>() != kFileVersion) return fail(TQEC_ERR_INVALID, "unsupported program file version");
  if (r.get<uint32_t>() != kByteOrderMark) return fail(TQEC_ERR_INVALID, "program file written with another byte order");
  tqec_options o;
  std::memset(&o, 0, sizeof(o));
  o.precision = r.get<int32_t>();
  o.flags = r.get<uint32_t>();
  o.device = r.get<int32_t>();
  o.group = r.get<int32_t>();
  o.threads = r.get<int32_t>();
  o.margin = r.get<double>();
  o.big_elems = r.get<int32_t>();
  const int32_t T = r.get<int32_t>();
  const uint64_t cap = uint64_t(1) << 28;
  auto ix_offsets = r.get_vec<int32_t>(cap);
  auto ix_labels = r.get_vec<int32_t>(cap);
  auto data_offsets = r.get_vec<int64_t>(cap);
  auto data = r.get_vec<double>(cap);
  auto out_labels = r.get_vec<int32_t>(cap);
  auto syndrome_tensors = r.get_vec<int32_t>(cap);
  auto steps = r.get_vec<int32_t>(cap);
  const uint64_t fingerprint = r.get<uint64_t>();
  const int32_t sm_count = r.get<int32_t>();
  const uint64_t smem_limit = r.get<uint64_t>();
  Shape shape[3];
  std::vector<std::pair<int64_t, Shape>> sized[3];
  for (int prec = 0; prec < 3 && r.ok; ++prec) {
    shape[prec] = r.get_shape();
    const int32_t ns = r.get<int32_t>();
    if (ns < 0 || ns > 64) r.ok = false;
    for (int32_t i = 0; i < ns && r.ok; ++i) {
      const int64_t rows = r.get<int64_t>();
      sized[prec].push_back({rows, r.get_shape()});
    }
  }
  const Shape recheck = r.get_shape();
  if (!r.ok || r.left != 0) return fail(TQEC_ERR_INVALID, "malformed program file");
  // the arrays must describe a network before the planner reads them
  bool sane = T >= 1 && ix_offsets.size() == size_t(T) + 1 && data_offsets.size() == size_t(T) + 1 &&
              ix_offsets[0] == 0 && data_offsets[0] == 0 && size_t(ix_offsets[T]) == ix_labels.size() &&
              uint64_t(data_offsets[T]) == data.size() && out_labels.size() <= (size_t(1) << 20) &&
              syndrome_tensors.size() <= size_t(T) && steps.size() == 2 * (size_t(T) - 1);
  for (int32_t i = 0; sane && i < T; ++i)
    sane = ix_offsets[i + 1] >= ix_offsets[i] && data_offsets[i + 1] >= data_offsets[i];
  if (!sane) return fail(TQEC_ERR_INVALID, "malformed network in program file");
  if (device >= 0) o.device = device;
  tqec_network net{T,
                   ix_offsets.data(),
                   ix_labels.data(),
                   data_offsets.data(),
                   data.data(),
                   (int32_t)out_labels.size(),
                   out_labels.empty() ? nullptr : out_labels.data(),
                   (int32_t)syndrome_tensors.size(),
                   syndrome_tensors.empty() ? nullptr : syndrome_tensors.data()};
  tqec_tree tree{T - 1, steps.empty() ? nullptr : steps.data()};
  tqec_program* p = nullptr;
  int rc = tqec_program_create(&net, &tree, &o, &p);
  if (rc) return rc;
  if (plan_fingerprint(p->plan) != fingerprint) {
    tqec_program_destroy(p);
    return fail(TQEC_ERR_INVALID, "the network compiles to a different program than the one saved");
  }
  // the stored shapes, when the device matches and every one is consistent
  const int rp = p->plan.map_mode ? TQEC_F64 : recheck_precision(p);
  bool take = sm_count == p->sm_count && smem_limit == uint64_t(tqec::contract_smem_limit(p->device)) &&
              shape_consistent(p, rp, recheck);
  for (int prec = 0; take && prec < 3; ++prec) {
    if (prec == TQEC_F32X2 && p->plan.map_mode) continue;
    take = shape_consistent(p, prec, shape[prec]);
    for (const auto& [rows, s] : sized[prec]) take = take && rows > 0 && shape_consistent(p, prec, s);
  }
  if (take) {
    for (int prec = 0; prec < 3; ++prec) {
      if (prec == TQEC_F32X2 && p->plan.map_mode) continue;
      p->shape[prec] = shape[prec];
      p->sized[prec] = sized[prec];
    }
    p->recheck_shape = recheck;
  }
  g_last_error.clear();
  *out = p;
  return TQEC_OK;
}

}  // extern "C"
