// multi.cu -- several compiled programs decoded by one persistent launch per
// batch (uneven code sizes in one launch).
//
// A batch is a set of rows of every program (row ranges fixed by
// tqec_multi_set_work).  Decoding a batch is three launches with no host
// synchronisation and no allocation, so a caller can capture one
// tqec_multi_launch into a CUDA graph and replay it once per batch:
//   1. the float32 multi-program kernel: blocks claim (program, row group)
//      units of the current batch from a device counter, largest programs
//      first, and flag rows whose class margin is inside the float32 bound;
//   2. the recheck kernel (double-float, or float64 when every program asks
//      for it) over every program's flagged rows -- except the rows of wide
//      programs (those with a cluster form for their recheck), which one
//      launch per such program re-contracts with one thread-block cluster
//      per row: a large code's recheck row no longer holds one block for the
//      whole batch;
//   3. an advance kernel: next batch, counters back to zero.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/tqec_gb300.h"
#include "contract.cuh"
#include "program_view.h"

namespace tqec {
std::string& last_error_ref();
}

namespace {

int mfail(int code, const std::string& m) {
  tqec::last_error_ref() = m;
  return code;
}

#define MQ_CUDA(x)                                                                      \
  do {                                                                                  \
    cudaError_t e_ = (x);                                                               \
    if (e_ != cudaSuccess) return mfail(TQEC_ERR_CUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
  } while (0)

struct Placement {
  int G = 1;
  bool arena_smem = false;
  size_t smem = 0;
};

// Largest power-of-two group whose shared-memory need fits `budget` (with
// at most 64K output elements of the widest step per block), else one
// syndrome with its arena in global memory.
Placement place(const tqec::ProgramMultiView& v, int precision, size_t budget, bool allow_group) {
  auto bytes = [&](int G, bool arena_smem) {
    return tqec::contract_smem_bytes(precision, v.n_steps, v.syn_words, G, v.arena_elems, arena_smem, 0, 0);
  };
  Placement pl;
  if (bytes(1, true) <= budget) {
    int G = 1;
    while (allow_group && G < 256 && bytes(G * 2, true) <= budget && (int64_t(G) * 2 << v.width) <= 16 * 4096)
      G *= 2;
    pl.G = G;
    pl.arena_smem = true;
  }
  pl.smem = bytes(pl.G, pl.arena_smem);
  return pl;
}

struct DevArray {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t put(const void* src, size_t n) {
    if (n > bytes) {
      if (p) cudaFree(p);
      p = nullptr;
      bytes = 0;
      cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 16));
      if (e != cudaSuccess) return e;
      bytes = std::max<size_t>(n, 16);
    }
    return n ? cudaMemcpy(p, src, n, cudaMemcpyHostToDevice) : cudaSuccess;
  }
  cudaError_t zeros(size_t n) {
    if (n > bytes) {
      if (p) cudaFree(p);
      p = nullptr;
      bytes = 0;
      cudaError_t e = cudaMalloc(&p, std::max<size_t>(n, 16));
      if (e != cudaSuccess) return e;
      bytes = std::max<size_t>(n, 16);
    }
    return cudaMemset(p, 0, std::max<size_t>(n, 16));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

}  // namespace

struct tqec_multi {
  int device = 0;
  int sm_count = 1;
  int n = 0;
  std::vector<tqec_program*> progs;
  std::vector<tqec::ProgramMultiView> views;
  std::vector<Placement> pl32, plr;
  size_t smem32 = 0, smem_r = 0;
  int grid32 = 1, grid_r = 1;
  int64_t arena_block32 = 0, arena_block_r = 0;  // elements per block
  DevArray arena32, arena_r;
  DevArray k32, k_r;  // KArgs per program
  int rprec = 2;       // arithmetic of the recheck launch (TQEC_F32X2 or TQEC_F64)
  DevArray units, unit_offsets, batch_rows, state, counts;
  std::vector<DevArray> lists;
  // wide programs' recheck on clusters: per program its arena (cap clusters)
  // and the launch description, and a zero word the list kernel reads as
  // those programs' count
  std::vector<DevArray> carena;
  std::vector<tqec::KArgs> kcl;
  std::vector<int> ccl;  // clusters per launch (0: the program rechecks in the list kernel)
  DevArray zero;
  int32_t n_batches = 0;
  bool ready = false;
  std::mutex mu;
};

extern "C" {

int tqec_multi_create(tqec_program* const* progs, int32_t n_progs, tqec_multi** out) {
  if (!progs || n_progs <= 0 || !out) return mfail(TQEC_ERR_INVALID, "bad argument");
  *out = nullptr;
  auto* m = new tqec_multi();
  auto bail = [&](int c, const std::string& msg) {
    tqec_multi_destroy(m);
    return mfail(c, msg);
  };
  m->n = n_progs;
  for (int i = 0; i < n_progs; ++i) {
    tqec::ProgramMultiView v;
    if (!progs[i] || tqec::program_multi_view(progs[i], &v) != TQEC_OK) return bail(TQEC_ERR_INVALID, "bad program");
    if (v.map_mode) return bail(TQEC_ERR_INVALID, "TQEC_FLAG_MAP programs decode with tqec_map_decode_batch");
    if (i > 0 && v.device != m->views[0].device) return bail(TQEC_ERR_INVALID, "programs on different devices");
    if (i > 0 && v.recheck_precision != m->views[0].recheck_precision)
      return bail(TQEC_ERR_INVALID, "programs disagree on the recheck arithmetic (TQEC_FLAG_RECHECK_F64)");
    m->progs.push_back(progs[i]);
    m->views.push_back(v);
  }
  m->device = m->views[0].device;
  m->rprec = m->views[0].recheck_precision;
  m->sm_count = m->views[0].sm_count;
  if (cudaSetDevice(m->device) != cudaSuccess) return bail(TQEC_ERR_CUDA, "cudaSetDevice");
  const size_t limit = tqec::contract_smem_limit(m->device);
  // one 512-thread block per SM (its 128 registers per thread fill the
  // register file), so a block may take all the shared memory
  const size_t budget32 = limit - 1024, budget_r = limit - 1024;
  for (const auto& v : m->views) {
    m->pl32.push_back(place(v, 1, budget32, true));
    m->plr.push_back(place(v, m->rprec, budget_r, false));
  }
  for (int i = 0; i < m->n; ++i) {
    m->smem32 = std::max(m->smem32, m->pl32[i].smem);
    m->smem_r = std::max(m->smem_r, m->plr[i].smem);
    if (!m->pl32[i].arena_smem) m->arena_block32 = std::max<int64_t>(m->arena_block32, m->views[i].arena_elems);
    if (!m->plr[i].arena_smem) m->arena_block_r = std::max<int64_t>(m->arena_block_r, m->views[i].arena_elems);
  }
  if (m->smem32 > limit || m->smem_r > limit) return bail(TQEC_ERR_UNSUPPORTED, "a program does not fit shared memory");
  const int occ32 = tqec::contract_multi_occupancy(1, tqec::kMultiThreads, m->smem32);
  const int occ_r = tqec::contract_multi_occupancy(m->rprec, tqec::kMultiThreads, m->smem_r);
  if (occ32 < 1 || occ_r < 1) return bail(TQEC_ERR_UNSUPPORTED, "multi-program launch cannot be resident");
  m->grid32 = occ32 * m->sm_count;
  m->grid_r = m->sm_count;
  if (m->arena_block32 && m->arena32.zeros(size_t(m->grid32) * m->arena_block32 * 4) != cudaSuccess)
    return bail(TQEC_ERR_OOM, "float32 arenas");
  if (m->arena_block_r && m->arena_r.zeros(size_t(m->grid_r) * m->arena_block_r * 8) != cudaSuccess)
    return bail(TQEC_ERR_OOM, "recheck arenas");
  if (m->state.zeros(2 * sizeof(int32_t)) != cudaSuccess || m->counts.zeros(sizeof(int32_t) * m->n) != cudaSuccess ||
      m->zero.zeros(sizeof(int32_t)) != cudaSuccess)
    return bail(TQEC_ERR_OOM, "counters");
  m->carena.resize(m->n);
  m->kcl.resize(m->n);
  m->ccl.assign(m->n, 0);
  for (int i = 0; i < m->n; ++i) {
    const auto& v = m->views[i];
    if (v.cluster_blocks <= 0) continue;
    // kernel attributes now: the launches may later be captured into a graph
    if (tqec::contract_cluster_configure(m->rprec, v.cluster_blocks, v.cluster_threads, v.cluster_smem) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    if (m->carena[i].zeros(size_t(v.cluster_cap) * size_t(std::max<int64_t>(v.cluster_arena_elems, 1)) * 8) !=
        cudaSuccess)
      return bail(TQEC_ERR_OOM, "cluster recheck arenas");
    m->ccl[i] = v.cluster_cap;
  }
  *out = m;
  return TQEC_OK;
}

int tqec_multi_destroy(tqec_multi* m) {
  if (!m) return TQEC_OK;
  cudaSetDevice(m->device);
  cudaDeviceSynchronize();
  for (DevArray* a : {&m->arena32, &m->arena_r, &m->k32, &m->k_r, &m->units, &m->unit_offsets, &m->batch_rows,
                      &m->state, &m->counts, &m->zero})
    a->release();
  for (auto& l : m->lists) l.release();
  for (auto& c : m->carena) c.release();
  delete m;
  return TQEC_OK;
}

int tqec_multi_set_work(tqec_multi* m, int32_t n_batches, const int64_t* batch_end_rows,
                        const uint8_t* const* syndromes, int32_t* const* class_out) {
  if (!m || n_batches <= 0 || !batch_end_rows || !syndromes || !class_out) return mfail(TQEC_ERR_INVALID, "bad argument");
  std::lock_guard<std::mutex> lk(m->mu);
  MQ_CUDA(cudaSetDevice(m->device));
  const int n = m->n;
  for (int i = 0; i < n; ++i) {
    if (!syndromes[i] || !class_out[i]) return mfail(TQEC_ERR_INVALID, "NULL program buffer");
    for (int b = 0; b < n_batches; ++b) {
      const int64_t lo = b ? batch_end_rows[(b - 1) * n + i] : 0, hi = batch_end_rows[b * n + i];
      if (hi < lo || hi > INT32_MAX) return mfail(TQEC_ERR_INVALID, "batch rows must be non-decreasing");
    }
  }
  // units, largest programs first inside each batch (they bound the batch's length)
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int x, int y) {
    return m->views[x].flops_per_syndrome * m->pl32[x].G > m->views[y].flops_per_syndrome * m->pl32[y].G;
  });
  std::vector<tqec::MultiUnit> units;
  std::vector<int64_t> offs = {0};
  std::vector<int64_t> max_rows(n, 0);
  for (int b = 0; b < n_batches; ++b) {
    for (int i : order) {
      const int64_t lo = b ? batch_end_rows[(b - 1) * n + i] : 0, hi = batch_end_rows[b * n + i];
      max_rows[i] = std::max(max_rows[i], hi - lo);
      for (int64_t r = lo; r < hi; r += m->pl32[i].G) units.push_back({i, 0, r});
    }
    offs.push_back((int64_t)units.size());
  }
  m->lists.resize(n);
  std::vector<tqec::KArgs> a32(n), a_r(n);
  for (int i = 0; i < n; ++i) {
    if (m->lists[i].zeros(sizeof(int32_t) * std::max<int64_t>(max_rows[i], 1)) != cudaSuccess)
      return mfail(TQEC_ERR_OOM, "recheck lists");
    int32_t* list = static_cast<int32_t*>(m->lists[i].p);
    int32_t* count = static_cast<int32_t*>(m->counts.p) + i;
    for (int prec : {1, m->rprec}) {
      tqec::KArgs a = prec == 1 ? m->views[i].args32 : m->views[i].args_recheck;
      const Placement& pl = prec == 1 ? m->pl32[i] : m->plr[i];
      a.G = pl.G;
      a.lg = 0;
      while ((1 << a.lg) < pl.G) a.lg++;
      // a non-null arena pointer marks a global arena: the kernel uses the block's slice
      a.arena_global = pl.arena_smem ? nullptr : (prec == 1 ? m->arena32.p : m->arena_r.p);
      a.syn = syndromes[i];
      a.class_out = class_out[i];
      a.logp_out = nullptr;
      a.err_out = nullptr;
      a.row_offset = 0;
      if (prec == 1) {
        a.list = nullptr;
        a.list_count = nullptr;
        a.recheck_margin = m->views[i].recheck_margin;
        a.recheck_list = list;
        a.recheck_count = count;
        a32[i] = a;
      } else {
        a.list = list;
        a.list_count = count;
        a.recheck_margin = -1.0;
        a.recheck_list = nullptr;
        a.recheck_count = nullptr;
        a_r[i] = a;
        if (m->ccl[i] > 0) {
          // this program's rows go to its cluster launch; the list kernel
          // sees none
          a_r[i].list_count = static_cast<const int32_t*>(m->zero.p);
          tqec::KArgs c = m->views[i].args_cluster;
          c.syn = syndromes[i];
          c.class_out = class_out[i];
          c.logp_out = nullptr;
          c.err_out = nullptr;
          c.row_offset = 0;
          c.list = list;
          c.list_count = count;
          c.n = std::max<int64_t>(max_rows[i], 1);
          c.recheck_margin = -1.0;
          c.recheck_list = nullptr;
          c.recheck_count = nullptr;
          c.arena_global = m->carena[i].p;
          m->kcl[i] = c;
        }
      }
    }
  }
  if (m->k32.put(a32.data(), sizeof(tqec::KArgs) * n) != cudaSuccess ||
      m->k_r.put(a_r.data(), sizeof(tqec::KArgs) * n) != cudaSuccess ||
      m->units.put(units.data(), sizeof(tqec::MultiUnit) * std::max<size_t>(units.size(), 1)) != cudaSuccess ||
      m->unit_offsets.put(offs.data(), sizeof(int64_t) * offs.size()) != cudaSuccess ||
      m->batch_rows.put(batch_end_rows, sizeof(int64_t) * size_t(n_batches) * n) != cudaSuccess)
    return mfail(TQEC_ERR_OOM, "work description");
  m->n_batches = n_batches;
  m->ready = true;
  MQ_CUDA(cudaMemset(m->state.p, 0, 2 * sizeof(int32_t)));
  MQ_CUDA(cudaMemset(m->counts.p, 0, sizeof(int32_t) * n));
  return TQEC_OK;
}

int tqec_multi_reset(tqec_multi* m, void* stream) {
  if (!m || !m->ready) return mfail(TQEC_ERR_INVALID, "no work set");
  std::lock_guard<std::mutex> lk(m->mu);
  MQ_CUDA(cudaSetDevice(m->device));
  cudaStream_t st = (cudaStream_t)stream;
  MQ_CUDA(cudaMemsetAsync(m->state.p, 0, 2 * sizeof(int32_t), st));
  MQ_CUDA(cudaMemsetAsync(m->counts.p, 0, sizeof(int32_t) * m->n, st));
  return TQEC_OK;
}

int tqec_multi_launch(tqec_multi* m, void* stream) {
  if (!m || !m->ready) return mfail(TQEC_ERR_INVALID, "no work set");
  std::lock_guard<std::mutex> lk(m->mu);
  cudaStream_t st = (cudaStream_t)stream;
  int32_t* batch = static_cast<int32_t*>(m->state.p);
  int32_t* next = batch + 1;
  tqec::MultiArgs a;
  std::memset(&a, 0, sizeof(a));
  a.n_progs = m->n;
  a.n_batches = m->n_batches;
  a.units = static_cast<const tqec::MultiUnit*>(m->units.p);
  a.unit_offsets = static_cast<const int64_t*>(m->unit_offsets.p);
  a.batch_rows = static_cast<const int64_t*>(m->batch_rows.p);
  a.batch = batch;
  a.next_unit = next;
  a.progs = static_cast<const tqec::KArgs*>(m->k32.p);
  a.list_mode = 0;
  a.arena_global = m->arena32.p;
  a.arena_per_block = m->arena_block32;
  MQ_CUDA(tqec::contract_multi_launch(1, a, m->grid32, tqec::kMultiThreads, m->smem32, st));
  a.progs = static_cast<const tqec::KArgs*>(m->k_r.p);
  a.list_mode = 1;
  a.arena_global = m->arena_r.p;
  a.arena_per_block = m->arena_block_r;
  MQ_CUDA(tqec::contract_multi_launch(m->rprec, a, m->grid_r, tqec::kMultiThreads, m->smem_r, st));
  for (int i = 0; i < m->n; ++i) {
    if (m->ccl[i] <= 0) continue;
    const auto& v = m->views[i];
    const int clusters = int(std::min<int64_t>(m->kcl[i].n, m->ccl[i]));
    MQ_CUDA(tqec::contract_cluster_launch(m->rprec, m->kcl[i], clusters, v.cluster_blocks, v.cluster_threads,
                                          v.cluster_smem, st, false));
  }
  MQ_CUDA(tqec::contract_multi_advance(batch, next, static_cast<int32_t*>(m->counts.p), m->n, st));
  return TQEC_OK;
}

int tqec_multi_info(const tqec_multi* m, int32_t* groups, int32_t* arena_in_smem, int32_t* grid) {
  if (!m) return mfail(TQEC_ERR_INVALID, "NULL argument");
  for (int i = 0; i < m->n; ++i) {
    if (groups) groups[i] = m->pl32[i].G;
    if (arena_in_smem) arena_in_smem[i] = m->pl32[i].arena_smem ? 1 : 0;
  }
  if (grid) *grid = m->grid32;
  return TQEC_OK;
}

}  // extern "C"
