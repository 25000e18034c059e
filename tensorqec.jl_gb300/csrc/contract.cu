// contract.cu -- batched contraction of a syndrome-conditioned factor graph.
//
// This evaluates, for many syndromes at once, what TensorQEC evaluates one
// syndrome at a time with `ct.code(ct.tensors...)` followed by `findmax`
// (src/decoding/tndecoder.jl:160-165, :248-253).  A thread block owns G
// syndromes and walks the program (plan.h) step by step; each syndrome's
// intermediates live in its arena (shared memory when it fits, otherwise a
// per-block slice of global memory that stays resident in L2).  All threads
// of the block share every step: work items are (syndrome, output element)
// pairs, so small steps are filled with many syndromes and large steps with
// many elements of one syndrome.
//
// float32 arithmetic keeps every intermediate normalised: a step records the
// maximum of its output per syndrome, and the consumer scales the operand by
// the power of two that brings that maximum to [1, 2).  Scaling by powers of
// two is exact, so the only rounding is that of the products and sums.  The
// exponents are summed into the final log-probability.
#include <cuda_bf16.h>

#include <cstdio>
#include <map>
#include <mutex>
#include <type_traits>
#include <utility>

#include "contract.cuh"
#include "dfloat.cuh"
#include "tcgen05.cuh"

namespace tqec {
namespace {

__device__ __forceinline__ int syn_bit(const uint32_t* syn, int j) {
  return (syn[j >> 5] >> (j & 31)) & 1;
}

template <typename T>
__device__ __forceinline__ T parity_val(int idx, int s) {
  return ((__popc(idx) ^ s) & 1) ? T(0) : T(1);
}

// Power-of-two normaliser of a tensor whose maximum has float bits `m`:
// returns 2^-E with E = floor(log2(max)); writes E.
__device__ __forceinline__ float norm_factor(uint32_t m, int* e) {
  if (m == 0u) {
    *e = 0;
    return 1.0f;
  }
  int be = int((m >> 23) & 0xffu);
  be = be < 1 ? 1 : (be > 253 ? 253 : be);
  *e = be - 127;
  return __uint_as_float(uint32_t(254 - be) << 23);
}

// A syndrome's intermediates: offsets below `split` live in `small` (the
// whole arena, or the pool of small tensors kept in shared memory), the rest
// in `big` (the pool of large tensors in global memory; `big` is biased by
// -split so that big + offset addresses it).  of(g) steps to syndrome g of
// the block.
template <typename T>
struct Arena {
  T* small;
  T* big;
  int32_t split;
  int32_t ss, bs;  // per-syndrome strides of the two pools
  __device__ __forceinline__ Arena of(int g) const {
    return Arena{small + int64_t(g) * ss, big + int64_t(g) * bs, split, ss, bs};
  }
  __device__ __forceinline__ T* at(int32_t off) const { return off < split ? small + off : big + off; }
};

template <typename T>
__device__ __forceinline__ const T* operand_ptr(int kind, int32_t ref, const int8_t* sel, int obits,
                                                const Arena<T>& arena_g, const T* consts, const uint32_t* syn) {
  if (kind == OP_ARENA) return arena_g.at(ref);
  int v = 0;
#pragma unroll
  for (int i = 0; i < kMaxSel; ++i)
    if (sel[i] >= 0) v |= syn_bit(syn, sel[i]) << i;
  return consts + ref + (int64_t(v) << obits);
}

// Permutation tables: int32 entries (global or shared memory) or uint16
// entries (shared memory, programs of width <= 16).
struct PermTab {
  const void* base;
  bool is16;
  __device__ __forceinline__ int at(int idx) const {
    return is16 ? int(static_cast<const uint16_t*>(base)[idx]) : static_cast<const int32_t*>(base)[idx];
  }
  // VW consecutive entries starting at idx (idx a multiple of VW, tables
  // 16-byte aligned)
  template <int VW>
  __device__ __forceinline__ void vec(int idx, int out[VW]) const {
    if (is16) {
      const uint16_t* p = static_cast<const uint16_t*>(base) + idx;
      if (VW == 8) {
        const uint4 x = *reinterpret_cast<const uint4*>(p);
        const uint32_t w[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          out[2 * j] = int(w[j] & 0xffffu);
          out[2 * j + 1] = int(w[j] >> 16);
        }
      } else {
        const uint2 x = *reinterpret_cast<const uint2*>(p);
        out[0] = int(x.x & 0xffffu);
        out[1] = int(x.x >> 16);
        out[2] = int(x.y & 0xffffu);
        out[3] = int(x.y >> 16);
      }
    } else {
      const int32_t* p = static_cast<const int32_t*>(base) + idx;
#pragma unroll
      for (int j = 0; j < VW; j += 4) {
        const int4 x = *reinterpret_cast<const int4*>(p + j);
        out[j] = x.x;
        out[j + 1] = x.y;
        out[j + 2] = x.z;
        out[j + 3] = x.w;
      }
    }
  }
};

__device__ __forceinline__ int perm_addr(const PermTab& perm, int off, int e, int lw) {
  int addr = 0;
  int tab = off;
  for (int sh = 0; sh < lw; sh += 8) {
    const int cb = lw - sh < 8 ? lw - sh : 8;
    addr |= perm.at(tab + ((e >> sh) & ((1 << cb) - 1)));
    tab += 1 << cb;
  }
  return addr;
}

// An operand: a base pointer (arena slice or constant table) plus offset.
// A step's operand and output bases for one syndrome: select tables chosen
// by its syndrome bits, arena tensors located in their pool.  Filled once
// per syndrome group (fill_step_ptrs), so steps start with plain loads.
template <typename T>
struct StepPtrs {
  const T* a;
  const T* b;
  T* out;
};

template <typename T>
__device__ void fill_step_ptrs(const KArgs& a, const StepDesc* steps, const uint32_t* s_syn, const Arena<T>& arena,
                               const T* consts, StepPtrs<T>* ptrs) {
  for (int i = threadIdx.x; i < a.G * a.n_steps; i += blockDim.x) {
    const int g = i / a.n_steps, st = i - g * a.n_steps;
    const StepDesc& d = steps[st];
    const Arena<T> ag = arena.of(g);
    const uint32_t* syn = s_syn + g * a.syn_words;
    StepPtrs<T> p;
    p.a = operand_ptr<T>(d.a_kind, d.a_ref, d.a_sel, d.lh + d.lfa + d.lk, ag, consts, syn);
    p.b = operand_ptr<T>(d.b_kind, d.b_ref, d.b_sel, d.lh + d.lk + d.lfb, ag, consts, syn);
    p.out = ag.at(d.out_off);
    ptrs[i] = p;
  }
}

// Folds a thread's running maximum into the step's per-syndrome maximum
// (one warp reduction and one shared atomic per warp that had work).
__device__ __forceinline__ void flush_max(bool had_items, uint32_t bits, uint32_t* slot) {
  if (!__any_sync(0xffffffffu, had_items)) return;
  bits = __reduce_max_sync(0xffffffffu, bits);
  if ((threadIdx.x & 31) == 0) atomicMax(slot, bits);
}

// RB (the bf16 study launches): a stored intermediate is rounded to
// bfloat16's 8 significant bits (it stays in a float word); otherwise as is.
template <bool RB, typename T>
__device__ __forceinline__ T out_round(T v) {
  if constexpr (RB && std::is_same<T, float>::value) return __bfloat162float(__float2bfloat16_rn(v));
  return v;
}

// A team is the threads that contract one syndrome group together: the
// block, or in the cluster kernel every block of a thread-block cluster
// (threads numbered rank by rank).  Team sizes are powers of two.
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_blocks() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_id() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_count() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
  return r;
}
// The address of `p`'s counterpart in the shared memory of cluster block
// `rank` (a generic address: ordinary loads, stores and atomics reach it).
template <typename P>
__device__ __forceinline__ P* cluster_map(P* p, uint32_t rank) {
  uint64_t out;
  asm volatile("mapa.u64 %0, %1, %2;" : "=l"(out) : "l"(reinterpret_cast<uint64_t>(p)), "r"(rank));
  return reinterpret_cast<P*>(out);
}
template <bool CL>
__device__ __forceinline__ int team_tid() {
  return CL ? int(cluster_rank() * blockDim.x + threadIdx.x) : int(threadIdx.x);
}
template <bool CL>
__device__ __forceinline__ int team_size() {
  return CL ? int(cluster_blocks() * blockDim.x) : int(blockDim.x);
}
// Team barrier: for a cluster, arrive with release and wait with acquire
// semantics at cluster scope, which orders every block's arena writes
// (global memory) before the other blocks' reads of them.
template <bool CL>
__device__ __forceinline__ void team_sync() {
  if (CL) {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
  } else {
    __syncthreads();
  }
}

// Thread t's position in a step whose items start item_base threads into the
// team (team sizes n are powers of two; item_base is a multiple of 32).
__device__ __forceinline__ int rotated(int t, int item_base, int n) { return (t - item_base) & (n - 1); }

// The normalisers of a step's arena operands (1 for constant operands).
template <typename T, bool NORM>
__device__ __forceinline__ void step_norms(const StepDesc& d, const uint32_t* s_max, T* fa, T* fb) {
  *fa = T(1);
  *fb = T(1);
  if (NORM) {
    int ee;
    if (d.a_kind == OP_ARENA) *fa = T(norm_factor(s_max[d.a_prod], &ee));
    if (d.b_kind == OP_ARENA) *fb = T(norm_factor(s_max[d.b_prod], &ee));
  }
}

// Segmented warp maximum of multi-syndrome work items (items of one syndrome
// are consecutive lanes).
__device__ __forceinline__ void segment_max(bool valid, uint32_t bits, int lw_items, uint32_t* slot) {
  const int seg = lw_items >= 5 ? 32 : (1 << lw_items);
  for (int o = 1; o < seg; o <<= 1) {
    const uint32_t other = __shfl_xor_sync(0xffffffffu, bits, o);
    bits = other > bits ? other : bits;
  }
  if (valid && (threadIdx.x & (seg - 1)) == 0) atomicMax(slot, bits);
}

// One output per work item.  G1: the step runs for one syndrome (the
// block's only one, or one of its G in turn), so its bases and normalisers
// are step invariants.
template <typename T, bool NORM, bool MAXP, bool G1, bool CL, bool RB = false>
__device__ void run_step(const KArgs& a, const StepDesc& dref, int st, int item_base, uint32_t* s_max,
                         const StepPtrs<T>* ptrs, const PermTab& ptab) {
  // a register copy: arena stores (same shared array) cannot alias it
  const StepDesc d = dref;
  const int lw = d.lh + d.lfa + d.lfb;
  const int total = 1 << (lw + (G1 ? 0 : a.lg));
  const int total_r = (total + 31) & ~31;
  const int mfb = (1 << d.lfb) - 1;
  const int mfa = (1 << d.lfa) - 1;
  const int mw = (1 << lw) - 1;
  const int K = 1 << d.lk;
  const bool bT = (d.flags & kStepTensor) != 0;
  const int kstride = bT ? 1 : (1 << d.lfb);
  const int nthr = team_size<CL>();
  const int i0 = rotated(team_tid<CL>(), item_base, nthr);
  StepPtrs<T> p1{};
  T fa1 = T(1), fb1 = T(1);
  if (G1) {
    p1 = ptrs[st];
    step_norms<T, NORM>(d, s_max, &fa1, &fb1);
  }
  uint32_t run_bits = 0u;
  for (int i = i0; i < (G1 ? total : total_r); i += nthr) {
    const bool valid = G1 || i < total;
    const int g = G1 ? 0 : (valid ? (i >> lw) : 0);
    const int e = i & mw;
    T acc = T(0);
    if (valid) {
      StepPtrs<T> p = p1;
      T fa_s = fa1, fb_s = fb1;
      if (!G1) {
        p = ptrs[g * a.n_steps + st];
        step_norms<T, NORM>(d, s_max + g * a.n_steps, &fa_s, &fb_s);
      }
      const int fb = e & mfb;
      const int fa = (e >> d.lfb) & mfa;
      const int h = e >> (d.lfb + d.lfa);
      const T* pa = p.a + (((h << d.lfa) | fa) << d.lk);
      // B is [h][k][fb], or [h][fb][k] for a GEMM-shaped step
      const T* pb = p.b + (bT ? (((h << d.lfb) | fb) << d.lk) : ((h << (d.lk + d.lfb)) | fb));
      for (int k = 0; k < K; ++k) {
        T a0 = pa[k];
        // both normalisers on the A value (exact powers of two): the output
        // needs no scaling of its own
        if (NORM) a0 = scale(scale(a0, fa_s), fb_s);
        if constexpr (MAXP) {
          const T v = a0 * pb[k * kstride];
          acc = v > acc ? v : acc;
        } else {
          acc = fma(a0, pb[k * kstride], acc);
        }
      }
      const int addr = d.perm_off < 0 ? e : perm_addr(ptab, d.perm_off, e, lw);
      acc = out_round<RB>(acc);
      p.out[addr] = acc;
    }
    if (NORM && G1) {
      const uint32_t bits = __float_as_uint(float(acc));
      run_bits = bits > run_bits ? bits : run_bits;
    } else if (NORM) {
      segment_max(valid, __float_as_uint(float(acc)), lw, &s_max[g * a.n_steps + st]);
    }
  }
  if (NORM && G1) flush_max(i0 < total, run_bits, &s_max[st]);
  return;
}

template <typename T>
__device__ __forceinline__ void load4(const T* p, T v[4]);
template <>
__device__ __forceinline__ void load4<float>(const float* p, float v[4]) {
  const float4 x = *reinterpret_cast<const float4*>(p);
  v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
}
template <>
__device__ __forceinline__ void load4<double>(const double* p, double v[4]) {
  const double2 x = reinterpret_cast<const double2*>(p)[0];
  const double2 y = reinterpret_cast<const double2*>(p)[1];
  v[0] = x.x; v[1] = x.y; v[2] = y.x; v[3] = y.y;
}

template <>
__device__ __forceinline__ void load4<dfloat>(const dfloat* p, dfloat v[4]) {
  const float4 x = reinterpret_cast<const float4*>(p)[0];
  const float4 y = reinterpret_cast<const float4*>(p)[1];
  v[0] = dfloat(x.x, x.y); v[1] = dfloat(x.z, x.w); v[2] = dfloat(y.x, y.y); v[3] = dfloat(y.z, y.w);
}

template <typename T>
__device__ __forceinline__ void store4(T* p, const T v[4]);
template <>
__device__ __forceinline__ void store4<float>(float* p, const float v[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
template <>
__device__ __forceinline__ void store4<double>(double* p, const double v[4]) {
  reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
}
template <>
__device__ __forceinline__ void store4<dfloat>(dfloat* p, const dfloat v[4]) {
  reinterpret_cast<float4*>(p)[0] = make_float4(v[0].hi, v[0].lo, v[1].hi, v[1].lo);
  reinterpret_cast<float4*>(p)[1] = make_float4(v[2].hi, v[2].lo, v[3].hi, v[3].lo);
}

// A step whose B-only group has at least log2(VW) bits: each work item is VW
// (4 or 8) consecutive outputs along fb, which share every A value and read
// B as 16-byte vectors.  Operand bases, fb offsets and k strides are
// multiples of 8 elements (arena and constant offsets are planned that way),
// so the vector accesses are aligned.  Permuted outputs are written in a
// lane-rotated order where the planner found that it spreads the stores of
// one warp instruction over more shared-memory banks.
template <typename T, int VW, bool NORM, bool MAXP, bool G1, bool CL, bool RB = false>
__device__ void run_step_vec(const KArgs& a, const StepDesc& dref, int st, int item_base, uint32_t* s_max,
                             const StepPtrs<T>* ptrs, const PermTab& ptab, bool contiguous) {
  constexpr int LV = VW == 8 ? 3 : 2;
  const StepDesc d = dref;
  const int lw = d.lh + d.lfa + d.lfb;
  const int lwv = lw - LV;
  const int total = 1 << (lwv + (G1 ? 0 : a.lg));
  const int total_r = (total + 31) & ~31;
  const int mfb = (1 << d.lfb) - 1;
  const int mfa = (1 << d.lfa) - 1;
  const int mwv = (1 << lwv) - 1;
  const int K = 1 << d.lk;
  const int bstride = 1 << d.lfb;
  const bool permuted = d.perm_off >= 0;
  const int cb0 = lw < 8 ? lw : 8;
  const int rot = threadIdx.x & (VW - 1);
  const int nthr = team_size<CL>();
  const int i0 = rotated(team_tid<CL>(), item_base, nthr);
  StepPtrs<T> p1{};
  T fa1 = T(1), fb1 = T(1);
  if (G1) {
    p1 = ptrs[st];
    step_norms<T, NORM>(d, s_max, &fa1, &fb1);
  }
  uint32_t run_bits = 0u;
  for (int i = i0; i < (G1 ? total : total_r); i += nthr) {
    const bool valid = G1 || i < total;
    const int g = G1 ? 0 : (valid ? (i >> lwv) : 0);
    const int e0 = (i & mwv) << LV;
    T acc[VW];
#pragma unroll
    for (int j = 0; j < VW; ++j) acc[j] = T(0);
    if (valid) {
      StepPtrs<T> p = p1;
      T fa_s = fa1, fb_s = fb1;
      if (!G1) {
        p = ptrs[g * a.n_steps + st];
        step_norms<T, NORM>(d, s_max + g * a.n_steps, &fa_s, &fb_s);
      }
      const int fb0 = e0 & mfb;
      const int fa = (e0 >> d.lfb) & mfa;
      const int h = e0 >> (d.lfb + d.lfa);
      const T* pa = p.a + (((h << d.lfa) | fa) << d.lk);
      const T* pb = p.b + ((h << (d.lk + d.lfb)) | fb0);
      auto body = [&](int k) {
        T av = pa[k];
        // both normalisers on the shared A value (exact powers of two), so
        // the VW outputs need no scaling of their own
        if (NORM) av = scale(scale(av, fa_s), fb_s);
        T bv[VW];
        const T* q = pb + k * bstride;
        load4<T>(q, bv);
        if (VW == 8) load4<T>(q + 4, bv + 4);
#pragma unroll
        for (int j = 0; j < VW; ++j) {
          if constexpr (MAXP) {
            const T v = av * bv[j];
            acc[j] = v > acc[j] ? v : acc[j];
          } else {
            acc[j] = fma(av, bv[j], acc[j]);
          }
        }
      };
      if (K == 1) {
        body(0);
      } else if (K >= 4) {
        // four k at a time with every load issued before the multiply-adds
        // (A as one 16-byte vector: rows are K >= 4 elements and operand
        // bases are 4-aligned), so a step whose operands come from L2 waits
        // once per four k instead of once per two
        for (int k = 0; k < K; k += 4) {
          T a4[4], b4[4][VW];
          load4<T>(pa + k, a4);
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            load4<T>(pb + (k + c) * bstride, b4[c]);
            if (VW == 8) load4<T>(pb + (k + c) * bstride + 4, b4[c] + 4);
          }
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            T av = a4[c];
            if (NORM) av = scale(scale(av, fa_s), fb_s);
#pragma unroll
            for (int j = 0; j < VW; ++j) {
              if constexpr (MAXP) {
                const T v = av * b4[c][j];
                acc[j] = v > acc[j] ? v : acc[j];
              } else {
                acc[j] = fma(av, b4[c][j], acc[j]);
              }
            }
          }
        }
      } else {
        for (int k = 0; k < K; k += 2) {
          body(k);
          body(k + 1);
        }
      }
      if constexpr (RB) {
#pragma unroll
        for (int j = 0; j < VW; ++j) acc[j] = out_round<RB>(acc[j]);
      }
      if (!permuted || contiguous) {
        // the permutation keeps the low log2(VW) index bits in place (or
        // there is none): the VW outputs are VW consecutive elements at the
        // image of the first, a multiple of VW
        T* out = p.out + (permuted ? perm_addr(ptab, d.perm_off, e0, lw) : e0);
        store4<T>(out, acc);
        if (VW == 8) store4<T>(out + 4, acc + 4);
      } else {
        int los[VW];
        ptab.vec<VW>(d.perm_off + (e0 & ((1 << cb0) - 1)), los);
        int hi = 0;
        int tab = d.perm_off + (1 << cb0);
        for (int sh = 8; sh < lw; sh += 8) {
          const int cb = lw - sh < 8 ? lw - sh : 8;
          hi |= ptab.at(tab + ((e0 >> sh) & ((1 << cb) - 1)));
          tab += 1 << cb;
        }
        T* out = p.out;
        if (d.flags & (VW == 8 ? kStepRotate8 : kStepRotate4)) {
          // barrel rotation: lane r stores its outputs starting at r mod VW,
          // so the lanes of one store instruction differ in the low bits too
#pragma unroll
          for (int b = 1; b < VW; b <<= 1) {
            if (rot & b) {
              int tl[VW];
              T tv[VW];
#pragma unroll
              for (int j = 0; j < VW; ++j) {
                tl[j] = los[(j + b) & (VW - 1)];
                tv[j] = acc[(j + b) & (VW - 1)];
              }
#pragma unroll
              for (int j = 0; j < VW; ++j) {
                los[j] = tl[j];
                acc[j] = tv[j];
              }
            }
          }
        }
#pragma unroll
        for (int j = 0; j < VW; ++j) out[los[j] | hi] = acc[j];
      }
    }
    if (NORM) {
      float m = float(acc[0]);
#pragma unroll
      for (int j = 1; j < VW; ++j) m = fmaxf(m, float(acc[j]));
      const uint32_t bits = __float_as_uint(m);
      if (G1) run_bits = bits > run_bits ? bits : run_bits;
      else segment_max(valid, bits, lwv, &s_max[g * a.n_steps + st]);
    }
  }
  if (NORM && G1) flush_max(i0 < total, run_bits, &s_max[st]);
}

// A step with few outputs and a long k range: TPO (a power of two, at most
// 32) consecutive lanes share one output, each summing every TPO-th k, and
// combine their partial sums with shuffles (maxima in max-product mode).
template <typename T, bool NORM, bool MAXP, bool G1, bool CL, bool RB = false>
__device__ void run_step_splitk(const KArgs& a, const StepDesc& dref, int st, int item_base, int lt,
                                uint32_t* s_max, const StepPtrs<T>* ptrs, const PermTab& ptab) {
  const StepDesc d = dref;
  const int tpo = 1 << lt;
  const int lw = d.lh + d.lfa + d.lfb;
  const int outs = 1 << (lw + (G1 ? 0 : a.lg));
  const int total = outs << lt;
  const int total_r = (total + 31) & ~31;
  const int mfb = (1 << d.lfb) - 1;
  const int mfa = (1 << d.lfa) - 1;
  const int mw = (1 << lw) - 1;
  const int K = 1 << d.lk;
  const int nthr = team_size<CL>();
  const int vt0 = rotated(team_tid<CL>(), item_base, nthr);
  uint32_t run_bits = 0u;
  // whole warps iterate together (the shuffles below need every lane)
  for (int vt = vt0; vt < total_r; vt += nthr) {
    const bool valid = vt < total;
    const int item = vt >> lt, sub = vt & (tpo - 1);
    const int g = G1 ? 0 : (valid ? (item >> lw) : 0);
    const int e = item & mw;
    T acc = T(0);
    StepPtrs<T> p{};
    T fa_s = T(1), fb_s = T(1);
    if (valid) {
      p = ptrs[g * a.n_steps + st];
      step_norms<T, NORM>(d, s_max + g * a.n_steps, &fa_s, &fb_s);
      const int fb = e & mfb;
      const int fa = (e >> d.lfb) & mfa;
      const int h = e >> (d.lfb + d.lfa);
      const T* pa = p.a + (((h << d.lfa) | fa) << d.lk);
      const bool bT = (d.flags & kStepTensor) != 0;
      const T* pb = p.b + (bT ? (((h << d.lfb) | fb) << d.lk) : ((h << (d.lk + d.lfb)) | fb));
      const int kstride = bT ? 1 : (1 << d.lfb);
      for (int k = sub; k < K; k += tpo) {
        const T av = scale(pa[k], fa_s);
        const T bv = pb[k * kstride];
        if constexpr (MAXP) {
          const T v = av * bv;
          acc = v > acc ? v : acc;
        } else {
          acc = fma(av, bv, acc);
        }
      }
    }
    for (int o = 1; o < tpo; o <<= 1) {
      const T other = __shfl_xor_sync(0xffffffffu, acc, o);
      if constexpr (MAXP) acc = other > acc ? other : acc;
      else acc = acc + other;
    }
    if (valid && sub == 0) {
      if (NORM) acc = scale(acc, fb_s);
      const int addr = d.perm_off < 0 ? e : perm_addr(ptab, d.perm_off, e, lw);
      acc = out_round<RB>(acc);
      p.out[addr] = acc;
      if (NORM) {
        const uint32_t bits = __float_as_uint(float(acc));
        if (G1) run_bits = bits > run_bits ? bits : run_bits;
        else atomicMax(&s_max[g * a.n_steps + st], bits);
      }
    }
  }
  if (NORM && G1) flush_max(vt0 < total, run_bits, &s_max[st]);
}

// A step of four-output items (as SK_VEC4) with fewer items than the team
// has threads: TPO = 2^lt consecutive lanes share an item, lane `sub` sums
// the k run [sub*K/TPO, (sub+1)*K/TPO) (at least four k, loaded before the
// multiply-adds), and the partial sums meet by shuffles.  Used where one
// syndrome has a whole block or cluster to itself, so a step's chain of
// dependent operand loads is shortened by the lanes that would otherwise idle.
template <typename T, bool NORM, bool MAXP, bool G1, bool CL, bool RB = false>
__device__ void run_step_vsplit(const KArgs& a, const StepDesc& dref, int st, int item_base, int lt,
                                uint32_t* s_max, const StepPtrs<T>* ptrs, const PermTab& ptab, bool contiguous) {
  const StepDesc d = dref;
  const int tpo = 1 << lt;
  const int lw = d.lh + d.lfa + d.lfb;
  const int lwv = lw - 2;
  const int items = 1 << (lwv + (G1 ? 0 : a.lg));
  const int total = items << lt;
  const int total_r = (total + 31) & ~31;
  const int mfb = (1 << d.lfb) - 1;
  const int mfa = (1 << d.lfa) - 1;
  const int mwv = (1 << lwv) - 1;
  const int kc = (1 << d.lk) >> lt;  // k per lane, a multiple of 4
  const int bstride = 1 << d.lfb;
  const bool permuted = d.perm_off >= 0;
  const int cb0 = lw < 8 ? lw : 8;
  const int nthr = team_size<CL>();
  const int vt0 = rotated(team_tid<CL>(), item_base, nthr);
  uint32_t run_bits = 0u;
  // whole warps iterate together (the shuffles below need every lane)
  for (int vt = vt0; vt < total_r; vt += nthr) {
    const bool valid = vt < total;
    const int item = vt >> lt, sub = vt & (tpo - 1);
    const int g = G1 ? 0 : (valid ? (item >> lwv) : 0);
    const int e0 = (item & mwv) << 2;
    T acc[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[j] = T(0);
    StepPtrs<T> p{};
    if (valid) {
      p = ptrs[g * a.n_steps + st];
      T fa_s = T(1), fb_s = T(1);
      step_norms<T, NORM>(d, s_max + g * a.n_steps, &fa_s, &fb_s);
      const int fb0 = e0 & mfb;
      const int fa = (e0 >> d.lfb) & mfa;
      const int h = e0 >> (d.lfb + d.lfa);
      const T* pa = p.a + (((h << d.lfa) | fa) << d.lk) + sub * kc;
      const T* pb = p.b + ((h << (d.lk + d.lfb)) | fb0) + sub * kc * bstride;
      for (int k = 0; k < kc; k += 4) {
        T a4[4], b4[4][4];
        load4<T>(pa + k, a4);
#pragma unroll
        for (int c = 0; c < 4; ++c) load4<T>(pb + (k + c) * bstride, b4[c]);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          T av = a4[c];
          if (NORM) av = scale(scale(av, fa_s), fb_s);
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            if constexpr (MAXP) {
              const T v = av * b4[c][j];
              acc[j] = v > acc[j] ? v : acc[j];
            } else {
              acc[j] = fma(av, b4[c][j], acc[j]);
            }
          }
        }
      }
    }
    for (int o = 1; o < tpo; o <<= 1) {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const T other = __shfl_xor_sync(0xffffffffu, acc[j], o);
        if constexpr (MAXP) acc[j] = other > acc[j] ? other : acc[j];
        else acc[j] = acc[j] + other;
      }
    }
    const bool writer = valid && sub == 0;
    if (writer) {
      if constexpr (RB) {
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[j] = out_round<RB>(acc[j]);
      }
      if (!permuted || contiguous) {
        store4<T>(p.out + (permuted ? perm_addr(ptab, d.perm_off, e0, lw) : e0), acc);
      } else {
        int los[4];
        ptab.vec<4>(d.perm_off + (e0 & ((1 << cb0) - 1)), los);
        int hi = 0;
        int tab = d.perm_off + (1 << cb0);
        for (int sh = 8; sh < lw; sh += 8) {
          const int cb = lw - sh < 8 ? lw - sh : 8;
          hi |= ptab.at(tab + ((e0 >> sh) & ((1 << cb) - 1)));
          tab += 1 << cb;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) p.out[los[j] | hi] = acc[j];
      }
    }
    if (NORM && writer) {
      const float m = fmaxf(fmaxf(float(acc[0]), float(acc[1])), fmaxf(float(acc[2]), float(acc[3])));
      const uint32_t bits = __float_as_uint(m);
      if (G1) run_bits = bits > run_bits ? bits : run_bits;
      else atomicMax(&s_max[g * a.n_steps + st], bits);
    }
  }
  if (NORM && G1) flush_max(vt0 < total, run_bits, &s_max[st]);
}

// Most probable configuration: after the max-product pass every runtime
// step's output is still in the arena.  Walking the steps from the root
// down, the values of a step's output labels are known (set by its
// consumer), which fixes (h, fa, fb); the k maximising A[h,fa,k] B[h,k,fb]
// (first maximum) gives the values of the labels the step maximised over.
// One warp per syndrome; lanes split the k range.
template <typename T>
__device__ void backtrack(const KArgs& a, const StepDesc* s_steps, const uint32_t* s_syn, uint32_t* s_asg,
                          const Arena<T>& arena,
                          const T* consts, int64_t base, int64_t nrows) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nwarps = blockDim.x >> 5;
  for (int g = warp; g < a.G; g += nwarps) {
    const int64_t r = base + g;
    if (r >= nrows) continue;
    uint32_t* asg = s_asg + g * a.var_words;
    const uint32_t* syn = s_syn + g * a.syn_words;
    const Arena<T> arena_g = arena.of(g);
    for (int w = lane; w < a.var_words; w += 32) {
      uint32_t v = 0;
      for (int b = 0; b < 32; ++b) {
        const int id = w * 32 + b;
        if (id < a.n_vars && a.fixed[id] == 1) v |= 1u << b;
      }
      asg[w] = v;
    }
    __syncwarp();
    for (int st = a.n_steps - 1; st >= 0; --st) {
      const StepDesc& d = s_steps[st];
      const int32_t* vt = a.vartab + d.var_off;
      auto bit = [&](int id) { return int((asg[id >> 5] >> (id & 31)) & 1u); };
      int fb = 0, fa = 0, h = 0;
      for (int j = 0; j < d.lfb; ++j) fb |= bit(vt[j]) << j;
      for (int j = 0; j < d.lfa; ++j) fa |= bit(vt[d.lfb + j]) << j;
      for (int j = 0; j < d.lh; ++j) h |= bit(vt[d.lfb + d.lfa + j]) << j;
      const int abase = ((h << d.lfa) | fa) << d.lk;
      const int bbase = (h << (d.lk + d.lfb)) | fb;
      const int abits = d.lh + d.lfa + d.lk, bbits = d.lh + d.lk + d.lfb;
      const bool apar = d.a_kind == OP_PARITY, bpar = d.b_kind == OP_PARITY;
      const T* ap = apar ? nullptr : operand_ptr<T>(d.a_kind, d.a_ref, d.a_sel, abits, arena_g, consts, syn);
      const T* bp = bpar ? nullptr : operand_ptr<T>(d.b_kind, d.b_ref, d.b_sel, bbits, arena_g, consts, syn);
      const int as = apar ? syn_bit(syn, d.a_ref) : 0, bs = bpar ? syn_bit(syn, d.b_ref) : 0;
      T best = T(-1);
      int bk = 0;
      for (int k = lane; k < (1 << d.lk); k += 32) {
        const int ai = abase + k, bi = bbase + (k << d.lfb);
        const T av = apar ? parity_val<T>(ai, as) : ap[ai];
        const T bv = bpar ? parity_val<T>(bi, bs) : bp[bi];
        const T v = av * bv;
        if (v > best) {
          best = v;
          bk = k;
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const T ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int okk = __shfl_xor_sync(0xffffffffu, bk, o);
        if (ob > best || (ob == best && okk < bk)) {
          best = ob;
          bk = okk;
        }
      }
      if (lane == 0) {
        const int32_t* kv = vt + d.lfb + d.lfa + d.lh;
        for (int j = 0; j < d.lk; ++j) {
          const int id = kv[j];
          const uint32_t m = 1u << (id & 31);
          if ((bk >> j) & 1) asg[id >> 5] |= m;
          else asg[id >> 5] &= ~m;
        }
      }
      __syncwarp();
    }
    if (a.assign_out) {
      const int rb = (a.n_report + 7) / 8;
      const int64_t row = a.list ? int64_t(a.list[r]) : r + a.row_offset;
      for (int byte = lane; byte < rb; byte += 32) {
        uint32_t v = 0;
        for (int b = 0; b < 8; ++b) {
          const int i = byte * 8 + b;
          if (i < a.n_report) {
            const int id = a.report[i];
            v |= ((asg[id >> 5] >> (id & 31)) & 1u) << b;
          }
        }
        a.assign_out[row * rb + byte] = uint8_t(v);
      }
    }
  }
}

// How a step is executed and how many work items it has (rounded up to a
// warp): several lanes per output for few outputs over a long k range,
// eight or four outputs per item along fb, else one output per item.
enum StepKind { SK_SPLITK, SK_VEC8, SK_VEC4, SK_SCALAR, SK_TENSOR, SK_VSPLIT };
struct StepShape {
  int kind;
  int lt;       // SK_SPLITK / SK_VSPLIT: log2 of the lanes per output / per four outputs
  int total_r;  // work items (threads for SK_SPLITK), a multiple of 32
  bool contiguous;  // SK_VEC8 / SK_VEC4: the output permutation keeps the item's low bits in place
};

template <typename T>
__device__ __forceinline__ StepShape step_shape(int lh, int lfa, int lfb, int lk, int lg, int flags, bool tensor,
                                                int64_t bd, bool vsplit = false) {
  const int lw = lh + lfa + lfb;
  const int64_t outs = int64_t(1) << (lw + lg);
  StepShape sh;
  sh.lt = 0;
  sh.contiguous = false;
  const bool bT = (flags & kStepTensor) != 0;
  if (bT && tensor) {  // the tensor cores, the whole block per syndrome
    sh.kind = SK_TENSOR;
    sh.total_r = int(bd);
    return sh;
  }
  int lt = 0;
  while (lt < 5 && (outs << (lt + 1)) <= bd && (lt + 1) + 2 <= lk) ++lt;
  int64_t total;
  if (lt >= 2) {
    sh.kind = SK_SPLITK;
    total = outs << lt;
  } else if (bT) {  // B is K-major: no vector loads along fb
    sh.kind = SK_SCALAR;
    total = outs;
  } else if (sizeof(T) == 4 && lfb >= 3 && (outs >> 3) >= bd) {
    sh.kind = SK_VEC8;
    total = outs >> 3;
  } else if (lfb >= 2) {
    // four outputs per item; where that leaves threads idle (and vsplit is
    // allowed), 2-8 lanes share an item, each taking a run of >= 4 k
    int vl = 0;
    if (vsplit)
      while (vl < 3 && ((outs >> 2) << (vl + 1)) <= bd && lk - (vl + 1) >= 2) ++vl;
    sh.kind = vl ? SK_VSPLIT : SK_VEC4;
    total = (outs >> 2) << vl;
    lt = vl;
  } else {
    sh.kind = SK_SCALAR;
    total = outs;
  }
  sh.lt = lt;
  sh.total_r = int((total + 31) & ~int64_t(31));
  return sh;
}

// Tensor-core state of a block: the mbarrier the MMAs complete on, the
// phase it is at, the tensor memory, and whether a wait gave up.
struct TcState {
  uint64_t bar;
  uint32_t tmem;
  uint32_t phase;
  int32_t abort;
  int32_t pad;
};

// Stages rows [0, rows) x k [k0, k0+32) of a K-major float32 matrix (rows
// `ld` elements apart) into two 128-byte-swizzled tiles holding the tf32
// high and low parts of scale * x.
__device__ __forceinline__ void stage_split(const float* src, int rows, int ld, int k0, float scale,
                                            unsigned char* hi, unsigned char* lo) {
  for (int i = threadIdx.x; i < rows * 8; i += blockDim.x) {
    const int r = i >> 3, c = i & 7;
    const float4 v = *reinterpret_cast<const float4*>(src + int64_t(r) * ld + k0 + 4 * c);
    float4 h, l;
    tc::split_tf32(v.x * scale, &h.x, &l.x);
    tc::split_tf32(v.y * scale, &h.y, &l.y);
    tc::split_tf32(v.z * scale, &h.z, &l.z);
    tc::split_tf32(v.w * scale, &h.w, &l.w);
    const int off = r * 128 + ((c ^ (r & 7)) << 4);
    *reinterpret_cast<float4*>(hi + off) = h;
    *reinterpret_cast<float4*>(lo + off) = l;
  }
}

// A GEMM-shaped step on the tensor cores, for one syndrome: per h, 128-row
// tiles of A ([h][fa][k]) times up to 128-column tiles of B ([h][fb][k]),
// k in chunks of 32 staged by the whole block as tf32 high/low parts; one
// thread issues hi*hi + hi*lo + lo*hi per 8-element k step into tensor
// memory (float32 accumulation); every warp then reads a quarter of the
// tile's rows back (tcgen05.ld), scales, and stores through the step's
// permutation.  A's normaliser is applied while staging (exact), B's on the
// way out.
template <typename T, bool NORM>
__device__ void run_step_tc(const KArgs& a, const StepDesc& dref, int st, uint32_t* s_max, const StepPtrs<T>* ptrs,
                            const PermTab& ptab, TcState* ts, unsigned char* tbuf) {
  const StepDesc d = dref;
  const StepPtrs<T> p = ptrs[st];
  T fa_s, fb_s;
  step_norms<T, NORM>(d, s_max, &fa_s, &fb_s);
  const int M = 1 << d.lfa, N = 1 << d.lfb, K = 1 << d.lk, H = 1 << d.lh;
  const int lw = d.lh + d.lfa + d.lfb;
  const int n_tile = N < tc::kNMax ? N : tc::kNMax;
  const uint32_t idesc = tc::idesc_tf32(n_tile);
  unsigned char* a_hi = tbuf;
  unsigned char* a_lo = tbuf + tc::kTileBytes;
  unsigned char* b_hi = tbuf + 2 * tc::kTileBytes;
  unsigned char* b_lo = tbuf + 3 * tc::kTileBytes;
  const uint64_t dah = tc::sdesc(tc::smem_u32(a_hi)), dal = tc::sdesc(tc::smem_u32(a_lo));
  const uint64_t dbh = tc::sdesc(tc::smem_u32(b_hi)), dbl = tc::sdesc(tc::smem_u32(b_lo));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, groups = int(blockDim.x >> 7);
  uint32_t phase = ts->phase;
  uint32_t run_bits = 0u;
  for (int h = 0; h < H; ++h)
    for (int m0 = 0; m0 < M; m0 += tc::kM)
      for (int n0 = 0; n0 < N; n0 += n_tile) {
        const float* A = reinterpret_cast<const float*>(p.a) + (int64_t(h) * M + m0) * K;
        const float* B = reinterpret_cast<const float*>(p.b) + (int64_t(h) * N + n0) * K;
        for (int k0 = 0; k0 < K; k0 += tc::kK) {
          if (ts->abort) break;  // block-uniform (written before a barrier)
          stage_split(A, tc::kM, K, k0, float(fa_s), a_hi, a_lo);
          stage_split(B, n_tile, K, k0, 1.0f, b_hi, b_lo);
          tc::fence_proxy_async();
          tc::fence_before();
          __syncthreads();
          tc::fence_after();
          if (threadIdx.x == 0) {
#pragma unroll
            for (int kk = 0; kk < tc::kK / 8; ++kk) {  // 8 tf32 = 32 bytes along k per instruction
              const uint64_t o = uint64_t(kk * 2);
              tc::mma_tf32(ts->tmem, dah + o, dbh + o, idesc, (k0 | kk) != 0 ? 1u : 0u);
              tc::mma_tf32(ts->tmem, dah + o, dbl + o, idesc, 1u);
              tc::mma_tf32(ts->tmem, dal + o, dbh + o, idesc, 1u);
            }
            tc::commit(&ts->bar);
          }
          // the staging buffers are reused once the MMAs have read them
          const bool ok = tc::mbar_wait(&ts->bar, phase);
          phase ^= 1u;
          if (!ok) {
            ts->abort = 1;
            *static_cast<volatile int32_t*>(a.tc_err) = 1;
          }
          __syncthreads();
        }
        tc::fence_after();
        if (!ts->abort) {
          const int q = warp & 3;
          const int m = m0 + q * 32 + lane;
          for (int c = warp >> 2; c < n_tile / 32; c += groups) {
            uint32_t r[32];
            tc::ld32(ts->tmem + (uint32_t(q * 32) << 16) + uint32_t(c * 32), r);
            // the 32 outputs differ in index bits 0-4 only: one lookup in the
            // permutation's low table each, the higher tables once
            const int e0 = (((h << d.lfa) | m) << d.lfb) | (n0 + c * 32);
            int hi = 0, lo0 = 0;
            if (d.perm_off >= 0) {
              int tab = d.perm_off + 256;
              for (int sh = 8; sh < lw; sh += 8) {
                const int cb = lw - sh < 8 ? lw - sh : 8;
                hi |= ptab.at(tab + ((e0 >> sh) & ((1 << cb) - 1)));
                tab += 1 << cb;
              }
              lo0 = d.perm_off + (e0 & 0xE0);
            }
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const float v = __uint_as_float(r[j]) * float(fb_s);
              const int addr = d.perm_off < 0 ? e0 + j : (ptab.at(lo0 + j) | hi);
              p.out[addr] = T(v);
              const uint32_t bits = __float_as_uint(v);
              run_bits = bits > run_bits ? bits : run_bits;
            }
          }
        }
        // tensor-memory reads are done before the next tile's MMAs overwrite it
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
      }
  if (threadIdx.x == 0) ts->phase = phase;
  if (NORM) flush_max(true, run_bits, &s_max[st]);
  __syncthreads();
}

// The planner hands the kernel arena and constant operands only (parity
// operands become syndrome-selected tables), so each step shape has one code
// path: the kernel stays small enough for the instruction caches.
template <typename T, bool NORM, bool MAXP, bool G1, bool TENSOR, bool CL, bool VS = false, bool RB = false>
__device__ __forceinline__ void dispatch_step(const KArgs& a, const StepDesc& d, const StepShape& sh, int st,
                                              int item_base, uint32_t* s_max, const StepPtrs<T>* ptrs,
                                              const PermTab& ptab, TcState* ts, unsigned char* tbuf) {
  if constexpr (TENSOR && !CL && !RB && std::is_same<T, float>::value && NORM && !MAXP && G1) {
    if (sh.kind == SK_TENSOR) {
      run_step_tc<T, NORM>(a, d, st, s_max, ptrs, ptab, ts, tbuf);
      return;
    }
  }
  switch (sh.kind) {
    case SK_SPLITK:
      run_step_splitk<T, NORM, MAXP, G1, CL, RB>(a, d, st, item_base, sh.lt, s_max, ptrs, ptab);
      break;
    case SK_VSPLIT:  // planned where the launch allows it (KArgs::vsplit, the cluster kernel)
      if constexpr (VS) run_step_vsplit<T, NORM, MAXP, G1, CL, RB>(a, d, st, item_base, sh.lt, s_max, ptrs, ptab,
                                                                   sh.contiguous);
      break;
    case SK_VEC8:  // float32 only (step_shape)
      if constexpr (sizeof(T) == 4)
        run_step_vec<T, 8, NORM, MAXP, G1, CL, RB>(a, d, st, item_base, s_max, ptrs, ptab, sh.contiguous);
      break;
    case SK_VEC4:
      run_step_vec<T, 4, NORM, MAXP, G1, CL, RB>(a, d, st, item_base, s_max, ptrs, ptab, sh.contiguous);
      break;
    default:
      run_step<T, NORM, MAXP, G1, CL, RB>(a, d, st, item_base, s_max, ptrs, ptab);
  }
}

// Shared-memory layout of a block working on program `a`: step records,
// syndrome words, per-step maxima (float32), MAP assignments, then the
// staged tables (if any) and the arena (if in shared memory).
struct BlockSmem {
  StepDesc* steps;
  int2* plan;  // per step: x = kind | lt << 8 | per-syndrome << 16 | contiguous << 17 | solo << 18 |
               // block barrier << 19, y = items (fill_step_plan)
  void* ptrs;  // per syndrome and step: StepPtrs (operand and output bases)
  uint32_t* syn;
  uint32_t* max;
  uint32_t* asg;
  TcState* tc;           // tensor-core state (kernels with tensor-core steps)
  unsigned char* tbuf;   // tensor-core staging tiles, 1024-byte aligned
  size_t tail;  // first free byte (16-byte aligned)
};

template <bool NORM, bool MAXP>
__device__ __forceinline__ BlockSmem carve_smem(const KArgs& a, unsigned char* smem) {
  BlockSmem b;
  b.steps = reinterpret_cast<StepDesc*>(smem);
  size_t off = size_t(a.n_steps) * sizeof(StepDesc);
  b.plan = reinterpret_cast<int2*>(smem + off);
  off += size_t(a.n_steps) * sizeof(int2);
  b.ptrs = smem + off;
  off += size_t(a.G) * a.n_steps * 3 * sizeof(void*);
  b.syn = reinterpret_cast<uint32_t*>(smem + off);
  off += size_t(a.G) * a.syn_words * 4;
  b.max = reinterpret_cast<uint32_t*>(smem + off);
  if (NORM) off += size_t(a.G) * a.n_steps * 4;
  b.asg = reinterpret_cast<uint32_t*>(smem + off);
  if (MAXP) off += size_t(a.G) * a.var_words * 4;
  b.tc = nullptr;
  b.tbuf = nullptr;
  if (a.tc) {
    // staging tiles on a 1024-byte boundary (the swizzle atom), then the state
    const uintptr_t base = reinterpret_cast<uintptr_t>(smem + off);
    b.tbuf = reinterpret_cast<unsigned char*>((base + 1023) & ~uintptr_t(1023));
    b.tc = reinterpret_cast<TcState*>(b.tbuf + 4 * tc::kTileBytes);
    off += tc::kSmemBytes;
  }
  b.tail = (off + 15) & ~size_t(15);
  return b;
}

__device__ __forceinline__ void copy16(void* dst, const void* src, size_t bytes) {
  const int4* s = reinterpret_cast<const int4*>(src);
  int4* d = reinterpret_cast<int4*>(dst);
  const int n16 = int(bytes / 16);
  for (int i = threadIdx.x; i < n16; i += blockDim.x) d[i] = s[i];
}

// Each step's execution plan for this block size and group: its shape (kind
// and lanes per output), whether it runs syndrome by syndrome (a step that
// fills the block for one syndrome alone, in a block of several), and how
// many items (threads' worth) it takes, which also rotates the next member of
// its barrier group.  `ptab` is read for the output permutations (staged in
// shared memory where the launch staged its tables).  In a cluster, a first
// pass writes every step's cluster-wide and block-sized plans to `scratch`
// (2 x n_steps int2) and a second picks, per barrier group, whether it runs
// on the first block alone; the block barrier between the passes is inside.
// Otherwise one thread per step; the caller synchronises.
template <typename T, bool tensor_ok, bool CL, bool VS = false>
__device__ __forceinline__ void fill_step_plan(const KArgs& a, const StepDesc* steps, int2* plan,
                                               const PermTab& ptab, int2* scratch = nullptr) {
  const bool tensor = tensor_ok && a.tc != 0;
  // the plan of step d for a team of bd threads
  auto plan_of = [&](const StepDesc& d, int bd, bool vsplit) {
    const StepShape sh = step_shape<T>(d.lh, d.lfa, d.lfb, d.lk, a.lg, d.flags, tensor, bd, vsplit);
    const StepShape sh1 =
        a.G > 1 ? step_shape<T>(d.lh, d.lfa, d.lfb, d.lk, 0, d.flags, tensor, bd, vsplit) : sh;
    const bool per_syndrome = a.G > 1 && sh1.total_r >= bd;
    const StepShape& use = per_syndrome ? sh1 : sh;
    // does the output permutation map index bits 0 .. log2(VW)-1 to
    // themselves?  (it moves whole bits, so checking each bit suffices)
    int contiguous = 0;
    if ((use.kind == SK_VEC8 || use.kind == SK_VEC4 || use.kind == SK_VSPLIT) && d.perm_off >= 0) {
      const int lw = d.lh + d.lfa + d.lfb;
      const int lv = use.kind == SK_VEC8 ? 3 : 2;
      contiguous = 1;
      for (int b = 0; b < lv; ++b)
        if (perm_addr(ptab, d.perm_off, 1 << b, lw) != (1 << b)) contiguous = 0;
    }
    return make_int2(use.kind | (use.lt << 8) | (int(per_syndrome) << 16) | (contiguous << 17),
                     per_syndrome ? bd : sh.total_r);
  };
  auto opt = [&](int st) { return a.step_opts ? int(a.step_opts[st]) : 0; };
  if (!CL) {
    for (int st = threadIdx.x; st < a.n_steps; st += blockDim.x)  // only kernels with the body share items
      plan[st] = plan_of(steps[st], blockDim.x, VS && a.vsplit != 0 && !(opt(st) & kOptNoShare));
    return;
  }
  int2* team_plan = scratch;
  int2* block_plan = scratch + a.n_steps;
  for (int st = threadIdx.x; st < a.n_steps; st += blockDim.x) {
    const bool share = !(opt(st) & kOptNoShare);
    team_plan[st] = plan_of(steps[st], team_size<CL>(), share);
    block_plan[st] = plan_of(steps[st], blockDim.x, share);
  }
  __syncthreads();
  // k summed by one lane of a step planned as pl
  auto k_per_lane = [](const StepDesc& d, int2 pl) {
    const int kind = pl.x & 0xff, lt = (pl.x >> 8) & 0xff;
    return (kind == SK_SPLITK || kind == SK_VSPLIT) ? (1 << d.lk) >> lt : (1 << d.lk);
  };
  // a barrier group (steps s0..s1) whose items all fit the first block runs
  // there alone (block-sized plans), unless that would lengthen a lane's run
  // of k beyond max(8, its run on the whole cluster)
  auto solo_group = [&](int s0, int s1) {
    int items = 0;
    for (int s = s0; s <= s1; ++s) {
      if (opt(s) & kOptNoSolo) return false;
      const int kb = k_per_lane(steps[s], block_plan[s]), kt = k_per_lane(steps[s], team_plan[s]);
      if (!(opt(s) & kOptSoloAlways) && kb > (kt > 8 ? kt : 8)) return false;
      items += block_plan[s].y;
    }
    return items <= int(blockDim.x);  // always required: the items live on the first block
  };
  auto group_end = [&](int s) {
    while (s + 1 < a.n_steps && !(steps[s].flags & kStepSync)) ++s;
    return s;
  };
  for (int st = threadIdx.x; st < a.n_steps; st += blockDim.x) {
    int g0 = st;
    while (g0 > 0 && !(steps[g0 - 1].flags & kStepSync)) --g0;
    const int g1 = group_end(st);
    const bool solo = solo_group(g0, g1);
    int2 pl = solo ? block_plan[st] : team_plan[st];
    if (solo) {
      pl.x |= 1 << 18;
      // the group's end needs only a block barrier when the next group (or,
      // after the last, the epilogue) also runs on the first block alone
      if (st == g1 && (g1 + 1 == a.n_steps || solo_group(g1 + 1, group_end(g1 + 1)))) pl.x |= 1 << 19;
    }
    plan[st] = pl;
  }
}

// One group of up to G syndromes (rows base .. base+G-1 below nrows) through
// the whole program: load the syndrome words, run every step, back-track
// (MAP), then the epilogue.  Ends with a block barrier.
template <typename T, bool NORM, bool MAXP, bool TENSOR, bool CL, bool VS, bool RB = false>
__device__ void contract_group(const KArgs& a, int64_t base, int64_t nrows, const BlockSmem& sm,
                               const Arena<T>& arena,
                               const T* consts, const PermTab& ptab) {
  const StepDesc* s_steps = sm.steps;
  uint32_t* s_syn = sm.syn;
  uint32_t* s_max = sm.max;
  StepPtrs<T>* s_ptrs = static_cast<StepPtrs<T>*>(sm.ptrs);
  for (int i = threadIdx.x; i < a.G * a.syn_words; i += blockDim.x) {
    const int g = i / a.syn_words, w = i - g * a.syn_words;
    const int64_t r = base + g;
    uint32_t word = 0;
    if (r < nrows) {
      const int64_t row = a.list ? int64_t(a.list[r]) : r + a.row_offset;
      const uint8_t* p = a.syn + row * a.syn_bytes;
      for (int b = 0; b < 4; ++b) {
        const int byte = 4 * w + b;
        if (byte < a.syn_bytes) word |= uint32_t(p[byte]) << (8 * b);
      }
    }
    s_syn[i] = word;
  }
  // the step maxima (in a cluster: the first block's, which every block
  // updates and reads) start at zero before any block's step runs
  if (NORM && (!CL || cluster_rank() == 0))
    for (int i = threadIdx.x; i < a.G * a.n_steps; i += blockDim.x) s_max[i] = 0u;
  team_sync<CL>();
  fill_step_ptrs<T>(a, s_steps, s_syn, arena, consts, s_ptrs);
  __syncthreads();
  int item_base = 0;
  for (int st = 0; st < a.n_steps; ++st) {
    const StepDesc& d = s_steps[st];
    const int2 pl = sm.plan[st];
    StepShape sh;
    sh.kind = pl.x & 0xff;
    sh.lt = (pl.x >> 8) & 0xff;
    sh.contiguous = ((pl.x >> 17) & 1) != 0;
    sh.total_r = pl.y;
    const bool per_syndrome = (pl.x >> 16) & 1;
    const int items = pl.y;
    if (CL && ((pl.x >> 18) & 1)) {
      // a small group on the cluster's first block alone, planned for the
      // block (the other blocks go on to the next cluster barrier)
      if (cluster_rank() == 0 && rotated(threadIdx.x & ~31, item_base, blockDim.x) < items)
        dispatch_step<T, NORM, MAXP, true, TENSOR, false, true>(a, d, sh, st, item_base, s_max, s_ptrs, ptab, sm.tc,
                                                                sm.tbuf);
      if (d.flags & kStepSync) {
        if ((pl.x >> 19) & 1) {
          if (cluster_rank() == 0) __syncthreads();
        } else {
          team_sync<CL>();
        }
        item_base = 0;
      } else {
        item_base += items;
      }
      continue;
    }
    // first virtual thread of this warp (steps of a barrier group start on
    // different warps); a warp past the step's items goes to the barrier
    const int vt_warp = rotated(team_tid<CL>() & ~31, item_base, team_size<CL>());
    if (vt_warp < items) {
      if (a.G == 1) {
        dispatch_step<T, NORM, MAXP, true, TENSOR, CL, VS, RB>(a, d, sh, st, item_base, s_max, s_ptrs, ptab, sm.tc,
                                                           sm.tbuf);
      } else if (per_syndrome) {
        // the block's syndromes one after another with hoisted invariants
        for (int g = 0; g < a.G; ++g)
          dispatch_step<T, NORM, MAXP, true, TENSOR, CL, VS, RB>(a, d, sh, st, item_base, s_max + g * a.n_steps,
                                                             s_ptrs + g * a.n_steps, ptab, sm.tc, sm.tbuf);
      } else {
        dispatch_step<T, NORM, MAXP, false, TENSOR, CL, VS, RB>(a, d, sh, st, item_base, s_max, s_ptrs, ptab, sm.tc,
                                                            sm.tbuf);
      }
    }
    if (d.flags & kStepSync) {
      team_sync<CL>();
      item_base = 0;
    } else {
      item_base += items;
    }
  }
  if constexpr (MAXP) {
    backtrack<T>(a, s_steps, s_syn, sm.asg, arena, consts, base, nrows);
    __syncthreads();
  }
  // epilogue: log-marginals, first argmax (Julia findmax order), recheck flag
  if (a.G == 1) {
    // one syndrome: the team's first warp, a lane per class (and per step
    // for the normalisers' exponents)
    if (team_tid<CL>() < 32 && base < nrows) {
      const int lane = threadIdx.x & 31;
      const int64_t row = a.list ? int64_t(a.list[base]) : base + a.row_offset;
      const T* rv = s_ptrs[a.n_steps - 1].out;
      double lsc = 0.0;
      if (NORM) {
        int e_sum = 0;
        for (int st = lane; st < a.n_steps - 1; st += 32) {
          int ee;
          norm_factor(s_max[st], &ee);
          e_sum += ee;
        }
        for (int o = 16; o > 0; o >>= 1) e_sum += __shfl_xor_sync(0xffffffffu, e_sum, o);
        lsc = double(e_sum) * 0.69314718055994530942;
      }
      // per lane: the best and second-best of its classes (lane, lane + 32,
      // ...) in class order; a lane without classes holds index INT_MAX
      double lb = -INFINITY, ls = -INFINITY;
      int li = lane < a.n_classes ? lane : INT_MAX;
      for (int c = lane; c < a.n_classes; c += 32) {
        const double v = double(rv[c]);
        const double lp = v > 0.0 ? log(v) + lsc : -INFINITY;
        if (a.logp_out) a.logp_out[row * a.n_classes + c] = lp;
        if (lp > lb) {
          ls = lb;
          lb = lp;
          li = c;
        } else if (lp > ls) {
          ls = lp;
        }
      }
      // the first maximum over the lanes (equal values: the lower class)
      double best = lb;
      int bc = li;
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bc, o);
        if (ob > best || (ob == best && oi < bc)) {
          best = ob;
          bc = oi;
        }
      }
      // the largest value of every other class
      double second = li == bc ? ls : lb;
      for (int o = 16; o > 0; o >>= 1) second = fmax(second, __shfl_xor_sync(0xffffffffu, second, o));
      if (lane == 0) {
        if (a.class_out) a.class_out[row] = bc;
        if (a.err_out) a.err_out[row] = a.err_bound;
        if (a.recheck_margin >= 0.0) {
          const double margin = best - second;
          if (!(margin >= a.recheck_margin) || best == -INFINITY) {
            const int slot = atomicAdd(a.recheck_count, 1);
            a.recheck_list[slot] = int32_t(row);
          }
        }
      }
    }
  } else
  for (int g = team_tid<CL>(); g < a.G; g += team_size<CL>()) {
    const int64_t r = base + g;
    if (r >= nrows) continue;
    const int64_t row = a.list ? int64_t(a.list[r]) : r + a.row_offset;
    const T* rv = s_ptrs[g * a.n_steps + a.n_steps - 1].out;
    double lsc = 0.0;
    if (NORM) {
      for (int st = 0; st < a.n_steps - 1; ++st) {
        int ee;
        norm_factor(s_max[g * a.n_steps + st], &ee);
        lsc += double(ee);
      }
      lsc *= 0.69314718055994530942;
    }
    double best = -INFINITY, second = -INFINITY;
    int bc = 0;
    for (int c = 0; c < a.n_classes; ++c) {
      const double v = double(rv[c]);
      const double lp = v > 0.0 ? log(v) + lsc : -INFINITY;
      if (a.logp_out) a.logp_out[row * a.n_classes + c] = lp;
      if (lp > best) {
        second = best;
        best = lp;
        bc = c;
      } else if (lp > second) {
        second = lp;
      }
    }
    if (a.class_out) a.class_out[row] = bc;
    if (a.err_out) a.err_out[row] = a.err_bound;
    if (a.recheck_margin >= 0.0) {
      const double margin = best - second;
      if (!(margin >= a.recheck_margin) || best == -INFINITY) {
        const int slot = atomicAdd(a.recheck_count, 1);
        a.recheck_list[slot] = int32_t(row);
      }
    }
  }
  team_sync<CL>();
}

// Stages the program's tables (if requested) after the fixed layout; returns
// the constants, the permutation tables and the shared arena pointer.
// The mbarrier the table copies of stage_tables complete on (one per block).
__shared__ uint64_t s_stage_bar;

// Waits (bounded) for the bulk copies stage_tables issued with wait = false.
__device__ __forceinline__ void stage_tables_wait(const KArgs& a) {
  if (!a.tables_smem) return;
  if (!tc::mbar_wait(&s_stage_bar, 0)) {
    // the copies never completed (not expected): the results are flagged as
    // invalid; the block still runs to its end, so no barrier waits for it
    if (a.tc_err) *static_cast<volatile int32_t*>(a.tc_err) = 2;
  }
}

template <typename T>
__device__ __forceinline__ void stage_tables(const KArgs& a, unsigned char* smem, size_t* off, const T** consts,
                                             PermTab* ptab, bool wait = true) {
  *consts = reinterpret_cast<const T*>(a.consts);
  *ptab = PermTab{a.perm, false};
  if (!a.tables_smem) return;
  T* s_consts = reinterpret_cast<T*>(smem + *off);
  const size_t const_bytes = size_t(a.n_consts) * sizeof(T);
  *off += (const_bytes + 15) & ~size_t(15);
  void* s_perm = smem + *off;
  const size_t perm_bytes = size_t(a.n_perm) * (a.perm16 ? 2 : 4);
  *off += (perm_bytes + 15) & ~size_t(15);
  const void* perm_src = a.perm16 ? static_cast<const void*>(a.perm16) : static_cast<const void*>(a.perm);
  // the 16-byte multiples by bulk asynchronous copies (one instruction each,
  // issued by thread 0, completing on one mbarrier) instead of a load and a
  // store per thread and 16 bytes; the few bytes past them by plain loads
  uint64_t* const s_bar = &s_stage_bar;
  const uint32_t m0 = uint32_t(const_bytes & ~size_t(15)), m1 = uint32_t(perm_bytes & ~size_t(15));
  if (threadIdx.x == 0) {
    tc::mbar_init(s_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n\tfence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(s_bar)),
                 "r"(m0 + m1)
                 : "memory");
    if (m0)
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                       tc::smem_u32(s_consts)),
                   "l"(a.consts), "r"(m0), "r"(tc::smem_u32(s_bar))
                   : "memory");
    if (m1)
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                       tc::smem_u32(s_perm)),
                   "l"(perm_src), "r"(m1), "r"(tc::smem_u32(s_bar))
                   : "memory");
  }
  for (int i = threadIdx.x; i < int(const_bytes - m0); i += blockDim.x)
    reinterpret_cast<unsigned char*>(s_consts)[m0 + i] = static_cast<const unsigned char*>(a.consts)[m0 + i];
  for (int i = threadIdx.x; i < int(perm_bytes - m1); i += blockDim.x)
    static_cast<unsigned char*>(s_perm)[m1 + i] = static_cast<const unsigned char*>(perm_src)[m1 + i];
  if (wait) stage_tables_wait(a);
  *consts = s_consts;
  *ptab = PermTab{s_perm, a.perm16 != nullptr};
}

// The block's arenas: all in shared memory (smem_tail) or all in global
// memory, or -- with a.arena_small set -- the small-tensor pools in shared
// memory and the big-tensor pools in global memory.
template <typename T>
__device__ __forceinline__ Arena<T> block_arena(const KArgs& a, unsigned char* smem_tail, void* global) {
  T* sm = reinterpret_cast<T*>(smem_tail);
  if (a.arena_small > 0) {
    const int64_t big = a.arena_elems - a.arena_small;
    T* gb = reinterpret_cast<T*>(global) + int64_t(blockIdx.x) * a.G * big;
    return Arena<T>{sm, gb - a.arena_small, int32_t(a.arena_small), int32_t(a.arena_small), int32_t(big)};
  }
  T* base = global ? reinterpret_cast<T*>(global) + int64_t(blockIdx.x) * a.G * a.arena_elems : sm;
  return Arena<T>{base, base, INT32_MAX, int32_t(a.arena_elems), int32_t(a.arena_elems)};
}

// float64 blocks, and blocks running tensor-core steps, are capped at 512
// threads, which leaves them 128 registers
// VS: the kernel has the SK_VSPLIT step body (launches with KArgs::vsplit
// plan it); the float32 kernel without it is kept for launches that do not,
// its 64 registers a thread being the tighter budget.
template <typename T, bool NORM, bool MAXP, bool TENSOR, bool VS = (sizeof(T) == 8), bool RB = false>
__global__ void __launch_bounds__(sizeof(T) == 8 || TENSOR ? 512 : 1024) tn_contract_kernel(KArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  // a dependent launch (the recheck's clusters) may be scheduled once every
  // block has started; it waits for this grid before reading what it writes
  asm volatile("griddepcontrol.launch_dependents;");
  const BlockSmem sm = carve_smem<NORM, MAXP>(a, smem);
  size_t off = sm.tail;
  const T* consts;
  PermTab ptab;
  stage_tables<T>(a, smem, &off, &consts, &ptab);
  const Arena<T> arena = block_arena<T>(a, smem + off, a.arena_global);
  copy16(sm.steps, a.steps, size_t(a.n_steps) * sizeof(StepDesc));
  __syncthreads();
  constexpr bool kTensor = TENSOR && std::is_same<T, float>::value && NORM && !MAXP;
  fill_step_plan<T, kTensor, false, VS>(a, sm.steps, sm.plan, ptab);
  const bool tensor = kTensor && a.tc;
  if (tensor) {
    if (threadIdx.x == 0) {
      tc::mbar_init(&sm.tc->bar, 1);
      sm.tc->phase = 0;
      sm.tc->abort = 0;
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if ((threadIdx.x >> 5) == 0) tc::alloc(&sm.tc->tmem, tc::kCols);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
  }
  const int64_t nrows = a.list ? int64_t(*a.list_count) : a.n;
  for (int64_t base = int64_t(blockIdx.x) * a.G; base < nrows; base += int64_t(gridDim.x) * a.G)
    contract_group<T, NORM, MAXP, TENSOR, false, VS, RB>(a, base, nrows, sm, arena, consts, ptab);
  if (tensor) {
    tc::fence_before();
    __syncthreads();
    // after a wait that gave up, the MMAs still in flight finish first (bounded)
    if (sm.tc->abort && threadIdx.x == 0) tc::mbar_wait(&sm.tc->bar, sm.tc->phase);
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) {
      tc::fence_after();
      tc::dealloc(sm.tc->tmem, tc::kCols);
    }
  }
}

// One syndrome per thread-block cluster: the latency form for a few rows
// (the plain float64 decode of single syndromes, the recheck of the rows
// inside the float32 bound).  Every block of the cluster copies the step
// records, plans and tables into its own shared memory; the cluster's
// threads share each step's work items (rank-major numbering), the arena is
// the cluster's slice of global memory, and the per-step maxima live in the
// first block's shared memory, which the others update and read through
// distributed shared memory.  Steps of a barrier group are separated by
// cluster barriers (release/acquire at cluster scope).  Rows are taken
// cluster by cluster in a grid-stride loop.
template <typename T, bool NORM>
__global__ void __launch_bounds__(512) tn_contract_cluster_kernel(KArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  BlockSmem sm = carve_smem<NORM, false>(a, smem);
  size_t off = sm.tail;
  const T* consts;
  PermTab ptab;
  // the table copies run while the step records are copied
  stage_tables<T>(a, smem, &off, &consts, &ptab, false);
  copy16(sm.steps, a.steps, size_t(a.n_steps) * sizeof(StepDesc));
  stage_tables_wait(a);
  __syncthreads();
  fill_step_plan<T, false, true>(a, sm.steps, sm.plan, ptab, static_cast<int2*>(sm.ptrs));
  // everything above reads only the program (steps, tables); a launch that
  // may start while the preceding kernel of its stream finishes (programmatic
  // dependent launch) waits for that kernel here, before the rows, their
  // count and the outputs it may have written
  asm volatile("griddepcontrol.wait;" ::: "memory");
  // a cluster without rows (the same answer for all its blocks) leaves now:
  // it has reached no cluster barrier and no other block's memory
  if (int64_t(cluster_id()) * a.G >= (a.list ? int64_t(*a.list_count) : a.n)) return;
  if (NORM) sm.max = cluster_map(sm.max, 0);
  const int64_t nrows = a.list ? int64_t(*a.list_count) : a.n;
  const int64_t cid = cluster_id(), ncl = cluster_count();
  Arena<T> arena;
  if (a.arena_small > 0) {
    // the small tensors in the first block's shared memory (reached by every
    // block through distributed shared memory), the large ones in the
    // cluster's slice of global memory
    const int64_t big = a.arena_elems - a.arena_small;
    T* slice = reinterpret_cast<T*>(a.arena_global) + cid * big;
    T* small = cluster_map(reinterpret_cast<T*>(smem + off), 0);
    arena = Arena<T>{small, slice - a.arena_small, int32_t(a.arena_small), int32_t(a.arena_small), int32_t(big)};
  } else {
    T* slice = reinterpret_cast<T*>(a.arena_global) + cid * int64_t(a.G) * a.arena_elems;
    arena = Arena<T>{slice, slice, INT32_MAX, int32_t(a.arena_elems), int32_t(a.arena_elems)};
  }
  for (int64_t base = cid * a.G; base < nrows; base += ncl * a.G)
    contract_group<T, NORM, false, false, true, true>(a, base, nrows, sm, arena, consts, ptab);
  // the first block's shared memory stays until no block of the cluster
  // can still reach it
  team_sync<true>();
}

// Several programs in one persistent launch.  Work units (program, first
// row) of the current batch are claimed from a device counter; each unit's
// program descriptor and steps are copied into shared memory, then one group
// of its rows is contracted.  With `list_mode` every program instead
// contracts the rows of its own device-side list (the recheck), block
// by block in a grid-stride loop.
template <typename T, bool NORM>
__global__ void __launch_bounds__(kMultiThreads) tn_contract_multi_kernel(MultiArgs m) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ __align__(16) KArgs s_ka;
  __shared__ int64_t s_unit;
  const int32_t b = *m.batch;
  const KArgs* progs = m.progs;
  T* gslice = m.arena_global ? reinterpret_cast<T*>(m.arena_global) + int64_t(blockIdx.x) * m.arena_per_block
                             : nullptr;
  auto run_unit = [&](int32_t prog, int64_t base, int64_t nrows, bool first) {
    if (first) {
      copy16(&s_ka, progs + prog, sizeof(KArgs));
      __syncthreads();
    }
    const KArgs& a = s_ka;
    const BlockSmem sm = carve_smem<NORM, false>(a, smem);
    if (first) {
      copy16(sm.steps, a.steps, size_t(a.n_steps) * sizeof(StepDesc));
      __syncthreads();
      fill_step_plan<T, false, false>(a, sm.steps, sm.plan, PermTab{a.perm, false});
      __syncthreads();
    }
    T* abase = a.arena_global ? gslice : reinterpret_cast<T*>(smem + sm.tail);
    const Arena<T> arena{abase, abase, INT32_MAX, int32_t(a.arena_elems), int32_t(a.arena_elems)};
    contract_group<T, NORM, false, false, false, false>(a, base, nrows, sm, arena, reinterpret_cast<const T*>(a.consts),
                                          PermTab{a.perm, false});
  };
  if (m.list_mode) {
    for (int32_t prog = 0; prog < m.n_progs; ++prog) {
      __syncthreads();
      copy16(&s_ka, progs + prog, sizeof(KArgs));
      __syncthreads();
      const int64_t nrows = int64_t(*s_ka.list_count);
      if (int64_t(blockIdx.x) * s_ka.G >= nrows) continue;  // block-uniform
      const BlockSmem sm = carve_smem<NORM, false>(s_ka, smem);
      copy16(sm.steps, s_ka.steps, size_t(s_ka.n_steps) * sizeof(StepDesc));
      __syncthreads();
      fill_step_plan<T, false, false>(s_ka, sm.steps, sm.plan, PermTab{s_ka.perm, false});
      __syncthreads();
      for (int64_t base = int64_t(blockIdx.x) * s_ka.G; base < nrows; base += int64_t(gridDim.x) * s_ka.G)
        run_unit(prog, base, nrows, false);
    }
    return;
  }
  if (b < 0 || b >= m.n_batches) return;
  const int64_t u0 = m.unit_offsets[b], u1 = m.unit_offsets[b + 1];
  int32_t cur = -1;
  for (;;) {
    if (threadIdx.x == 0) s_unit = u0 + atomicAdd(m.next_unit, 1);
    __syncthreads();
    const int64_t u = s_unit;
    if (u >= u1) break;
    const MultiUnit w = m.units[u];
    const int64_t nrows = m.batch_rows[int64_t(b) * m.n_progs + w.prog];
    run_unit(w.prog, w.first_row, nrows, w.prog != cur);
    cur = w.prog;
  }
}

__global__ void multi_advance_kernel(int32_t* batch, int32_t* next_unit, int32_t* counts, int32_t n_progs) {
  const int i = threadIdx.x;
  if (i == 0) {
    *batch += 1;
    *next_unit = 0;
  }
  for (int p = i; p < n_progs; p += blockDim.x) counts[p] = 0;
}

}  // namespace

size_t contract_smem_bytes(int precision, int32_t n_steps, int32_t syn_words, int G,
                           int64_t arena_elems, bool arena_in_smem, int32_t var_words, size_t table_bytes,
                           bool tensor) {
  const bool norm = precision != 0;  // float32 and double-float keep per-step maxima
  size_t off = size_t(n_steps) * (sizeof(StepDesc) + 8) + size_t(G) * n_steps * 3 * sizeof(void*) +
               size_t(G) * syn_words * 4;
  if (norm) off += size_t(G) * n_steps * 4;
  off += size_t(G) * var_words * 4;
  if (tensor) off += tc::kSmemBytes;
  off = (off + 15) & ~size_t(15);
  off += table_bytes;
  if (arena_in_smem) off += size_t(G) * size_t(arena_elems) * (precision == 1 ? 4 : 8);
  return off;
}

size_t contract_table_bytes(int precision, int64_t n_consts, int64_t n_perm, bool perm16) {
  const size_t c = (size_t(n_consts) * (precision == 1 ? 4 : 8) + 15) & ~size_t(15);
  const size_t p = (size_t(n_perm) * (perm16 ? 2 : 4) + 15) & ~size_t(15);
  return c + p;
}

size_t contract_smem_limit(int device) {
  int v = 0;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess) return 48 * 1024;
  return size_t(v);
}

// Raises a kernel's dynamic shared-memory limit to at least smem. The limit
// only ever grows (to the largest any program or program set asked for), so a
// launch prepared earlier -- one captured in a CUDA graph among them -- stays
// valid after another program's set-up. The kernels of one family share a
// function type, so the limit is kept per kernel address (and device).
template <typename K>
cudaError_t grow_smem_limit(K kernel, size_t smem) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> granted;  // per kernel and device
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  size_t& g = granted[{reinterpret_cast<const void*>(kernel), dev}];
  if (smem <= g) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e == cudaSuccess) g = smem;
  return e;
}

template <typename K>
int occupancy_of(K kernel, int threads, size_t smem) {
  int blocks = 0;
  if (grow_smem_limit(kernel, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, threads, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return blocks;
}

int contract_occupancy(int precision, int threads, size_t smem, bool map_mode, bool tensor) {
  if (precision == 1) {
    if (map_mode) return occupancy_of(tn_contract_kernel<float, true, true, false>, threads, smem);
    return tensor ? occupancy_of(tn_contract_kernel<float, true, false, true>, threads, smem)
                  : occupancy_of(tn_contract_kernel<float, true, false, false>, threads, smem);  // same registers with VS
  }
  if (precision == 2) return map_mode ? 0 : occupancy_of(tn_contract_kernel<dfloat, true, false, false>, threads, smem);
  return map_mode ? occupancy_of(tn_contract_kernel<double, false, true, false>, threads, smem)
                  : occupancy_of(tn_contract_kernel<double, false, false, false>, threads, smem);
}

template <typename K>
cudaError_t launch_with(K kernel, const KArgs& a, int grid, int threads, size_t smem, cudaStream_t stream) {
  cudaError_t e = grow_smem_limit(kernel, smem);
  if (e != cudaSuccess) return e;
  kernel<<<grid, threads, smem, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t contract_launch(int precision, const KArgs& a, int grid, int threads, size_t smem,
                            cudaStream_t stream) {
  if (precision == 1) {
    if (a.map_mode) return launch_with(tn_contract_kernel<float, true, true, false>, a, grid, threads, smem, stream);
    if (a.round_bf16)  // the bf16 study: SIMT steps only, vsplit as planned
      return launch_with(tn_contract_kernel<float, true, false, false, true, true>, a, grid, threads, smem, stream);
    if (a.tc) return launch_with(tn_contract_kernel<float, true, false, true>, a, grid, threads, smem, stream);
    return a.vsplit ? launch_with(tn_contract_kernel<float, true, false, false, true>, a, grid, threads, smem, stream)
                    : launch_with(tn_contract_kernel<float, true, false, false>, a, grid, threads, smem, stream);
  }
  if (precision == 2) {
    if (a.map_mode) return cudaErrorInvalidValue;  // max-product runs in float32 or float64
    return launch_with(tn_contract_kernel<dfloat, true, false, false>, a, grid, threads, smem, stream);
  }
  return a.map_mode ? launch_with(tn_contract_kernel<double, false, true, false>, a, grid, threads, smem, stream)
                    : launch_with(tn_contract_kernel<double, false, false, false>, a, grid, threads, smem, stream);
}

template <typename K>
cudaError_t cluster_config(K kernel, int csize, int threads, size_t smem) {
  cudaError_t e = grow_smem_limit(kernel, smem);
  if (e != cudaSuccess || csize <= 8) return e;
  // clusters above the portable 8 blocks: allowed once per kernel
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, bool> allowed;  // per kernel and device
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lk(mu);
  bool& ok = allowed[{reinterpret_cast<const void*>(kernel), dev}];
  if (!ok) {
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    ok = e == cudaSuccess;
  }
  return e;
}

template <typename K>
int cluster_capacity_of(K kernel, int csize, int threads, size_t smem) {
  if (cluster_config(kernel, csize, threads, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(csize);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, kernel, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

template <typename K>
cudaError_t cluster_launch_with(K kernel, const KArgs& a, int clusters, int csize, int threads, size_t smem,
                                cudaStream_t stream, bool configure) {
  if (configure) {
    cudaError_t e = cluster_config(kernel, csize, threads, smem);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(unsigned(clusters) * unsigned(csize));
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = csize;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (configure) {
    // a standalone launch (not one captured into a graph) may begin its
    // prologue while the stream's preceding kernel finishes; the kernel
    // waits for that kernel (griddepcontrol.wait) before touching its data
    at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.numAttrs = 2;
  }
  return cudaLaunchKernelEx(&cfg, kernel, a);
}

int contract_cluster_capacity(int precision, int csize, int threads, size_t smem) {
  if (precision == 2) return cluster_capacity_of(tn_contract_cluster_kernel<dfloat, true>, csize, threads, smem);
  if (precision == 0) return cluster_capacity_of(tn_contract_cluster_kernel<double, false>, csize, threads, smem);
  return 0;
}

cudaError_t contract_cluster_launch(int precision, const KArgs& a, int clusters, int csize, int threads, size_t smem,
                                    cudaStream_t stream, bool configure) {
  if (a.map_mode || a.G != 1) return cudaErrorInvalidValue;
  if (precision == 2)
    return cluster_launch_with(tn_contract_cluster_kernel<dfloat, true>, a, clusters, csize, threads, smem, stream,
                               configure);
  if (precision == 0)
    return cluster_launch_with(tn_contract_cluster_kernel<double, false>, a, clusters, csize, threads, smem, stream,
                               configure);
  return cudaErrorInvalidValue;
}

cudaError_t contract_cluster_configure(int precision, int csize, int threads, size_t smem) {
  if (precision == 2) return cluster_config(tn_contract_cluster_kernel<dfloat, true>, csize, threads, smem);
  if (precision == 0) return cluster_config(tn_contract_cluster_kernel<double, false>, csize, threads, smem);
  return cudaErrorInvalidValue;
}

// Sets the shared-memory limit (outside any stream capture) and returns the
// resident blocks per SM.
int contract_multi_occupancy(int precision, int threads, size_t smem) {
  if (precision == 2) return occupancy_of(tn_contract_multi_kernel<dfloat, true>, threads, smem);
  return precision == 1 ? occupancy_of(tn_contract_multi_kernel<float, true>, threads, smem)
                        : occupancy_of(tn_contract_multi_kernel<double, false>, threads, smem);
}

// No attribute calls here: the launch may be captured into a CUDA graph.
cudaError_t contract_multi_launch(int precision, const MultiArgs& m, int grid, int threads, size_t smem,
                                  cudaStream_t stream) {
  if (precision == 1)
    tn_contract_multi_kernel<float, true><<<grid, threads, smem, stream>>>(m);
  else if (precision == 2)
    tn_contract_multi_kernel<dfloat, true><<<grid, threads, smem, stream>>>(m);
  else
    tn_contract_multi_kernel<double, false><<<grid, threads, smem, stream>>>(m);
  return cudaGetLastError();
}

cudaError_t contract_multi_advance(int32_t* batch, int32_t* next_unit, int32_t* counts, int32_t n_progs,
                                   cudaStream_t stream) {
  multi_advance_kernel<<<1, 256, 0, stream>>>(batch, next_unit, counts, n_progs);
  return cudaGetLastError();
}

}  // namespace tqec
