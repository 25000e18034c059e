// umma_gemm.cu -- the surrogate's hidden-layer GEMM on the 5th-generation
// tensor cores: D[M, N] = relu(A[M, K] * B[N, K]^T + bias) in bf16, float32
// accumulation in tensor memory.
//
// One CTA computes a 128 x 256 tile.  Warp 0 streams 128x64 A and 256x64 B
// tiles (bf16, K-major, 128-byte swizzle) into a 4-stage shared-memory ring
// with TMA; warp 1's elected thread issues tcgen05.mma (M=128, N=256, K=16,
// four per stage) into a 256-column TMEM accumulator and frees each stage
// with tcgen05.commit; warps 4-7 wait for the accumulator, read it back with
// tcgen05.ld (one TMEM lane quadrant per warp), add the bias, apply ReLU and
// store bf16.  Every mbarrier wait is bounded: on timeout the kernel records
// an error flag, stops issuing work and still releases its TMEM.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "mlp.cuh"

namespace tqec {
namespace {

constexpr int UM = 128, UN = 256, UK = 64;
constexpr int A_BYTES = UM * UK * 2;  // 16 KB
constexpr int B_BYTES = UN * UK * 2;  // 32 KB
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr uint32_t TMEM_COLS = 256;
constexpr int UMMA_THREADS = 256;
constexpr uint32_t WAIT_LIMIT = 1u << 24;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait on a phase; false (and the error flag set) on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err) {
  for (uint32_t i = 0; i < WAIT_LIMIT; ++i)
    if (mbar_test(bar, parity)) return true;
  atomicExch(err, 1);
  return false;
}

__device__ __forceinline__ void tma_load_2d(const CUtensorMap* map, uint64_t* bar, void* dst, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_addr(bar)), "r"(x), "r"(y)
      : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms
// 1024 bytes apart.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= uint64_t((saddr >> 4) & 0x3FFFu);
  d |= uint64_t(1) << 16;             // leading byte offset (unused for swizzled K-major)
  d |= uint64_t(1024 >> 4) << 32;     // stride byte offset
  d |= uint64_t(1) << 46;             // descriptor version
  d |= uint64_t(2) << 61;             // 128-byte swizzle
  return d;
}

// Instruction descriptor of kind::f16: bf16 A and B, float32 D, both K-major.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(UN >> 3) << 17) | (uint32_t(UM >> 4) << 24);

__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// STAGES-deep TMA ring; MINB blocks per SM (4 stages: one 193 KB block per
// SM; 2 stages: two 97 KB blocks, one's epilogue overlapping the other's
// main loop)
template <int STAGES, int MINB>
__global__ void __launch_bounds__(UMMA_THREADS, MINB)
    umma_gemm_relu_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                          int M, int N, int K, const float* __restrict__ bias, __nv_bfloat16* __restrict__ out,
                          int ldo, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // stage buffers on a 1024-byte boundary (the 128-byte swizzle atom)
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                         ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* acc_ready = empty + STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acc_ready + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * UM, n0 = blockIdx.x * UN;
  const int kblocks = K / UK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(acc_ready, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // TMA producer
    int issued = 0;
    for (int kb = 0; kb < kblocks; ++kb) {
      const int s = kb % STAGES;
      if (kb >= STAGES && !mbar_wait(&empty[s], uint32_t((kb / STAGES - 1) & 1), err)) {
        *abort_flag = 1;
        break;
      }
      if (*abort_flag) break;
      unsigned char* sa = smem + s * STAGE_BYTES;
      mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
      tma_load_2d(&map_a, &full[s], sa, kb * UK, m0);
      tma_load_2d(&map_b, &full[s], sa + A_BYTES, kb * UK, n0);
      issued = kb + 1;
    }
    // the copies still in flight land before the block exits (bounded)
    for (int kb = issued > STAGES ? issued - STAGES : 0; kb < issued; ++kb)
      mbar_wait(&full[kb % STAGES], uint32_t((kb / STAGES) & 1), err);
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    bool ok = true;
    for (int kb = 0; kb < kblocks && ok; ++kb) {
      const int s = kb % STAGES;
      if (!mbar_wait(&full[s], uint32_t((kb / STAGES) & 1), err)) {
        *abort_flag = 1;
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t sa = smem_addr(smem + s * STAGE_BYTES);
      const uint64_t da = sdesc(sa), db = sdesc(sa + A_BYTES);
#pragma unroll
      for (int kk = 0; kk < UK / 16; ++kk)  // advance 16 bf16 = 32 bytes along K inside the swizzle atom
        umma(tmem, da + uint64_t(kk * 2), db + uint64_t(kk * 2), (kb | kk) != 0 ? 1u : 0u);
      umma_commit(&empty[s]);
    }
    umma_commit(acc_ready);
  } else if (warp >= 4) {
    // epilogue: warp w reads TMEM lanes 32*(w%4) .. +31, one output row per thread
    const int q = warp & 3;
    const int row = m0 + q * 32 + lane;
    const bool waited = mbar_wait(acc_ready, 0u, err);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // tcgen05.ld is warp-collective: decide for the whole warp
    const bool go = __all_sync(0xffffffffu, waited && *abort_flag == 0);
    if (go) {
#pragma unroll 1
      for (int c = 0; c < UN / 32; ++c) {
        uint32_t r[32];
        tmem_ld32(tmem + (uint32_t(q * 32) << 16) + uint32_t(c * 32), r);
        const int col = n0 + c * 32;
        if (row < M && col < N) {
          __align__(16) __nv_bfloat16 v[32];
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const float x = __uint_as_float(r[j]) + bias[col + j];
            v[j] = __float2bfloat16(x > 0.f ? x : 0.f);
          }
          uint4* dst = reinterpret_cast<uint4*>(out + int64_t(row) * ldo + col);
          const uint4* src = reinterpret_cast<const uint4*>(v);
#pragma unroll
          for (int j = 0; j < 4; ++j) dst[j] = src[j];
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

bool make_map(CUtensorMap* map, const __nv_bfloat16* base, int rows, int cols, int ld, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {cuuint64_t(cols), cuuint64_t(rows)};
  const cuuint64_t strides[1] = {cuuint64_t(ld) * 2};
  const cuuint32_t box[2] = {cuuint32_t(UK), cuuint32_t(box_rows)};
  const cuuint32_t estr[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// ---- the whole surrogate forward in one persistent kernel ----------------
//
// Hidden width 512, three ReLU layers and a small output layer.  A CTA owns
// 128-row tiles in turn.  The layer input lives in shared memory as eight
// 128x64 bf16 k-tiles (128 KB, the 128-byte-swizzled K-major layout the MMA
// reads); the 512-wide float32 accumulator fills all of tensor memory (two
// 256-column halves).  Warp 0 streams 256x64 weight tiles through a 3-stage
// ring with TMA; warp 1 issues the MMAs of a layer once its input is ready
// and commits the accumulator; two groups of four epilogue warps (4-7 and
// 8-11: one TMEM lane quadrant per warp, one row per thread, the group's
// half of the 512 columns) write the layer-1 input from the packed syndrome
// bits, turn each accumulator into the next layer's bf16 input (bias, ReLU),
// and for the last hidden layer compute the output logits directly from
// tensor memory (the two halves' partial sums meet in shared memory).  No
// activation leaves the SM.  Every mbarrier wait is bounded; the epilogue
// groups' named barrier sits outside every conditional, so both groups
// always reach it.
constexpr int FM = 128, FH = 512, FNH = 256, FSTAGES = 3;
constexpr int FA_TILE = FM * UK * 2;           // 16 KB: 128 rows x 64 bf16
constexpr int FA_BYTES = (FH / UK) * FA_TILE;  // 128 KB: a layer input
constexpr int FB_STAGE = FNH * UK * 2;         // 32 KB: 256 weight rows x 64 bf16
constexpr uint32_t FTMEM_COLS = 512;
constexpr int FTHREADS = 384;
constexpr int FEPI = 256;  // epilogue threads (warps 4-11)
constexpr int FMAX_OUT = 16;
constexpr size_t FUSED_SMEM = size_t(FA_BYTES) + size_t(FSTAGES) * FB_STAGE + 256 + 1024;

struct FusedArgs {
  const uint8_t* syn;
  int sb, n_in;
  int64_t n;
  const float* bias[3];
  const __nv_bfloat16* w4;  // [n_out][512]
  const float* b4;
  int n_out, ldl;
  float* logits;
  int* err;
  // the gate, fused into the last epilogue when cls is set: the argmax class
  // and the softmax confidence of every row, and the rows below threshold
  // appended to list (count), exactly as gate_kernel computes them
  float threshold;
  int32_t* cls;
  float* conf;
  int32_t* list;
  int32_t* count;
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&v);
}

__global__ void __launch_bounds__(FTHREADS, 1)
    mlp_fused_kernel(const __grid_constant__ CUtensorMap w1, const __grid_constant__ CUtensorMap w2,
                     const __grid_constant__ CUtensorMap w3, const __grid_constant__ FusedArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                         ~uintptr_t(1023));
  unsigned char* sA = smem;
  unsigned char* sB = smem + FA_BYTES;
  uint64_t* full = reinterpret_cast<uint64_t*>(sB + FSTAGES * FB_STAGE);
  uint64_t* empty = full + FSTAGES;
  uint64_t* acc_ready = empty + FSTAGES;
  uint64_t* a_ready = acc_ready + 1;
  uint64_t* mma_done = a_ready + 1;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t ntiles = (a.n + FM - 1) / FM;

  if (threadIdx.x == 0) {
    for (int s = 0; s < FSTAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(acc_ready, 1);
    mbar_init(a_ready, FEPI);  // every epilogue thread
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                 "r"(FTMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0 && lane == 0) {
    // TMA producer: per tile, per layer, per 256-row half of the weights,
    // per 64-wide k slice
    uint32_t q = 0;
    bool ok = true;
    for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
      for (int L = 0; L < 3 && ok; ++L) {
        const CUtensorMap* map = L == 0 ? &w1 : (L == 1 ? &w2 : &w3);
        const int kbs = L == 0 ? 1 : FH / UK;
        for (int h = 0; h < 2 && ok; ++h) {
          for (int kb = 0; kb < kbs; ++kb) {
            const int s = int(q % FSTAGES);
            if (q >= uint32_t(FSTAGES) && !mbar_wait(&empty[s], uint32_t((q / FSTAGES - 1) & 1), a.err)) {
              *abort_flag = 1;
              ok = false;
              break;
            }
            if (*abort_flag) {
              ok = false;
              break;
            }
            mbar_arrive_expect_tx(&full[s], FB_STAGE);
            tma_load_2d(map, &full[s], sB + s * FB_STAGE, kb * UK, h * FNH);
            ++q;
          }
        }
      }
    }
    // the copies still in flight land before the block exits (bounded)
    for (uint32_t k = q > uint32_t(FSTAGES) ? q - FSTAGES : 0; k < q; ++k)
      mbar_wait(&full[k % FSTAGES], uint32_t((k / FSTAGES) & 1), a.err);
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    uint32_t q = 0, c = 0;
    bool ok = true;
    for (int64_t t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
      for (int L = 0; L < 3 && ok; ++L) {
        if (!mbar_wait(a_ready, c & 1u, a.err) || *abort_flag) {
          *abort_flag = 1;
          ok = false;
          break;
        }
        ++c;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int kbs = L == 0 ? 1 : FH / UK;
        for (int h = 0; h < 2 && ok; ++h) {
          for (int kb = 0; kb < kbs; ++kb) {
            const int s = int(q % FSTAGES);
            if (!mbar_wait(&full[s], uint32_t((q / FSTAGES) & 1), a.err)) {
              *abort_flag = 1;
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint64_t da = sdesc(smem_addr(sA + kb * FA_TILE)), db = sdesc(smem_addr(sB + s * FB_STAGE));
#pragma unroll
            for (int kk = 0; kk < UK / 16; ++kk)
              umma(tmem + uint32_t(h * FNH), da + uint64_t(kk * 2), db + uint64_t(kk * 2), (kb | kk) != 0 ? 1u : 0u);
            umma_commit(&empty[s]);
            ++q;
          }
        }
        if (ok) umma_commit(acc_ready);
      }
    }
    // every MMA issued has completed before the tensor memory is freed
    umma_commit(mma_done);
    mbar_wait(mma_done, 0u, a.err);
  } else if (warp >= 4) {
    // epilogue: TMEM lane quadrant qd, row r of the tile per thread; group
    // `half` owns columns [256 half, 256 half + 256) of every accumulator
    const int qd = warp & 3;
    const int half = (warp - 4) >> 2;
    const int r = qd * 32 + lane;
    float* partial = reinterpret_cast<float*>(sA);  // [128][FMAX_OUT], last layer only
    uint32_t c = 0;
    bool ok = true;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const int64_t row = t * FM + r;
      {
        // layer-1 input: the syndrome bits as bf16 0/1 in k-tile 0
        uint32_t bytes[8];
#pragma unroll
        for (int b = 0; b < 8; ++b) bytes[b] = (row < a.n && b < a.sb) ? uint32_t(a.syn[row * a.sb + b]) : 0u;
#pragma unroll
        for (int ch = 4 * half; ch < 4 * half + 4; ++ch) {
          uint32_t w[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int c0 = ch * 8 + 2 * j;
            const float v0 = c0 < a.n_in ? float((bytes[c0 >> 3] >> (c0 & 7)) & 1u) : 0.f;
            const float v1 = c0 + 1 < a.n_in ? float((bytes[(c0 + 1) >> 3] >> ((c0 + 1) & 7)) & 1u) : 0.f;
            w[j] = pack_bf16x2(v0, v1);
          }
          *reinterpret_cast<uint4*>(sA + r * 128 + ((ch ^ (r & 7)) << 4)) = make_uint4(w[0], w[1], w[2], w[3]);
        }
      }
      fence_proxy_async_smem();
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(a_ready);
      for (int L = 0; L < 3; ++L) {
        if (ok && !mbar_wait(acc_ready, c & 1u, a.err)) {
          *abort_flag = 1;
          ok = false;
        }
        ++c;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // tcgen05.ld is warp-collective: decide for the whole warp
        const bool go = __all_sync(0xffffffffu, ok && *abort_flag == 0);
        float lg[FMAX_OUT];
#pragma unroll
        for (int o = 0; o < FMAX_OUT; ++o) lg[o] = 0.f;
        if (go) {
          const float* bias = a.bias[L];
#pragma unroll 1
          for (int cc = half * (FH / 64); cc < (half + 1) * (FH / 64); ++cc) {
            uint32_t v[32];
            tmem_ld32(tmem + (uint32_t(qd * 32) << 16) + uint32_t(cc * 32), v);
            float x[32];
#pragma unroll
            for (int j = 0; j < 32; j += 4) {
              const float4 b = *reinterpret_cast<const float4*>(bias + cc * 32 + j);
              x[j] = fmaxf(__uint_as_float(v[j]) + b.x, 0.f);
              x[j + 1] = fmaxf(__uint_as_float(v[j + 1]) + b.y, 0.f);
              x[j + 2] = fmaxf(__uint_as_float(v[j + 2]) + b.z, 0.f);
              x[j + 3] = fmaxf(__uint_as_float(v[j + 3]) + b.w, 0.f);
            }
            if (L < 2) {
              // the next layer's input: bf16, k-tile cc/2, 16-byte chunks
              // (cc%2)*4 .. +3 of row r
              unsigned char* tile = sA + (cc >> 1) * FA_TILE + r * 128;
#pragma unroll
              for (int u = 0; u < 4; ++u) {
                const int chunk = (cc & 1) * 4 + u;
                *reinterpret_cast<uint4*>(tile + ((chunk ^ (r & 7)) << 4)) =
                    make_uint4(pack_bf16x2(x[8 * u], x[8 * u + 1]), pack_bf16x2(x[8 * u + 2], x[8 * u + 3]),
                               pack_bf16x2(x[8 * u + 4], x[8 * u + 5]), pack_bf16x2(x[8 * u + 6], x[8 * u + 7]));
              }
            } else {
              // output layer on the bf16-rounded activations
#pragma unroll
              for (int j = 0; j < 32; ++j) x[j] = __bfloat162float(__float2bfloat16(x[j]));
              for (int o = 0; o < a.n_out; ++o) {
                const __nv_bfloat16* wrow = a.w4 + o * FH + cc * 32;
                float s = 0.f;
#pragma unroll
                for (int j = 0; j < 32; j += 8) {
                  const uint4 wv = *reinterpret_cast<const uint4*>(wrow + j);
                  const __nv_bfloat162* w2 = reinterpret_cast<const __nv_bfloat162*>(&wv);
#pragma unroll
                  for (int u = 0; u < 4; ++u) {
                    const float2 wf = __bfloat1622float2(w2[u]);
                    s = fmaf(x[j + 2 * u], wf.x, s);
                    s = fmaf(x[j + 2 * u + 1], wf.y, s);
                  }
                }
                lg[o] += s;
              }
            }
          }
        }
        if (L < 2) {
          fence_proxy_async_smem();
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          mbar_arrive(a_ready);
        } else {
          // the last layer's input has been read by every MMA (acc_ready), so
          // its shared memory holds the second group's partial sums
          if (half == 1)
            for (int o = 0; o < a.n_out; ++o) partial[r * FMAX_OUT + o] = lg[o];
          asm volatile("bar.sync 1, %0;" ::"n"(FEPI) : "memory");
          if (half == 0 && go && row < a.n) {
            for (int o = 0; o < a.n_out; ++o) {
              lg[o] = lg[o] + partial[r * FMAX_OUT + o] + a.b4[o];
              a.logits[row * a.ldl + o] = lg[o];
            }
            if (a.cls) {
              // the gate on this row's logits (the same arithmetic as gate_kernel)
              float mx = lg[0];
              int bc = 0;
              for (int o = 1; o < a.n_out; ++o)
                if (lg[o] > mx) {
                  mx = lg[o];
                  bc = o;
                }
              float sum = 0.f;
              for (int o = 0; o < a.n_out; ++o) sum += __expf(lg[o] - mx);
              const float pr = 1.0f / sum;
              a.cls[row] = bc;
              if (a.conf) a.conf[row] = pr;
              if (a.list && !(pr >= a.threshold)) a.list[atomicAdd(a.count, 1)] = int32_t(row);
            }
          }
          // the next tile's layer-1 input overwrites that memory only after
          asm volatile("bar.sync 1, %0;" ::"n"(FEPI) : "memory");
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(FTMEM_COLS));
  }
}

}  // namespace

bool umma_gemm_supported(int M, int N, int K, int lda, int ldb, int ldo, const void* A, const void* B,
                         const void* out) {
  return M > 0 && N % UN == 0 && K % UK == 0 && K > 0 && lda % 8 == 0 && ldb % 8 == 0 && ldo % 8 == 0 &&
         (reinterpret_cast<uintptr_t>(A) % 16) == 0 && (reinterpret_cast<uintptr_t>(B) % 16) == 0 &&
         (reinterpret_cast<uintptr_t>(out) % 16) == 0 && encode_fn() != nullptr;
}

namespace {

template <int STAGES, int MINB>
cudaError_t launch_umma(const CUtensorMap& ma, const CUtensorMap& mb, int M, int N, int K, const float* bias,
                        __nv_bfloat16* out, int ldo, int* err, cudaStream_t st) {
  const size_t smem = size_t(STAGES) * STAGE_BYTES + 1024 + 256;
  auto kernel = umma_gemm_relu_kernel<STAGES, MINB>;
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) return e;
  dim3 grid(N / UN, (M + UM - 1) / UM);
  kernel<<<grid, UMMA_THREADS, smem, st>>>(ma, mb, M, N, K, bias, out, ldo, err);
  return cudaGetLastError();
}

}  // namespace

cudaError_t umma_gemm_bias_relu(int M, int N, int K, const __nv_bfloat16* A, int lda, const __nv_bfloat16* B,
                                int ldb, const float* bias, __nv_bfloat16* out, int ldo, int* err,
                                cudaStream_t st, int variant) {
  CUtensorMap ma, mb;
  if (!make_map(&ma, A, M, K, lda, UM) || !make_map(&mb, B, N, K, ldb, UN)) return cudaErrorInvalidValue;
  return variant == 2 ? launch_umma<2, 2>(ma, mb, M, N, K, bias, out, ldo, err, st)
                      : launch_umma<4, 1>(ma, mb, M, N, K, bias, out, ldo, err, st);
}

bool mlp_fused_supported(int n_in, int in_pad, int hidden, int n_layers, int n_out, const __nv_bfloat16* const W[4],
                         const float* const bias[4]) {
  if (n_layers != 4 || hidden != FH || in_pad != UK || n_in <= 0 || n_in > UK || n_out <= 0 || n_out > FMAX_OUT ||
      encode_fn() == nullptr)
    return false;
  for (int l = 0; l < 4; ++l)
    if ((reinterpret_cast<uintptr_t>(W[l]) % 16) != 0 || (reinterpret_cast<uintptr_t>(bias[l]) % 16) != 0)
      return false;
  return true;
}

cudaError_t mlp_fused_logits(const uint8_t* syn, int64_t n, int sb, int n_in, const __nv_bfloat16* const W[4],
                             const float* const bias[4], int n_out, float* logits, int ldl, int* err,
                             cudaStream_t st, const FusedGate* gate) {
  if (n <= 0) return cudaSuccess;
  if (sb > 8) return cudaErrorInvalidValue;
  // the weights' tensor maps, the SM count and the kernel's shared-memory
  // limit are set up once per weight buffers and device (the step's first
  // kernel is then enqueued without host work in front of it)
  struct Cached {
    const void* w[3] = {nullptr, nullptr, nullptr};
    int dev = -1, sms = 1;
    CUtensorMap m[3];
  };
  static std::mutex mu;
  static Cached cache[8];
  int dev = 0;
  cudaGetDevice(&dev);
  CUtensorMap m1, m2, m3;
  int sms = 1;
  {
    std::lock_guard<std::mutex> lk(mu);
    Cached& c = cache[dev & 7];
    if (c.dev != dev || c.w[0] != W[0] || c.w[1] != W[1] || c.w[2] != W[2]) {
      c.dev = -1;
      if (!make_map(&c.m[0], W[0], FH, UK, UK, FNH) || !make_map(&c.m[1], W[1], FH, FH, FH, FNH) ||
          !make_map(&c.m[2], W[2], FH, FH, FH, FNH))
        return cudaErrorInvalidValue;
      cudaDeviceGetAttribute(&c.sms, cudaDevAttrMultiProcessorCount, dev);
      cudaError_t e = cudaFuncSetAttribute(mlp_fused_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           int(FUSED_SMEM));
      if (e != cudaSuccess) return e;
      for (int i = 0; i < 3; ++i) c.w[i] = W[i];
      c.dev = dev;
    }
    m1 = c.m[0];
    m2 = c.m[1];
    m3 = c.m[2];
    sms = c.sms;
  }
  FusedArgs a;
  a.syn = syn;
  a.sb = sb;
  a.n_in = n_in;
  a.n = n;
  for (int l = 0; l < 3; ++l) a.bias[l] = bias[l];
  a.w4 = W[3];
  a.b4 = bias[3];
  a.n_out = n_out;
  a.ldl = ldl;
  a.logits = logits;
  a.err = err;
  a.threshold = gate ? gate->threshold : 0.f;
  a.cls = gate ? gate->cls : nullptr;
  a.conf = gate ? gate->conf : nullptr;
  a.list = gate ? gate->list : nullptr;
  a.count = gate ? gate->count : nullptr;
  const int64_t ntiles = (n + FM - 1) / FM;
  const int grid = int(std::min<int64_t>(ntiles, sms));
  mlp_fused_kernel<<<grid, FTHREADS, FUSED_SMEM, st>>>(m1, m2, m3, a);
  return cudaGetLastError();
}

}  // namespace tqec
