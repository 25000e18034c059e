// mlp.cu -- kernels of the surrogate MLP: a bf16 x bf16 -> fp32 tiled GEMM
// with fused epilogues, syndrome unpacking, softmax cross-entropy, Adam and
// the confidence gate.
#include <algorithm>
#include <cfloat>

#include "mlp.cuh"

namespace tqec {
namespace {

constexpr int BM = 128, BN = 128, BK = 32, TM = 8, TN = 8;
constexpr int GEMM_THREADS = (BM / TM) * (BN / TN);  // 256

__device__ __forceinline__ float bf(const __nv_bfloat16 x) { return __bfloat162float(x); }

// C[m, n] = sum_k A(m, k) B(n, k) over the k-range of this block's split.
template <bool AK, bool BKM, int EPI>
__global__ void __launch_bounds__(GEMM_THREADS) gemm_kernel(int M, int N, int K, const __nv_bfloat16* __restrict__ A,
                                                            int lda, const __nv_bfloat16* __restrict__ B, int ldb,
                                                            void* C, int ldc, const float* __restrict__ bias,
                                                            const __nv_bfloat16* __restrict__ H, int ldh,
                                                            int k_per_split) {
  __shared__ float As[BK][BM + 4];
  __shared__ float Bs[BK][BN + 4];
  const int tid = threadIdx.x;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int k_begin = blockIdx.z * k_per_split;
  const int k_end = min(K, k_begin + k_per_split);
  const int tr = tid / (BN / TN), tc = tid % (BN / TN);
  float acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = 0.f;
  for (int k0 = k_begin; k0 < k_end; k0 += BK) {
    // stage A tile (BM x BK) and B tile (BN x BK) as float, k-major in smem
    for (int i = tid; i < BM * BK; i += GEMM_THREADS) {
      int mm, kk;
      if (AK) { mm = i / BK; kk = i % BK; } else { kk = i / BM; mm = i % BM; }
      const int gm = m0 + mm, gk = k0 + kk;
      float v = 0.f;
      if (gm < M && gk < k_end) v = bf(AK ? A[int64_t(gm) * lda + gk] : A[int64_t(gk) * lda + gm]);
      As[kk][mm] = v;
    }
    for (int i = tid; i < BN * BK; i += GEMM_THREADS) {
      int nn, kk;
      if (BKM) { nn = i / BK; kk = i % BK; } else { kk = i / BN; nn = i % BN; }
      const int gn = n0 + nn, gk = k0 + kk;
      float v = 0.f;
      if (gn < N && gk < k_end) v = bf(BKM ? B[int64_t(gn) * ldb + gk] : B[int64_t(gk) * ldb + gn]);
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < BK; ++kk) {
      float a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][tr * TM + i];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tc * TN + j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int gm = m0 + tr * TM + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int gn = n0 + tc * TN + j;
      if (gn >= N) continue;
      float v = acc[i][j];
      if (EPI == EPI_BIAS_RELU_BF16) {
        v += bias[gn];
        reinterpret_cast<__nv_bfloat16*>(C)[int64_t(gm) * ldc + gn] = __float2bfloat16(v > 0.f ? v : 0.f);
      } else if (EPI == EPI_BIAS_F32) {
        reinterpret_cast<float*>(C)[int64_t(gm) * ldc + gn] = v + bias[gn];
      } else if (EPI == EPI_MASK_BF16) {
        const float h = bf(H[int64_t(gm) * ldh + gn]);
        reinterpret_cast<__nv_bfloat16*>(C)[int64_t(gm) * ldc + gn] = __float2bfloat16(h > 0.f ? v : 0.f);
      } else {
        atomicAdd(reinterpret_cast<float*>(C) + int64_t(gm) * ldc + gn, v);
      }
    }
  }
}

__global__ void unpack_kernel(const uint8_t* __restrict__ syn, int64_t n, int syn_bytes, int n_bits,
                              __nv_bfloat16* __restrict__ X, int ldx) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t r = i / ldx;
  const int c = int(i % ldx);
  if (r >= n) return;
  float v = 0.f;
  if (c < n_bits) v = float((syn[r * syn_bytes + (c >> 3)] >> (c & 7)) & 1);
  X[r * ldx + c] = __float2bfloat16(v);
}

__global__ void softmax_xent_kernel(const float* __restrict__ logits, int ldl, const float* __restrict__ t,
                                    int64_t n, int n_out, __nv_bfloat16* __restrict__ d, int ldd,
                                    float* __restrict__ loss_sum) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  float loss = 0.f;
  if (r < n) {
    const float* l = logits + r * ldl;
    float mx = -FLT_MAX;
    for (int c = 0; c < n_out; ++c) mx = fmaxf(mx, l[c]);
    float s = 0.f;
    for (int c = 0; c < n_out; ++c) s += __expf(l[c] - mx);
    const float ls = __logf(s);
    const float inv_n = 1.0f / float(n);
    for (int c = 0; c < n_out; ++c) {
      const float lp = l[c] - mx - ls;
      const float tc = t[r * n_out + c];
      if (tc > 0.f) loss -= tc * lp;
      d[r * ldd + c] = __float2bfloat16((__expf(lp) - tc) * inv_n);
    }
    for (int c = n_out; c < ldd; ++c) d[r * ldd + c] = __float2bfloat16(0.f);
  }
  for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss_sum, loss);
}

__global__ void column_sums_kernel(const __nv_bfloat16* __restrict__ D, int ldd, int64_t rows, int cols,
                                   float* __restrict__ out) {
  // block: 32 columns x 8 row-lanes
  const int c = blockIdx.x * 32 + threadIdx.x;
  float s = 0.f;
  if (c < cols)
    for (int64_t r = blockIdx.y * 8 + threadIdx.y; r < rows; r += int64_t(gridDim.y) * 8) s += bf(D[r * ldd + c]);
  __shared__ float sh[8][33];
  sh[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && c < cols) {
    float t = 0.f;
    for (int y = 0; y < 8; ++y) t += sh[y][threadIdx.x];
    atomicAdd(out + c, t);
  }
}

__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, __nv_bfloat16* __restrict__ w16, int64_t n, float lr, float b1,
                            float b2, float eps, float c1, float c2) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
  w[i] = wi;
  if (w16) w16[i] = __float2bfloat16(wi);
}

__global__ void transpose_kernel(const __nv_bfloat16* __restrict__ in, int rows, int cols,
                                 __nv_bfloat16* __restrict__ out) {
  __shared__ __nv_bfloat16 tile[32][33];
  const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 32 + threadIdx.y;
  for (int j = 0; j < 32; j += 8)
    if (x < cols && y + j < rows) tile[threadIdx.y + j][threadIdx.x] = in[int64_t(y + j) * cols + x];
  __syncthreads();
  const int ox = blockIdx.y * 32 + threadIdx.x, oy = blockIdx.x * 32 + threadIdx.y;
  for (int j = 0; j < 32; j += 8)
    if (ox < rows && oy + j < cols) out[int64_t(oy + j) * rows + ox] = tile[threadIdx.x][threadIdx.y + j];
}

__global__ void gate_kernel(const float* __restrict__ logits, int ldl, int64_t n, int n_out, float thr,
                            int32_t* __restrict__ cls, float* __restrict__ conf, int32_t* __restrict__ list,
                            int32_t* __restrict__ count) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const float* l = logits + r * ldl;
  float mx = l[0];
  int bc = 0;
  for (int c = 1; c < n_out; ++c)
    if (l[c] > mx) { mx = l[c]; bc = c; }
  float s = 0.f;
  for (int c = 0; c < n_out; ++c) s += __expf(l[c] - mx);
  const float p = 1.0f / s;
  if (cls) cls[r] = bc;
  if (conf) conf[r] = p;
  if (list && !(p >= thr)) list[atomicAdd(count, 1)] = int32_t(r);
}

// One warp per row: lanes split k in chunks of 8 (one 16-byte load of the
// activation row per chunk), every class's partial sum is reduced over the
// warp.  The weights (N x K) sit in shared memory.
template <int NC>
__global__ void __launch_bounds__(256) small_out_kernel(int M, int N, int K, const __nv_bfloat16* __restrict__ A,
                                                        int lda, const __nv_bfloat16* __restrict__ W, int ldw,
                                                        const float* __restrict__ bias, float* __restrict__ C,
                                                        int ldc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __nv_bfloat16* sw = reinterpret_cast<__nv_bfloat16*>(smem_raw);
  for (int i = threadIdx.x; i < N * (K / 8); i += blockDim.x) {
    const int c = i / (K / 8), j = i % (K / 8);
    reinterpret_cast<uint4*>(sw + c * K)[j] = *reinterpret_cast<const uint4*>(W + int64_t(c) * ldw + 8 * j);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t warps = int64_t(gridDim.x) * (blockDim.x >> 5);
  for (int64_t r = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5); r < M; r += warps) {
    float acc[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) acc[c] = 0.f;
    const __nv_bfloat16* a = A + r * lda;
    for (int k0 = 8 * lane; k0 < K; k0 += 256) {
      const uint4 av = *reinterpret_cast<const uint4*>(a + k0);
      const __nv_bfloat162* a2 = reinterpret_cast<const __nv_bfloat162*>(&av);
      float2 af[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) af[j] = __bfloat1622float2(a2[j]);
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        if (c >= N) break;
        const uint4 wv = *reinterpret_cast<const uint4*>(sw + c * K + k0);
        const __nv_bfloat162* w2 = reinterpret_cast<const __nv_bfloat162*>(&wv);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float2 wf = __bfloat1622float2(w2[j]);
          acc[c] = fmaf(af[j].x, wf.x, acc[c]);
          acc[c] = fmaf(af[j].y, wf.y, acc[c]);
        }
      }
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      if (c >= N) break;
      float v = acc[c];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == c) C[r * ldc + c] = v + (bias ? bias[c] : 0.f);
    }
  }
}

__global__ void gather_kernel(const uint8_t* __restrict__ src, int row_bytes, const int32_t* __restrict__ list,
                              int64_t n, uint8_t* __restrict__ dst) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n * row_bytes) return;
  const int64_t r = i / row_bytes;
  const int b = int(i % row_bytes);
  dst[i] = src[int64_t(list[r]) * row_bytes + b];
}

__global__ void scatter_kernel(const int32_t* __restrict__ src, const int32_t* __restrict__ list, int64_t n,
                               int32_t* __restrict__ dst) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) dst[list[i]] = src[i];
}

unsigned blocks_for(int64_t n, int t) { return unsigned((n + t - 1) / t); }

}  // namespace

cudaError_t gemm_bf16(bool a_kmajor, bool b_kmajor, int epi, int M, int N, int K, const __nv_bfloat16* A, int lda,
                      const __nv_bfloat16* B, int ldb, void* C, int ldc, const float* bias, const __nv_bfloat16* H,
                      int ldh, int split_k, cudaStream_t st) {
  if (M <= 0 || N <= 0 || K <= 0) return cudaSuccess;
  split_k = split_k < 1 ? 1 : split_k;
  int kps = (K + split_k - 1) / split_k;
  kps = (kps + BK - 1) / BK * BK;
  const int splits = (K + kps - 1) / kps;
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, splits);
#define TQ_GEMM(AKM, BKMM, E) \
  gemm_kernel<AKM, BKMM, E><<<grid, GEMM_THREADS, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, H, ldh, kps)
  if (a_kmajor && b_kmajor) {
    if (epi == EPI_BIAS_RELU_BF16) TQ_GEMM(true, true, EPI_BIAS_RELU_BF16);
    else if (epi == EPI_BIAS_F32) TQ_GEMM(true, true, EPI_BIAS_F32);
    else return cudaErrorInvalidValue;
  } else if (a_kmajor && !b_kmajor) {
    if (epi == EPI_MASK_BF16) TQ_GEMM(true, false, EPI_MASK_BF16);
    else return cudaErrorInvalidValue;
  } else if (!a_kmajor && !b_kmajor) {
    if (epi == EPI_ATOMIC_F32) TQ_GEMM(false, false, EPI_ATOMIC_F32);
    else return cudaErrorInvalidValue;
  } else {
    return cudaErrorInvalidValue;
  }
#undef TQ_GEMM
  return cudaGetLastError();
}

bool small_out_supported(int N, int K, int lda, int ldw) {
  return N >= 1 && N <= 16 && K % 8 == 0 && lda % 8 == 0 && ldw % 8 == 0 && size_t(N) * K * 2 <= 96 * 1024;
}

cudaError_t small_out_gemm(int M, int N, int K, const __nv_bfloat16* A, int lda, const __nv_bfloat16* W, int ldw,
                           const float* bias, float* C, int ldc, cudaStream_t st) {
  if (M <= 0) return cudaSuccess;
  if (!small_out_supported(N, K, lda, ldw)) return cudaErrorInvalidValue;
  const size_t smem = size_t(N) * K * 2;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const unsigned grid = unsigned(std::min<int64_t>((int64_t(M) + 7) / 8, int64_t(sms) * 8));
  if (N <= 4) {
    cudaFuncSetAttribute(small_out_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    small_out_kernel<4><<<grid, 256, smem, st>>>(M, N, K, A, lda, W, ldw, bias, C, ldc);
  } else {
    cudaFuncSetAttribute(small_out_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    small_out_kernel<16><<<grid, 256, smem, st>>>(M, N, K, A, lda, W, ldw, bias, C, ldc);
  }
  return cudaGetLastError();
}

cudaError_t unpack_syndromes_bf16(const uint8_t* syn, int64_t n, int syn_bytes, int n_bits, __nv_bfloat16* X, int ldx,
                                  cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  unpack_kernel<<<blocks_for(n * ldx, 256), 256, 0, st>>>(syn, n, syn_bytes, n_bits, X, ldx);
  return cudaGetLastError();
}

cudaError_t softmax_xent(const float* logits, int ldl, const float* targets, int64_t n, int n_out,
                         __nv_bfloat16* dlogits, int ldd, float* loss_sum, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  softmax_xent_kernel<<<blocks_for(n, 256), 256, 0, st>>>(logits, ldl, targets, n, n_out, dlogits, ldd, loss_sum);
  return cudaGetLastError();
}

cudaError_t column_sums_bf16(const __nv_bfloat16* D, int ldd, int64_t rows, int cols, float* out, cudaStream_t st) {
  if (rows <= 0) return cudaSuccess;
  dim3 grid((cols + 31) / 32, (unsigned)std::min<int64_t>(64, (rows + 7) / 8));
  column_sums_kernel<<<grid, dim3(32, 8), 0, st>>>(D, ldd, rows, cols, out);
  return cudaGetLastError();
}

cudaError_t adam_update(float* w, const float* g, float* m, float* v, __nv_bfloat16* w16, int64_t n, float lr,
                        float b1, float b2, float eps, float c1, float c2, cudaStream_t st) {
  adam_kernel<<<blocks_for(n, 256), 256, 0, st>>>(w, g, m, v, w16, n, lr, b1, b2, eps, c1, c2);
  return cudaGetLastError();
}

cudaError_t transpose_bf16(const __nv_bfloat16* in, int rows, int cols, __nv_bfloat16* out, cudaStream_t st) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32);
  transpose_kernel<<<grid, dim3(32, 8), 0, st>>>(in, rows, cols, out);
  return cudaGetLastError();
}

cudaError_t gate_rows(const float* logits, int ldl, int64_t n, int n_out, float threshold, int32_t* cls, float* conf,
                      int32_t* fallback_list, int32_t* fallback_count, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  gate_kernel<<<blocks_for(n, 256), 256, 0, st>>>(logits, ldl, n, n_out, threshold, cls, conf, fallback_list,
                                                  fallback_count);
  return cudaGetLastError();
}

cudaError_t gather_rows(const uint8_t* src, int row_bytes, const int32_t* list, int64_t n, uint8_t* dst,
                        cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  gather_kernel<<<blocks_for(n * row_bytes, 256), 256, 0, st>>>(src, row_bytes, list, n, dst);
  return cudaGetLastError();
}

cudaError_t scatter_classes(const int32_t* src, const int32_t* list, int64_t n, int32_t* dst, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  scatter_kernel<<<blocks_for(n, 256), 256, 0, st>>>(src, list, n, dst);
  return cudaGetLastError();
}

}  // namespace tqec
