// mlp.cuh -- kernels of the learned surrogate (a ReLU MLP over syndrome
// bits that proposes the logical class with a confidence).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace tqec {

// Epilogues of the bf16 GEMM  C[m, n] = sum_k A(m, k) * B(n, k).
enum GemmEpilogue : int {
  EPI_BIAS_RELU_BF16 = 0,  // C = relu(acc + bias[n]) as bf16
  EPI_BIAS_F32 = 1,        // C = acc + bias[n] as float
  EPI_MASK_BF16 = 2,       // C = acc * (H[m, n] > 0) as bf16 (ReLU backward)
  EPI_ATOMIC_F32 = 3,      // C += acc with atomics (split-K weight gradients)
};

// A(m,k) = a_kmajor ? A[m*lda + k] : A[k*lda + m]; same for B(n,k).
cudaError_t gemm_bf16(bool a_kmajor, bool b_kmajor, int epi, int M, int N, int K, const __nv_bfloat16* A,
                      int lda, const __nv_bfloat16* B, int ldb, void* C, int ldc, const float* bias,
                      const __nv_bfloat16* H, int ldh, int split_k, cudaStream_t st);

// Output layer with few classes: C[m, c] = bias[c] + sum_k A[m*lda + k] *
// W[c*ldw + k] (float), one warp per row, W staged in shared memory.
// Needs N <= 16, K a multiple of 8 and lda, ldw multiples of 8.
bool small_out_supported(int N, int K, int lda, int ldw);
cudaError_t small_out_gemm(int M, int N, int K, const __nv_bfloat16* A, int lda, const __nv_bfloat16* W, int ldw,
                           const float* bias, float* C, int ldc, cudaStream_t st);

cudaError_t unpack_syndromes_bf16(const uint8_t* syn, int64_t n, int syn_bytes, int n_bits, __nv_bfloat16* X,
                                  int ldx, cudaStream_t st);

cudaError_t softmax_xent(const float* logits, int ldl, const float* targets, int64_t n, int n_out,
                         __nv_bfloat16* dlogits, int ldd, float* loss_sum, cudaStream_t st);

cudaError_t column_sums_bf16(const __nv_bfloat16* D, int ldd, int64_t rows, int cols, float* out,
                             cudaStream_t st);

cudaError_t adam_update(float* w, const float* g, float* m, float* v, __nv_bfloat16* w16, int64_t n, float lr,
                        float b1, float b2, float eps, float c1, float c2, cudaStream_t st);

cudaError_t transpose_bf16(const __nv_bfloat16* in, int rows, int cols, __nv_bfloat16* out, cudaStream_t st);

// softmax over each row of logits; class = first argmax, conf = its
// probability; rows with conf < threshold are appended to fallback_list.
cudaError_t gate_rows(const float* logits, int ldl, int64_t n, int n_out, float threshold, int32_t* cls,
                      float* conf, int32_t* fallback_list, int32_t* fallback_count, cudaStream_t st);

// tcgen05 GEMM (umma_gemm.cu): out = relu(A * B^T + bias) as bf16.
bool umma_gemm_supported(int M, int N, int K, int lda, int ldb, int ldo, const void* A, const void* B,
                         const void* out);
// variant 1: 4-stage ring, one block per SM; 2: 2-stage ring, two blocks per SM.
cudaError_t umma_gemm_bias_relu(int M, int N, int K, const __nv_bfloat16* A, int lda, const __nv_bfloat16* B,
                                int ldb, const float* bias, __nv_bfloat16* out, int ldo, int* err,
                                cudaStream_t st, int variant = 1);

cudaError_t gather_rows(const uint8_t* src, int row_bytes, const int32_t* list, int64_t n, uint8_t* dst,
                        cudaStream_t st);

// The whole forward of a 4-layer surrogate with hidden width 512 (inputs
// padded to 64, at most 16 outputs) in one persistent tcgen05 kernel
// (umma_gemm.cu): logits[n][ldl] from packed syndromes.  W[l] are the bf16
// weight matrices [dout][din] and bias[l] the float32 biases.
bool mlp_fused_supported(int n_in, int in_pad, int hidden, int n_layers, int n_out, const __nv_bfloat16* const W[4],
                         const float* const bias[4]);
// The gate fused into the fused forward's last epilogue (see gate_rows):
// classes, confidences (optional) and the rows below threshold (optional).
struct FusedGate {
  float threshold;
  int32_t* cls;
  float* conf;
  int32_t* list;
  int32_t* count;
};
cudaError_t mlp_fused_logits(const uint8_t* syn, int64_t n, int sb, int n_in, const __nv_bfloat16* const W[4],
                             const float* const bias[4], int n_out, float* logits, int ldl, int* err,
                             cudaStream_t st, const FusedGate* gate = nullptr);
cudaError_t scatter_classes(const int32_t* src, const int32_t* list, int64_t n, int32_t* dst, cudaStream_t st);

}  // namespace tqec
