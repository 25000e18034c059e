// surrogate.cu -- the learned surrogate in front of the exact contraction.
//
// A ReLU MLP (layers of `hidden` units) reads the syndrome bits and
// proposes the logical class; its softmax probability of that class is the
// confidence.  Rows whose confidence is below a threshold go to the exact
// contraction (tqec_decode_batch), which also produced the soft labels the
// network was trained on.  Weights are kept as float32 masters with bf16
// copies for the GEMMs; every GEMM accumulates in float32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <random>
#include <string>
#include <vector>

#include "../../include/tqec_gb300.h"
#include "mlp.cuh"

namespace tqec {
std::string& last_error_ref();
}

namespace {

int sfail(int code, const std::string& m) {
  tqec::last_error_ref() = m;
  return code;
}

#define SQ_CUDA(call)                                                                   \
  do {                                                                                  \
    cudaError_t e__ = (call);                                                           \
    if (e__ != cudaSuccess)                                                             \
      return sfail(e__ == cudaErrorMemoryAllocation ? TQEC_ERR_OOM : TQEC_ERR_CUDA,     \
                   std::string(#call) + ": " + cudaGetErrorString(e__));                \
  } while (0)

bool dev_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

int round_up(int x, int m) { return (x + m - 1) / m * m; }

}  // namespace

struct tqec_mlp {
  tqec_mlp_config cfg;
  int in_pad = 64, out_pad = 16, L = 4;
  std::vector<int> din, dout;                 // per layer (din padded for layer 0)
  std::vector<size_t> w_off, b_off;           // into the parameter vector
  size_t n_params = 0;
  float *w32 = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  __nv_bfloat16* w16 = nullptr;
  int64_t cap = 0;
  __nv_bfloat16* X0 = nullptr;
  std::vector<__nv_bfloat16*> H;              // L-1 hidden activations
  float* logits = nullptr;
  __nv_bfloat16* dl = nullptr;
  __nv_bfloat16* dH[2] = {nullptr, nullptr};
  float* loss = nullptr;
  float* h_loss = nullptr;                    // pinned
  uint8_t* syn = nullptr;                     // staged inputs
  size_t syn_cap = 0;
  float* tgt = nullptr;
  int32_t *cls = nullptr, *list = nullptr, *count = nullptr, *h_count = nullptr;
  int32_t* h_counts = nullptr;                // pinned: rows each chunk of the last gated decode sent on
  int64_t h_counts_cap = 0, last_chunks = 0;
  int64_t fallback_hint = 0;                  // rows per chunk the gate sent on, when last read
  float* conf = nullptr;
  uint8_t* gathered = nullptr;
  int32_t* gcls = nullptr;
  int adam_t = 0;
  // hidden layers: 0 SIMT GEMM; tcgen05 GEMM layer by layer with 1 or 2
  // blocks per SM; 3 (default) inference by the fused forward kernel where
  // the shape allows (training keeps mode 2's GEMMs)
  int use_tensor_cores = 3;
  int* d_err = nullptr;                       // timeout flag of the tcgen05 kernel
  int* h_err = nullptr;                       // pinned
  int* d_bad = nullptr;                       // a gathered row index was outside the set
  cudaStream_t stream = nullptr;
  std::mutex mu;
};

namespace {

void free_acts(tqec_mlp* p) {
  cudaFree(p->X0);
  for (auto* h : p->H) cudaFree(h);
  p->H.clear();
  cudaFree(p->logits);
  cudaFree(p->dl);
  cudaFree(p->dH[0]);
  cudaFree(p->dH[1]);
  cudaFree(p->tgt);
  cudaFree(p->cls);
  cudaFree(p->list);
  cudaFree(p->conf);
  cudaFree(p->gathered);
  cudaFree(p->gcls);
  p->X0 = nullptr;
  p->logits = p->tgt = p->conf = nullptr;
  p->dl = p->dH[0] = p->dH[1] = nullptr;
  p->cls = p->list = p->gcls = nullptr;
  p->gathered = nullptr;
  p->cap = 0;
}

int ensure_cap(tqec_mlp* p, int64_t n) {
  if (n <= p->cap) return TQEC_OK;
  free_acts(p);
  const int64_t c = std::max<int64_t>(n, 1024);
  const int hid = p->cfg.hidden;
  SQ_CUDA(cudaMalloc(&p->X0, sizeof(__nv_bfloat16) * c * p->in_pad));
  for (int l = 0; l < p->L - 1; ++l) {
    __nv_bfloat16* h = nullptr;
    SQ_CUDA(cudaMalloc(&h, sizeof(__nv_bfloat16) * c * hid));
    p->H.push_back(h);
  }
  SQ_CUDA(cudaMalloc(&p->logits, sizeof(float) * c * p->out_pad));
  SQ_CUDA(cudaMalloc(&p->dl, sizeof(__nv_bfloat16) * c * p->out_pad));
  SQ_CUDA(cudaMalloc(&p->dH[0], sizeof(__nv_bfloat16) * c * hid));
  SQ_CUDA(cudaMalloc(&p->dH[1], sizeof(__nv_bfloat16) * c * hid));
  SQ_CUDA(cudaMalloc(&p->tgt, sizeof(float) * c * p->cfg.n_out));
  SQ_CUDA(cudaMalloc(&p->cls, sizeof(int32_t) * c));
  SQ_CUDA(cudaMalloc(&p->list, sizeof(int32_t) * c));
  SQ_CUDA(cudaMalloc(&p->conf, sizeof(float) * c));
  SQ_CUDA(cudaMalloc(&p->gathered, size_t(c) * ((p->cfg.n_in + 7) / 8)));
  SQ_CUDA(cudaMalloc(&p->gcls, sizeof(int32_t) * c));
  p->cap = c;
  return TQEC_OK;
}

int stage_syn(tqec_mlp* p, const uint8_t* syn, int64_t n, cudaStream_t st, const uint8_t** out) {
  const size_t bytes = size_t(n) * ((p->cfg.n_in + 7) / 8);
  if (dev_ptr(syn)) {
    *out = syn;
    return TQEC_OK;
  }
  if (bytes > p->syn_cap) {
    cudaFree(p->syn);
    p->syn = nullptr;
    p->syn_cap = 0;
    SQ_CUDA(cudaMalloc(&p->syn, std::max<size_t>(bytes, 64)));
    p->syn_cap = std::max<size_t>(bytes, 64);
  }
  if (bytes) SQ_CUDA(cudaMemcpyAsync(p->syn, syn, bytes, cudaMemcpyHostToDevice, st));
  *out = p->syn;
  return TQEC_OK;
}

// forward over rows [0, n) of already-staged syndromes; logits in p->logits
int forward(tqec_mlp* p, const uint8_t* dsyn, int64_t n, cudaStream_t st) {
  const int sb = (p->cfg.n_in + 7) / 8;
  SQ_CUDA(tqec::unpack_syndromes_bf16(dsyn, n, sb, p->cfg.n_in, p->X0, p->in_pad, st));
  const __nv_bfloat16* x = p->X0;
  int ldx = p->in_pad;
  for (int l = 0; l < p->L; ++l) {
    const __nv_bfloat16* W = p->w16 + p->w_off[l];
    const float* b = p->w32 + p->b_off[l];
    if (l < p->L - 1) {
      if (p->use_tensor_cores &&
          tqec::umma_gemm_supported((int)n, p->dout[l], p->din[l], ldx, p->din[l], p->cfg.hidden, x, W, p->H[l]))
        SQ_CUDA(tqec::umma_gemm_bias_relu((int)n, p->dout[l], p->din[l], x, ldx, W, p->din[l], b, p->H[l],
                                          p->cfg.hidden, p->d_err, st, p->use_tensor_cores == 1 ? 1 : 2));
      else
        SQ_CUDA(tqec::gemm_bf16(true, true, tqec::EPI_BIAS_RELU_BF16, (int)n, p->dout[l], p->din[l], x, ldx, W,
                                p->din[l], p->H[l], p->cfg.hidden, b, nullptr, 0, 1, st));
      x = p->H[l];
      ldx = p->cfg.hidden;
    } else if (tqec::small_out_supported(p->dout[l], p->din[l], ldx, p->din[l])) {
      // few classes: a row-per-warp kernel instead of a mostly empty GEMM tile
      SQ_CUDA(tqec::small_out_gemm((int)n, p->dout[l], p->din[l], x, ldx, W, p->din[l], b, p->logits, p->out_pad,
                                   st));
    } else {
      SQ_CUDA(tqec::gemm_bf16(true, true, tqec::EPI_BIAS_F32, (int)n, p->dout[l], p->din[l], x, ldx, W, p->din[l],
                              p->logits, p->out_pad, b, nullptr, 0, 1, st));
    }
  }
  return TQEC_OK;
}

// Inference forward: the fused kernel (all layers in one persistent launch,
// activations kept on chip) in mode 3 where the shape allows, else forward().
// The inference forward; with `gate` (and the fused kernel) the gate runs in
// its last epilogue and *gated is set, else the caller runs gate_rows.
int forward_infer(tqec_mlp* p, const uint8_t* dsyn, int64_t n, cudaStream_t st,
                  const tqec::FusedGate* gate = nullptr, bool* gated = nullptr) {
  if (gated) *gated = false;
  if (p->use_tensor_cores == 3) {
    const __nv_bfloat16* W[4];
    const float* B[4];
    for (int l = 0; l < p->L && l < 4; ++l) {
      W[l] = p->w16 + p->w_off[l];
      B[l] = p->w32 + p->b_off[l];
    }
    if (tqec::mlp_fused_supported(p->cfg.n_in, p->in_pad, p->cfg.hidden, p->L, p->cfg.n_out, W, B)) {
      SQ_CUDA(tqec::mlp_fused_logits(dsyn, n, (p->cfg.n_in + 7) / 8, p->cfg.n_in, W, B, p->cfg.n_out, p->logits,
                                     p->out_pad, p->d_err, st, gate));
      if (gated) *gated = gate != nullptr;
      return TQEC_OK;
    }
  }
  return forward(p, dsyn, n, st);
}

// gradients into p->g for rows [0, n) with float targets already in p->tgt
int backward(tqec_mlp* p, int64_t n, cudaStream_t st) {
  SQ_CUDA(cudaMemsetAsync(p->g, 0, sizeof(float) * p->n_params, st));
  SQ_CUDA(cudaMemsetAsync(p->loss, 0, sizeof(float), st));
  SQ_CUDA(tqec::softmax_xent(p->logits, p->out_pad, p->tgt, n, p->cfg.n_out, p->dl, p->out_pad, p->loss, st));
  const __nv_bfloat16* dy = p->dl;
  int ldy = p->out_pad;
  int ping = 0;
  const int split = (int)std::max<int64_t>(1, std::min<int64_t>(64, n / 256));
  for (int l = p->L - 1; l >= 0; --l) {
    const __nv_bfloat16* x = l == 0 ? p->X0 : p->H[l - 1];
    const int ldx = l == 0 ? p->in_pad : p->cfg.hidden;
    // dW[dout, din] = dY^T X  (split over the batch)
    SQ_CUDA(tqec::gemm_bf16(false, false, tqec::EPI_ATOMIC_F32, p->dout[l], p->din[l], (int)n, dy, ldy, x, ldx,
                            p->g + p->w_off[l], p->din[l], nullptr, nullptr, 0, split, st));
    SQ_CUDA(tqec::column_sums_bf16(dy, ldy, n, p->dout[l], p->g + p->b_off[l], st));
    if (l > 0) {
      // dX[n, din] = dY W, masked by relu'(H[l-1])
      SQ_CUDA(tqec::gemm_bf16(true, false, tqec::EPI_MASK_BF16, (int)n, p->din[l], p->dout[l], dy, ldy,
                              p->w16 + p->w_off[l], p->din[l], p->dH[ping], p->cfg.hidden, nullptr, p->H[l - 1],
                              p->cfg.hidden, 1, st));
      dy = p->dH[ping];
      ldy = p->cfg.hidden;
      ping ^= 1;
    }
  }
  return TQEC_OK;
}

int refresh_bf16(tqec_mlp* p, cudaStream_t st) {
  // w16 = bf16(w32) via a zero-learning-rate Adam pass would disturb moments;
  // convert on the host instead (only used after set/load)
  std::vector<float> h(p->n_params);
  SQ_CUDA(cudaMemcpyAsync(h.data(), p->w32, sizeof(float) * p->n_params, cudaMemcpyDeviceToHost, st));
  SQ_CUDA(cudaStreamSynchronize(st));
  std::vector<__nv_bfloat16> b(p->n_params);
  for (size_t i = 0; i < p->n_params; ++i) b[i] = __float2bfloat16(h[i]);
  SQ_CUDA(cudaMemcpyAsync(p->w16, b.data(), sizeof(__nv_bfloat16) * p->n_params, cudaMemcpyHostToDevice, st));
  SQ_CUDA(cudaStreamSynchronize(st));
  return TQEC_OK;
}

// Reports a timed-out tcgen05 wait (recorded by the kernel) as an error.
int check_device_error(tqec_mlp* p, cudaStream_t st) {
  SQ_CUDA(cudaMemcpyAsync(p->h_err, p->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
  SQ_CUDA(cudaStreamSynchronize(st));
  if (*p->h_err) {
    cudaMemsetAsync(p->d_err, 0, sizeof(int), st);
    return sfail(TQEC_ERR_TIMEOUT, "a tensor-core GEMM wait timed out");
  }
  return TQEC_OK;
}

}  // namespace

extern "C" {

int tqec_mlp_set_gemm(tqec_mlp* p, int use_tensor_cores) {
  if (!p) return sfail(TQEC_ERR_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lk(p->mu);
  if (use_tensor_cores < 0 || use_tensor_cores > 3) return sfail(TQEC_ERR_INVALID, "GEMM mode must be 0 to 3");
  p->use_tensor_cores = use_tensor_cores;
  return TQEC_OK;
}

int tqec_mlp_forward_logits(tqec_mlp* p, const uint8_t* syn, int64_t n, float* logits_out) {
  if (!p || !syn || !logits_out || n <= 0) return sfail(TQEC_ERR_INVALID, "bad argument");
  std::lock_guard<std::mutex> lk(p->mu);
  SQ_CUDA(cudaSetDevice(p->cfg.device));
  cudaStream_t st = p->stream;
  int rc = ensure_cap(p, n);
  if (rc) return rc;
  const uint8_t* ds;
  if ((rc = stage_syn(p, syn, n, st, &ds))) return rc;
  if ((rc = forward_infer(p, ds, n, st))) return rc;
  SQ_CUDA(cudaMemcpy2DAsync(logits_out, sizeof(float) * p->cfg.n_out, p->logits, sizeof(float) * p->out_pad,
                            sizeof(float) * p->cfg.n_out, size_t(n), cudaMemcpyDeviceToHost, st));
  return check_device_error(p, st);
}

int tqec_mlp_create(const tqec_mlp_config* cfg, tqec_mlp** out) {
  if (!cfg || !out) return sfail(TQEC_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (cfg->n_in < 1 || cfg->n_in > 4096 || cfg->n_out < 2 || cfg->n_out > 16 || cfg->hidden < 32 ||
      cfg->hidden % 32 || cfg->n_layers < 2 || cfg->n_layers > 16)
    return sfail(TQEC_ERR_INVALID, "bad surrogate configuration");
  auto* p = new tqec_mlp();
  p->cfg = *cfg;
  p->L = cfg->n_layers;
  p->in_pad = round_up(cfg->n_in, 64);
  for (int l = 0; l < p->L; ++l) {
    p->din.push_back(l == 0 ? p->in_pad : cfg->hidden);
    p->dout.push_back(l == p->L - 1 ? cfg->n_out : cfg->hidden);
  }
  size_t off = 0;
  for (int l = 0; l < p->L; ++l) {
    p->w_off.push_back(off);
    off += size_t(p->din[l]) * p->dout[l];
    p->b_off.push_back(off);
    off += size_t(p->dout[l]);
    off = (off + 7) & ~size_t(7);
  }
  p->n_params = off;
  auto bail = [&](int c, const std::string& m) {
    tqec_mlp_destroy(p);
    return sfail(c, m);
  };
  if (cudaSetDevice(cfg->device) != cudaSuccess) return bail(TQEC_ERR_CUDA, "cudaSetDevice");
  if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(TQEC_ERR_CUDA, "stream");
  if (cudaMalloc(&p->w32, sizeof(float) * off) || cudaMalloc(&p->g, sizeof(float) * off) ||
      cudaMalloc(&p->m, sizeof(float) * off) || cudaMalloc(&p->v, sizeof(float) * off) ||
      cudaMalloc(&p->w16, sizeof(__nv_bfloat16) * off) || cudaMalloc(&p->loss, sizeof(float)) ||
      cudaMallocHost(&p->h_loss, sizeof(float)) || cudaMalloc(&p->count, sizeof(int32_t)) ||
      cudaMallocHost(&p->h_count, sizeof(int32_t)) || cudaMalloc(&p->d_err, sizeof(int)) ||
      cudaMallocHost(&p->h_err, sizeof(int)) || cudaMalloc(&p->d_bad, sizeof(int)))
    return bail(TQEC_ERR_OOM, "surrogate parameters");
  cudaMemset(p->d_err, 0, sizeof(int));
  cudaMemset(p->d_bad, 0, sizeof(int));
  cudaMemset(p->m, 0, sizeof(float) * off);
  cudaMemset(p->v, 0, sizeof(float) * off);
  // uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights and biases; the padded
  // input columns of layer 0 stay zero
  std::vector<float> h(off, 0.f);
  std::mt19937_64 rng(cfg->seed ? cfg->seed : 1);
  for (int l = 0; l < p->L; ++l) {
    const int fan_in = l == 0 ? cfg->n_in : p->din[l];
    const float a = 1.0f / std::sqrt(float(fan_in));
    std::uniform_real_distribution<float> U(-a, a);
    for (int o = 0; o < p->dout[l]; ++o)
      for (int i = 0; i < p->din[l]; ++i)
        h[p->w_off[l] + size_t(o) * p->din[l] + i] = (l == 0 && i >= cfg->n_in) ? 0.f : U(rng);
    for (int o = 0; o < p->dout[l]; ++o) h[p->b_off[l] + o] = U(rng);
  }
  cudaMemcpy(p->w32, h.data(), sizeof(float) * off, cudaMemcpyHostToDevice);
  if (refresh_bf16(p, p->stream) != TQEC_OK) return bail(TQEC_ERR_CUDA, "weights");
  *out = p;
  return TQEC_OK;
}

int tqec_mlp_destroy(tqec_mlp* p) {
  if (!p) return TQEC_OK;
  cudaSetDevice(p->cfg.device);
  if (p->stream) cudaStreamSynchronize(p->stream);
  free_acts(p);
  cudaFree(p->w32);
  cudaFree(p->g);
  cudaFree(p->m);
  cudaFree(p->v);
  cudaFree(p->w16);
  cudaFree(p->loss);
  cudaFree(p->count);
  cudaFree(p->syn);
  cudaFree(p->d_err);
  cudaFree(p->d_bad);
  if (p->h_err) cudaFreeHost(p->h_err);
  if (p->h_loss) cudaFreeHost(p->h_loss);
  if (p->h_count) cudaFreeHost(p->h_count);
  if (p->h_counts) cudaFreeHost(p->h_counts);
  if (p->stream) cudaStreamDestroy(p->stream);
  delete p;
  return TQEC_OK;
}

int tqec_mlp_param_count(const tqec_mlp* p, int64_t* n) {
  if (!p || !n) return sfail(TQEC_ERR_INVALID, "NULL argument");
  *n = (int64_t)p->n_params;
  return TQEC_OK;
}

int tqec_mlp_get_params(tqec_mlp* p, float* out, int64_t n) {
  if (!p || !out || n != (int64_t)p->n_params) return sfail(TQEC_ERR_INVALID, "bad argument");
  std::lock_guard<std::mutex> lk(p->mu);
  SQ_CUDA(cudaSetDevice(p->cfg.device));
  SQ_CUDA(cudaMemcpyAsync(out, p->w32, sizeof(float) * n, cudaMemcpyDeviceToHost, p->stream));
  SQ_CUDA(cudaStreamSynchronize(p->stream));
  return TQEC_OK;
}

int tqec_mlp_set_params(tqec_mlp* p, const float* in, int64_t n) {
  if (!p || !in || n != (int64_t)p->n_params) return sfail(TQEC_ERR_INVALID, "bad argument");
  std::lock_guard<std::mutex> lk(p->mu);
  SQ_CUDA(cudaSetDevice(p->cfg.device));
  SQ_CUDA(cudaMemcpyAsync(p->w32, in, sizeof(float) * n, cudaMemcpyHostToDevice, p->stream));
  SQ_CUDA(cudaMemsetAsync(p->m, 0, sizeof(float) * n, p->stream));
  SQ_CUDA(cudaMemsetAsync(p->v, 0, sizeof(float) * n, p->stream));
  p->adam_t = 0;
  return refresh_bf16(p, p->stream);
}

int tqec_mlp_gradients(tqec_mlp* p, const uint8_t* syn, const float* targets, int64_t n, float* grads_out,
                       float* loss_out) {
  if (!p || !syn || !targets || n <= 0) return sfail(TQEC_ERR_INVALID, "bad argument");
  std::lock_guard<std::mutex> lk(p->mu);
  SQ_CUDA(cudaSetDevice(p->cfg.device));
  cudaStream_t st = p->stream;
  int rc = ensure_cap(p, n);
  if (rc) return rc;
  const uint8_t* ds;
  if ((rc = stage_syn(p, syn, n, st, &ds))) return rc;
  SQ_CUDA(cudaMemcpyAsync(p->tgt, targets, sizeof(float) * n * p->cfg.n_out,
                          dev_ptr(targets) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
  if ((rc = forward(p, ds, n, st))) return rc;
  if ((rc = backward(p, n, st))) return rc;
  if (grads_out)
    SQ_CUDA(cudaMemcpyAsync(grads_out, p->g, sizeof(float) * p->n_params, cudaMemcpyDeviceToHost, st));
  SQ_CUDA(cudaMemcpyAsync(p->h_loss, p->loss, sizeof(float), cudaMemcpyDeviceToHost, st));
  SQ_CUDA(cudaStreamSynchronize(st));
  if (loss_out) *loss_out = *p->h_loss / float(n);
  return TQEC_OK;
}

}  // extern "C"

namespace {

// Forward, backward and one Adam step over rows [0, n) of staged syndromes
// `ds` with targets in p->tgt; the loss is read back (one synchronisation)
// only when asked for.
int train_rows(tqec_mlp* p, const uint8_t* ds, int64_t n, float lr, float* loss_out, cudaStream_t st) {
  int rc;
  if ((rc = forward(p, ds, n, st))) return rc;
  if ((rc = backward(p, n, st))) return rc;
  p->adam_t += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f / (1.0f - std::pow(b1, float(p->adam_t)));
  const float c2 = 1.0f / (1.0f - std::pow(b2, float(p->adam_t)));
  SQ_CUDA(tqec::adam_update(p->w32, p->g, p->m, p->v, p->w16, (int64_t)p->n_params, lr, b1, b2, 1e-8f, c1, c2, st));
  if (loss_out) {
    SQ_CUDA(cudaMemcpyAsync(p->h_loss, p->loss, sizeof(float), cudaMemcpyDeviceToHost, st));
    SQ_CUDA(cudaStreamSynchronize(st));
    *loss_out = *p->h_loss / float(n);
  }
  return TQEC_OK;
}

// rows[i] of a resident training set (syndromes `sb` bytes a row, targets
// `nc` floats a row) into the step buffers; an index outside [0, n_set)
// reads row 0 and raises *bad
__global__ void gather_rows_kernel(const uint8_t* syn, int sb, const float* tgt, int nc, int64_t n_set,
                                   const int32_t* rows, int64_t n, uint8_t* syn_out, float* tgt_out, int* bad) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    int64_t r = rows[i];
    if (r < 0 || r >= n_set) {
      atomicExch(bad, 1);
      r = 0;
    }
    for (int b = 0; b < sb; ++b) syn_out[i * sb + b] = syn[r * sb + b];
    for (int c = 0; c < nc; ++c) tgt_out[i * nc + c] = tgt[r * nc + c];
  }
}

}  // namespace

extern "C" {

int tqec_mlp_train_step(tqec_mlp* p, const uint8_t* syn, const float* targets, int64_t n, float lr, float* loss_out,
                        void* stream) {
  if (!p || !syn || !targets || n <= 0) return sfail(TQEC_ERR_INVALID, "bad argument");
  std::lock_guard<std::mutex> lk(p->mu);
  SQ_CUDA(cudaSetDevice(p->cfg.device));
  cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
  int rc = ensure_cap(p, n);
  if (rc) return rc;
  const uint8_t* ds;
  if ((rc = stage_syn(p, syn, n, st, &ds))) return rc;
  SQ_CUDA(cudaMemcpyAsync(p->tgt, targets, sizeof(float) * n * p->cfg.n_out,
                          dev_ptr(targets) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
  return train_rows(p, ds, n, lr, loss_out, st);
}

int tqec_mlp_train_step_rows(tqec_mlp* p, const uint8_t* syn, const float* targets, int64_t n_set,
                             const int32_t* rows, int64_t n, float lr, float* loss_out, void* stream) {
  if (!p || !syn || !targets || !rows || n <= 0 || n_set <= 0) return sfail(TQEC_ERR_INVALID, "bad argument");
  if (!dev_ptr(syn) || !dev_ptr(targets) || !dev_ptr(rows))
    return sfail(TQEC_ERR_INVALID, "the training set and the row indices must be in device memory");
  std::lock_guard<std::mutex> lk(p->mu);
  SQ_CUDA(cudaSetDevice(p->cfg.device));
  cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
  int rc = ensure_cap(p, n);
  if (rc) return rc;
  const int sb = (p->cfg.n_in + 7) / 8;
  const int grid = (int)std::min<int64_t>((n + 255) / 256, 4096);
  gather_rows_kernel<<<grid, 256, 0, st>>>(syn, sb, targets, p->cfg.n_out, n_set, rows, n, p->gathered, p->tgt,
                                           p->d_bad);
  SQ_CUDA(cudaGetLastError());
  if ((rc = train_rows(p, p->gathered, n, lr, loss_out, st))) return rc;
  if (loss_out) {
    int bad = 0;
    SQ_CUDA(cudaMemcpy(&bad, p->d_bad, sizeof(int), cudaMemcpyDeviceToHost));
    if (bad) {
      cudaMemset(p->d_bad, 0, sizeof(int));
      return sfail(TQEC_ERR_INVALID, "a row index was outside the training set");
    }
  }
  return TQEC_OK;
}

int tqec_mlp_infer(tqec_mlp* p, const uint8_t* syn, int64_t n, int32_t* class_out, float* conf_out, void* stream) {
  if (!p || (n > 0 && !syn) || n < 0) return sfail(TQEC_ERR_INVALID, "bad argument");
  std::lock_guard<std::mutex> lk(p->mu);
  SQ_CUDA(cudaSetDevice(p->cfg.device));
  cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
  const int64_t chunk = 65536;
  int rc = ensure_cap(p, std::min(n, chunk));
  if (rc) return rc;
  const int sb = (p->cfg.n_in + 7) / 8;
  const bool host_in = !dev_ptr(syn);
  const bool host_cls = class_out && !dev_ptr(class_out);
  const bool host_conf = conf_out && !dev_ptr(conf_out);
  for (int64_t r0 = 0; r0 < n; r0 += chunk) {
    const int64_t m = std::min(chunk, n - r0);
    const uint8_t* ds;
    if ((rc = stage_syn(p, syn + r0 * sb, m, st, &ds))) return rc;
    int32_t* c = host_cls ? p->cls : (class_out ? class_out + r0 : nullptr);
    float* f = host_conf ? p->conf : (conf_out ? conf_out + r0 : nullptr);
    const tqec::FusedGate g{0.f, c, f, nullptr, nullptr};
    bool gated = false;
    if ((rc = forward_infer(p, ds, m, st, c ? &g : nullptr, &gated))) return rc;
    if (!gated) SQ_CUDA(tqec::gate_rows(p->logits, p->out_pad, m, p->cfg.n_out, 0.f, c, f, nullptr, nullptr, st));
    if (host_cls) SQ_CUDA(cudaMemcpyAsync(class_out + r0, p->cls, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, st));
    if (host_conf) SQ_CUDA(cudaMemcpyAsync(conf_out + r0, p->conf, sizeof(float) * m, cudaMemcpyDeviceToHost, st));
    if (host_in || host_cls || host_conf) SQ_CUDA(cudaStreamSynchronize(st));
  }
  if (!stream) return check_device_error(p, st);
  return TQEC_OK;
}

int tqec_gated_decode(tqec_mlp* p, tqec_program* prog, float threshold, const uint8_t* syn, int64_t n,
                      int32_t* class_out, int64_t* n_fallback_out, void* stream) {
  if (!p || !prog || !class_out || (n > 0 && !syn) || n < 0) return sfail(TQEC_ERR_INVALID, "bad argument");
  tqec_program_info_t info;
  int rc = tqec_program_info(prog, &info);
  if (rc) return rc;
  if (info.n_syndrome != p->cfg.n_in || info.n_classes != p->cfg.n_out)
    return sfail(TQEC_ERR_INVALID, "surrogate and program disagree on syndrome bits or classes");
  std::lock_guard<std::mutex> lk(p->mu);
  SQ_CUDA(cudaSetDevice(p->cfg.device));
  cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
  const int64_t chunk = 65536;
  if ((rc = ensure_cap(p, std::min(n, chunk)))) return rc;
  const int sb = (p->cfg.n_in + 7) / 8;
  const bool host_cls = !dev_ptr(class_out);
  const int64_t n_chunks = (n + chunk - 1) / chunk;
  if (n_chunks > p->h_counts_cap) {
    if (p->h_counts) cudaFreeHost(p->h_counts);
    p->h_counts = nullptr;
    p->h_counts_cap = 0;
    SQ_CUDA(cudaMallocHost(&p->h_counts, sizeof(int32_t) * n_chunks));
    p->h_counts_cap = n_chunks;
  }
  // per chunk, all stream-ordered: the forward pass and the gate write the
  // surrogate's class of every row and list the rows below the threshold;
  // the exact contraction then overwrites the classes of the listed rows
  // (tqec_decode_rows, no host round trip), and the chunk's list length is
  // copied to a pinned word for tqec_gated_last_fallback
  for (int64_t c = 0; c < n_chunks; ++c) {
    const int64_t r0 = c * chunk;
    const int64_t m = std::min(chunk, n - r0);
    const uint8_t* ds;
    if ((rc = stage_syn(p, syn + r0 * sb, m, st, &ds))) return rc;
    int32_t* cls = host_cls ? p->cls : class_out + r0;
    SQ_CUDA(cudaMemsetAsync(p->count, 0, sizeof(int32_t), st));
    const tqec::FusedGate g{threshold, cls, p->conf, p->list, p->count};
    bool gated = false;
    if ((rc = forward_infer(p, ds, m, st, &g, &gated))) return rc;
    if (!gated)
      SQ_CUDA(tqec::gate_rows(p->logits, p->out_pad, m, p->cfg.n_out, threshold, cls, p->conf, p->list, p->count, st));
    rc = tqec_decode_rows(prog, ds, p->list, p->count, m, p->fallback_hint > 0 ? p->fallback_hint : m / 16, cls, st);
    if (rc) return rc;
    SQ_CUDA(cudaMemcpyAsync(p->h_counts + c, p->count, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    if (host_cls) {
      SQ_CUDA(cudaMemcpyAsync(class_out + r0, p->cls, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, st));
      SQ_CUDA(cudaStreamSynchronize(st));  // p->cls is reused by the next chunk
    }
  }
  p->last_chunks = n_chunks;
  if (n_fallback_out || !stream) {
    SQ_CUDA(cudaStreamSynchronize(st));
    int64_t total = 0;
    for (int64_t c = 0; c < n_chunks; ++c) total += p->h_counts[c];
    if (n_chunks > 0) p->fallback_hint = std::max<int64_t>(1, total / n_chunks);
    if (n_fallback_out) *n_fallback_out = total;
  }
  if (!stream) return check_device_error(p, st);
  return TQEC_OK;
}

int tqec_gated_last_fallback(tqec_mlp* p, int64_t* n_fallback) {
  if (!p || !n_fallback) return sfail(TQEC_ERR_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lk(p->mu);
  int64_t total = 0;
  for (int64_t c = 0; c < p->last_chunks; ++c) total += p->h_counts[c];
  if (p->last_chunks > 0) p->fallback_hint = std::max<int64_t>(1, total / p->last_chunks);
  *n_fallback = total;
  return TQEC_OK;
}

int tqec_mlp_save(tqec_mlp* p, const char* path) {
  if (!p || !path) return sfail(TQEC_ERR_INVALID, "NULL argument");
  std::vector<float> h(p->n_params);
  int rc = tqec_mlp_get_params(p, h.data(), (int64_t)p->n_params);
  if (rc) return rc;
  FILE* f = std::fopen(path, "wb");
  if (!f) return sfail(TQEC_ERR_IO, std::string("cannot write ") + path);
  char hdr[256];
  std::snprintf(hdr, sizeof(hdr),
                "{\"format\": \"tqec-mlp-1\", \"n_in\": %d, \"hidden\": %d, \"n_layers\": %d, \"n_out\": %d, "
                "\"n_params\": %zu}\n",
                p->cfg.n_in, p->cfg.hidden, p->cfg.n_layers, p->cfg.n_out, p->n_params);
  std::fputs(hdr, f);
  const size_t w = std::fwrite(h.data(), sizeof(float), h.size(), f);
  std::fclose(f);
  return w == h.size() ? TQEC_OK : sfail(TQEC_ERR_IO, "short write");
}

int tqec_mlp_load(tqec_mlp* p, const char* path) {
  if (!p || !path) return sfail(TQEC_ERR_INVALID, "NULL argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return sfail(TQEC_ERR_IO, std::string("cannot read ") + path);
  char hdr[512];
  if (!std::fgets(hdr, sizeof(hdr), f)) {
    std::fclose(f);
    return sfail(TQEC_ERR_IO, "missing header");
  }
  int n_in = 0, hidden = 0, layers = 0, n_out = 0;
  size_t np = 0;
  if (std::sscanf(hdr, "{\"format\": \"tqec-mlp-1\", \"n_in\": %d, \"hidden\": %d, \"n_layers\": %d, \"n_out\": %d, "
                       "\"n_params\": %zu}", &n_in, &hidden, &layers, &n_out, &np) != 5 ||
      n_in != p->cfg.n_in || hidden != p->cfg.hidden || layers != p->cfg.n_layers || n_out != p->cfg.n_out ||
      np != p->n_params) {
    std::fclose(f);
    return sfail(TQEC_ERR_INVALID, "checkpoint does not match this surrogate's shape");
  }
  std::vector<float> h(np);
  const size_t r = std::fread(h.data(), sizeof(float), np, f);
  std::fclose(f);
  if (r != np) return sfail(TQEC_ERR_IO, "short read");
  return tqec_mlp_set_params(p, h.data(), (int64_t)np);
}

}  // extern "C"
