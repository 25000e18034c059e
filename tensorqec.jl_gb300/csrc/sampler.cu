// sampler.cu -- seeded code-capacity sampling and the Monte-Carlo loop on
// the GPU.
//
// Per sample and qubit one uniform u decides the Pauli error as in
// random_error_pattern(::IndependentDepolarizingError)
// (src/decoding/error_model.jl:97-117): Y if u < py, X if u < px + py, Z if
// u < px + py + pz.  The syndrome follows syndrome_extraction
// (error_model.jl:131-146: sx = Hx ez, sz = Hz ex) and the true logical
// class is the Julia linear index of mar for a = lx . ez, b = lz . ex, so a
// decoded class equals it exactly when check_logical_error
// (error_model.jl:179-181) finds no logical error.
//
// Uniforms come from Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel
// random numbers: as easy as 1, 2, 3", SC 2011): key = seed, counter =
// (sample index, qubit block, stream offset).  The stream is this library's
// own, not Julia's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/tqec_gb300.h"

namespace tqec {
std::string& last_error_ref();
}

namespace {

constexpr int kSynWords = 4;  // each check half <= 256 bits
constexpr int kMaxQ = 1024;

int sfail2(int code, const std::string& m) {
  tqec::last_error_ref() = m;
  return code;
}

struct SamplerDev {
  int nq, nsx, nsz, k;
  const uint64_t* colx;  // per qubit: X-check bits flipped by a Z error (kSynWords)
  const uint64_t* colz;  // per qubit: Z-check bits flipped by an X error
  const uint32_t* lmask; // per qubit: bit i = lx[i][q], bit 16+i = lz[i][q]
  const double* thr;     // per qubit: py, px+py, px+py+pz
};

__host__ __device__ inline void philox_round(uint32_t c[4], const uint32_t k[2]) {
  const uint64_t p0 = uint64_t(0xD2511F53u) * c[0];
  const uint64_t p1 = uint64_t(0xCD9E8D57u) * c[2];
  const uint32_t hi0 = uint32_t(p0 >> 32), lo0 = uint32_t(p0);
  const uint32_t hi1 = uint32_t(p1 >> 32), lo1 = uint32_t(p1);
  const uint32_t n0 = hi1 ^ c[1] ^ k[0];
  const uint32_t n2 = hi0 ^ c[3] ^ k[1];
  c[0] = n0;
  c[1] = lo1;
  c[2] = n2;
  c[3] = lo0;
}

__host__ __device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  uint32_t k[2] = {k0, k1};
  for (int r = 0; r < 10; ++r) {
    philox_round(c, k);
    k[0] += 0x9E3779B9u;
    k[1] += 0xBB67AE85u;
  }
}

__global__ void sample_kernel(SamplerDev S, uint64_t seed, uint64_t offset, int64_t n, uint8_t* __restrict__ syn,
                              int syn_bytes, int32_t* __restrict__ cls) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const uint64_t idx = offset + uint64_t(r);
  uint64_t sx[kSynWords] = {0, 0, 0, 0}, sz[kSynWords] = {0, 0, 0, 0};
  uint32_t a = 0, b = 0;
  uint32_t u[4];
  for (int q = 0; q < S.nq; ++q) {
    if ((q & 3) == 0) {
      u[0] = uint32_t(idx);
      u[1] = uint32_t(idx >> 32);
      u[2] = uint32_t(q >> 2);
      u[3] = 0x7E5Au;
      philox4x32_10(u, uint32_t(seed), uint32_t(seed >> 32));
    }
    const double x = (double(u[q & 3]) + 0.5) * 2.3283064365386963e-10;  // (u + 1/2) / 2^32
    const double* t = S.thr + 3 * q;
    int ex = 0, ez = 0;
    if (x < t[0]) { ex = 1; ez = 1; }
    else if (x < t[1]) { ex = 1; }
    else if (x < t[2]) { ez = 1; }
    if (ex) {
      for (int w = 0; w < kSynWords; ++w) sz[w] ^= S.colz[q * kSynWords + w];
      b ^= S.lmask[q] >> 16;
    }
    if (ez) {
      for (int w = 0; w < kSynWords; ++w) sx[w] ^= S.colx[q * kSynWords + w];
      a ^= S.lmask[q] & 0xFFFFu;
    }
  }
  uint8_t* row = syn + r * syn_bytes;
  for (int byte = 0; byte < syn_bytes; ++byte) {
    uint32_t v = 0;
    for (int bit = 0; bit < 8; ++bit) {
      const int j = byte * 8 + bit;
      int s = 0;
      if (j < S.nsx) s = int((sx[j >> 6] >> (j & 63)) & 1);
      else if (j < S.nsx + S.nsz) {
        const int jj = j - S.nsx;
        s = int((sz[jj >> 6] >> (jj & 63)) & 1);
      }
      v |= uint32_t(s) << bit;
    }
    row[byte] = uint8_t(v);
  }
  if (cls) cls[r] = int32_t(a | (b << S.k));
}

__global__ void count_mismatch_kernel(const int32_t* __restrict__ a, const int32_t* __restrict__ b, int64_t n,
                                      unsigned long long* __restrict__ count) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int v = (r < n && a[r] != b[r]) ? 1 : 0;
  const unsigned m = __ballot_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0 && m) atomicAdd(count, (unsigned long long)__popc(m));
}

}  // namespace

struct tqec_sampler {
  SamplerDev dev;
  int device = 0;
  int syn_bytes = 0;
  void* buf = nullptr;
  cudaStream_t stream = nullptr;
  // Monte-Carlo scratch (grown on demand)
  uint8_t* mc_syn = nullptr;
  int32_t* mc_true = nullptr;
  int32_t* mc_dec = nullptr;
  unsigned long long* mc_count = nullptr;
  int64_t mc_cap = 0;
};

extern "C" {

int tqec_sampler_create(int32_t nq, int32_t n_sx, int32_t n_sz, const uint8_t* hx, const uint8_t* hz, int32_t k,
                        const uint8_t* lx, const uint8_t* lz, const double* px, const double* py, const double* pz,
                        int32_t device, tqec_sampler** out) {
  if (!out || nq < 1 || nq > kMaxQ || n_sx < 0 || n_sz < 0 || n_sx > 64 * kSynWords || n_sz > 64 * kSynWords ||
      k < 0 || k > 15 || (n_sx && !hx) || (n_sz && !hz) || (k && (!lx || !lz)) || !px || !py || !pz)
    return sfail2(TQEC_ERR_INVALID, "bad sampler arguments (nq <= 1024, check halves <= 256, k <= 15)");
  std::vector<uint64_t> colx(size_t(nq) * kSynWords, 0), colz(size_t(nq) * kSynWords, 0);
  std::vector<uint32_t> lmask(nq, 0);
  std::vector<double> thr(size_t(nq) * 3);
  for (int q = 0; q < nq; ++q) {
    for (int i = 0; i < n_sx; ++i)
      if (hx[size_t(i) * nq + q] & 1) colx[size_t(q) * kSynWords + (i >> 6)] |= uint64_t(1) << (i & 63);
    for (int i = 0; i < n_sz; ++i)
      if (hz[size_t(i) * nq + q] & 1) colz[size_t(q) * kSynWords + (i >> 6)] |= uint64_t(1) << (i & 63);
    for (int i = 0; i < k; ++i) {
      if (lx[size_t(i) * nq + q] & 1) lmask[q] |= 1u << i;
      if (lz[size_t(i) * nq + q] & 1) lmask[q] |= 1u << (16 + i);
    }
    thr[3 * q] = py[q];
    thr[3 * q + 1] = px[q] + py[q];
    thr[3 * q + 2] = px[q] + py[q] + pz[q];
  }
  auto* s = new tqec_sampler();
  s->device = device;
  s->syn_bytes = (n_sx + n_sz + 7) / 8;
  if (cudaSetDevice(device) != cudaSuccess) {
    delete s;
    return sfail2(TQEC_ERR_CUDA, "cudaSetDevice");
  }
  const size_t bytes = colx.size() * 8 * 2 + lmask.size() * 4 + thr.size() * 8 + 64;
  if (cudaMalloc(&s->buf, bytes) != cudaSuccess) {
    delete s;
    return sfail2(TQEC_ERR_OOM, "sampler tables");
  }
  char* b = static_cast<char*>(s->buf);
  cudaMemcpy(b, thr.data(), thr.size() * 8, cudaMemcpyHostToDevice);
  s->dev.thr = reinterpret_cast<const double*>(b);
  b += thr.size() * 8;
  cudaMemcpy(b, colx.data(), colx.size() * 8, cudaMemcpyHostToDevice);
  s->dev.colx = reinterpret_cast<const uint64_t*>(b);
  b += colx.size() * 8;
  cudaMemcpy(b, colz.data(), colz.size() * 8, cudaMemcpyHostToDevice);
  s->dev.colz = reinterpret_cast<const uint64_t*>(b);
  b += colz.size() * 8;
  cudaMemcpy(b, lmask.data(), lmask.size() * 4, cudaMemcpyHostToDevice);
  s->dev.lmask = reinterpret_cast<const uint32_t*>(b);
  s->dev.nq = nq;
  s->dev.nsx = n_sx;
  s->dev.nsz = n_sz;
  s->dev.k = k;
  cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (cudaGetLastError() != cudaSuccess) {
    tqec_sampler_destroy(s);
    return sfail2(TQEC_ERR_CUDA, "sampler setup");
  }
  *out = s;
  return TQEC_OK;
}

int tqec_sampler_destroy(tqec_sampler* s) {
  if (!s) return TQEC_OK;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  cudaFree(s->buf);
  cudaFree(s->mc_syn);
  cudaFree(s->mc_true);
  cudaFree(s->mc_dec);
  cudaFree(s->mc_count);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return TQEC_OK;
}

int tqec_sample(tqec_sampler* s, uint64_t seed, uint64_t offset, int64_t n, uint8_t* syndromes_out,
                int32_t* class_out, void* stream) {
  if (!s || n < 0 || (n > 0 && !syndromes_out)) return sfail2(TQEC_ERR_INVALID, "bad argument");
  if (n == 0) return TQEC_OK;
  if (cudaSetDevice(s->device) != cudaSuccess) return sfail2(TQEC_ERR_CUDA, "cudaSetDevice");
  cudaPointerAttributes at;
  bool dev_out = cudaPointerGetAttributes(&at, syndromes_out) == cudaSuccess &&
                 (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged);
  cudaGetLastError();
  if (class_out) {
    cudaPointerAttributes ac;
    dev_out = dev_out && cudaPointerGetAttributes(&ac, class_out) == cudaSuccess &&
              (ac.type == cudaMemoryTypeDevice || ac.type == cudaMemoryTypeManaged);
    cudaGetLastError();
  }
  cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
  uint8_t* ds = syndromes_out;
  int32_t* dc = class_out;
  if (!dev_out) {
    if (n > s->mc_cap) {
      cudaFree(s->mc_syn);
      cudaFree(s->mc_true);
      cudaFree(s->mc_dec);
      s->mc_syn = nullptr;
      s->mc_true = s->mc_dec = nullptr;
      s->mc_cap = 0;
      if (cudaMalloc(&s->mc_syn, size_t(n) * s->syn_bytes) || cudaMalloc(&s->mc_true, size_t(n) * 4) ||
          cudaMalloc(&s->mc_dec, size_t(n) * 4))
        return sfail2(TQEC_ERR_OOM, "sampler staging");
      s->mc_cap = n;
    }
    ds = s->mc_syn;
    dc = class_out ? s->mc_true : nullptr;
  }
  sample_kernel<<<unsigned((n + 127) / 128), 128, 0, st>>>(s->dev, seed, offset, n, ds, s->syn_bytes, dc);
  if (cudaGetLastError() != cudaSuccess) return sfail2(TQEC_ERR_CUDA, "sampler launch");
  if (!dev_out) {
    cudaMemcpyAsync(syndromes_out, ds, size_t(n) * s->syn_bytes, cudaMemcpyDeviceToHost, st);
    if (class_out) cudaMemcpyAsync(class_out, dc, size_t(n) * 4, cudaMemcpyDeviceToHost, st);
  }
  if (!stream || !dev_out) {
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return sfail2(TQEC_ERR_CUDA, cudaGetErrorString(e));
  }
  return TQEC_OK;
}

int tqec_monte_carlo(tqec_sampler* s, tqec_program* prog, tqec_mlp* mlp, float threshold, uint64_t seed,
                     int64_t n_total, int64_t batch, int64_t* n_logical_errors, int64_t* n_fallback) {
  if (!s || !prog || n_total < 0 || batch <= 0 || !n_logical_errors) return sfail2(TQEC_ERR_INVALID, "bad argument");
  if (cudaSetDevice(s->device) != cudaSuccess) return sfail2(TQEC_ERR_CUDA, "cudaSetDevice");
  const int64_t cap = std::min<int64_t>(batch, std::max<int64_t>(n_total, 1));
  if (cap > s->mc_cap) {
    cudaFree(s->mc_syn);
    cudaFree(s->mc_true);
    cudaFree(s->mc_dec);
    s->mc_syn = nullptr;
    s->mc_true = s->mc_dec = nullptr;
    s->mc_cap = 0;
    if (cudaMalloc(&s->mc_syn, size_t(cap) * s->syn_bytes) || cudaMalloc(&s->mc_true, size_t(cap) * 4) ||
        cudaMalloc(&s->mc_dec, size_t(cap) * 4))
      return sfail2(TQEC_ERR_OOM, "Monte-Carlo buffers");
    s->mc_cap = cap;
  }
  if (!s->mc_count && cudaMalloc(&s->mc_count, sizeof(unsigned long long)) != cudaSuccess)
    return sfail2(TQEC_ERR_OOM, "Monte-Carlo counter");
  cudaStream_t st = s->stream;
  cudaMemsetAsync(s->mc_count, 0, sizeof(unsigned long long), st);
  int64_t fb_total = 0;
  for (int64_t done = 0; done < n_total; done += cap) {
    const int64_t m = std::min(cap, n_total - done);
    sample_kernel<<<unsigned((m + 127) / 128), 128, 0, st>>>(s->dev, seed, uint64_t(done), m, s->mc_syn,
                                                             s->syn_bytes, s->mc_true);
    if (cudaGetLastError() != cudaSuccess) return sfail2(TQEC_ERR_CUDA, "sampler launch");
    int rc;
    if (mlp) {
      int64_t nf = 0;
      rc = tqec_gated_decode(mlp, prog, threshold, s->mc_syn, m, s->mc_dec, &nf, st);
      fb_total += nf;
    } else {
      rc = tqec_decode_batch(prog, s->mc_syn, m, s->mc_dec, nullptr, nullptr, st);
    }
    if (rc) return rc;
    count_mismatch_kernel<<<unsigned((m + 255) / 256), 256, 0, st>>>(s->mc_true, s->mc_dec, m, s->mc_count);
  }
  unsigned long long h = 0;
  cudaMemcpyAsync(&h, s->mc_count, sizeof(h), cudaMemcpyDeviceToHost, st);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return sfail2(TQEC_ERR_CUDA, cudaGetErrorString(e));
  *n_logical_errors = int64_t(h);
  if (n_fallback) *n_fallback = fb_total;
  return TQEC_OK;
}

}  // extern "C"
