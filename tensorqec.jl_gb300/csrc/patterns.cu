// patterns.cu -- batched error-pattern reconstruction for CSS codes.
//
// Replaces error_pattern(pos, ct, syndrome) (src/decoding/tndecoder.jl:167-174)
// at batch rate.  The reference asks SCIP for any error consistent with the
// syndrome (ipdecoder.jl:150-169) and then adds logical operators until the
// pattern's class equals the decoded one.  Here the first part is a fixed
// GF(2) right inverse R of each check matrix (e = R s, precomputed on the
// host), with a consistency mask that flags syndromes no error produces, and
// the second part is the reference's fix-up loop: for each logical i, if
// lz_i . ex differs from the class's b_i add lx_i to ex; if lx_i . ez differs
// from a_i add lz_i to ez.
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "../../include/tqec_gb300.h"

namespace tqec {
std::string& last_error_ref();
}

namespace {

constexpr int kWords = 4;   // syndrome halves up to 256 bits
constexpr int kQWords = 8;  // error patterns up to 512 bits

int pfail(int code, const std::string& m) {
  tqec::last_error_ref() = m;
  return code;
}

struct PatternDev {
  int nq, nsx, nsz, k;
  const uint64_t* rz;    // nq rows x kWords: ex = rz * sz
  const uint64_t* rx;    // nq rows x kWords: ez = rx * sx
  const uint64_t* chk_z; // nsz rows x kWords: sz consistent iff every row has even overlap
  const uint64_t* chk_x;
  int n_chk_z, n_chk_x;
  const uint64_t* lx;    // k rows x kQWords
  const uint64_t* lz;
};

__device__ __forceinline__ int parity_words(const uint64_t* a, const uint64_t* b, int words) {
  int p = 0;
  for (int w = 0; w < words; ++w) p ^= __popcll(a[w] & b[w]) & 1;
  return p;
}

__global__ void patterns_kernel(PatternDev P, const uint8_t* __restrict__ syn, int syn_bytes,
                                const int32_t* __restrict__ cls, int64_t n, uint8_t* __restrict__ ex_out,
                                uint8_t* __restrict__ ez_out, int q_bytes, uint8_t* __restrict__ ok_out) {
  const int64_t r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (r >= n) return;
  uint64_t sx[kWords] = {0, 0, 0, 0}, sz[kWords] = {0, 0, 0, 0};
  const uint8_t* row = syn + r * syn_bytes;
  for (int j = 0; j < P.nsx + P.nsz; ++j) {
    const int b = (row[j >> 3] >> (j & 7)) & 1;
    if (!b) continue;
    if (j < P.nsx) sx[j >> 6] |= uint64_t(1) << (j & 63);
    else {
      const int jj = j - P.nsx;
      sz[jj >> 6] |= uint64_t(1) << (jj & 63);
    }
  }
  int ok = 1;
  for (int i = 0; i < P.n_chk_z; ++i) ok &= 1 - parity_words(P.chk_z + i * kWords, sz, kWords);
  for (int i = 0; i < P.n_chk_x; ++i) ok &= 1 - parity_words(P.chk_x + i * kWords, sx, kWords);
  uint64_t ex[kQWords] = {0}, ez[kQWords] = {0};
  for (int q = 0; q < P.nq; ++q) {
    if (parity_words(P.rz + q * kWords, sz, kWords)) ex[q >> 6] |= uint64_t(1) << (q & 63);
    if (parity_words(P.rx + q * kWords, sx, kWords)) ez[q >> 6] |= uint64_t(1) << (q & 63);
  }
  const int c = cls[r];
  for (int i = 0; i < P.k; ++i) {
    const int a_i = (c >> i) & 1;
    const int b_i = (c >> (P.k + i)) & 1;
    if (parity_words(P.lz + i * kQWords, ex, kQWords) != b_i)
      for (int w = 0; w < kQWords; ++w) ex[w] ^= P.lx[i * kQWords + w];
    if (parity_words(P.lx + i * kQWords, ez, kQWords) != a_i)
      for (int w = 0; w < kQWords; ++w) ez[w] ^= P.lz[i * kQWords + w];
  }
  for (int b = 0; b < q_bytes; ++b) {
    ex_out[r * q_bytes + b] = uint8_t(ex[b >> 3] >> ((b & 7) * 8));
    ez_out[r * q_bytes + b] = uint8_t(ez[b >> 3] >> ((b & 7) * 8));
  }
  if (ok_out) ok_out[r] = uint8_t(ok);
}

bool on_device(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

}  // namespace

struct tqec_patterns {
  PatternDev dev;
  int device = 0;
  void* buf = nullptr;
  cudaStream_t stream = nullptr;
  // staging for host pointers
  void* stage = nullptr;
  size_t stage_bytes = 0;
};

extern "C" {

int tqec_patterns_create(int32_t nq, int32_t n_sx, int32_t n_sz, int32_t k, const uint8_t* rx, const uint8_t* rz,
                         int32_t n_chk_x, const uint8_t* chk_x, int32_t n_chk_z, const uint8_t* chk_z,
                         const uint8_t* lx, const uint8_t* lz, int32_t device, tqec_patterns** out) {
  if (!out || nq < 1 || nq > 64 * kQWords || n_sx < 0 || n_sz < 0 || n_sx > 64 * kWords || n_sz > 64 * kWords ||
      k < 0 || 2 * k > 30 || (nq && (!rx || !rz)) || (k && (!lx || !lz)) || n_chk_x < 0 || n_chk_z < 0 ||
      (n_chk_x && !chk_x) || (n_chk_z && !chk_z))
    return pfail(TQEC_ERR_INVALID, "bad pattern-decoder arguments (nq <= 512, check halves <= 256 bits)");
  auto pack_rows = [](const uint8_t* m, int rows, int cols, int words) {
    std::vector<uint64_t> v(size_t(rows) * words, 0);
    for (int r = 0; r < rows; ++r)
      for (int c = 0; c < cols; ++c)
        if (m[size_t(r) * cols + c] & 1) v[size_t(r) * words + (c >> 6)] |= uint64_t(1) << (c & 63);
    return v;
  };
  std::vector<uint64_t> h_rz = pack_rows(rz, nq, n_sz, kWords), h_rx = pack_rows(rx, nq, n_sx, kWords);
  std::vector<uint64_t> h_cz = pack_rows(chk_z, n_chk_z, n_sz, kWords), h_cx = pack_rows(chk_x, n_chk_x, n_sx, kWords);
  std::vector<uint64_t> h_lx = pack_rows(lx, k, nq, kQWords), h_lz = pack_rows(lz, k, nq, kQWords);
  auto* p = new tqec_patterns();
  p->device = device;
  if (cudaSetDevice(device) != cudaSuccess) {
    delete p;
    return pfail(TQEC_ERR_CUDA, "cudaSetDevice");
  }
  const size_t words = h_rz.size() + h_rx.size() + h_cz.size() + h_cx.size() + h_lx.size() + h_lz.size() + 1;
  if (cudaMalloc(&p->buf, words * 8) != cudaSuccess) {
    delete p;
    return pfail(TQEC_ERR_OOM, "pattern tables");
  }
  uint64_t* d = static_cast<uint64_t*>(p->buf);
  size_t off = 0;
  auto put = [&](const std::vector<uint64_t>& v) {
    const uint64_t* at = d + off;
    if (!v.empty()) cudaMemcpy(d + off, v.data(), v.size() * 8, cudaMemcpyHostToDevice);
    off += v.size();
    return at;
  };
  p->dev.nq = nq;
  p->dev.nsx = n_sx;
  p->dev.nsz = n_sz;
  p->dev.k = k;
  p->dev.rz = put(h_rz);
  p->dev.rx = put(h_rx);
  p->dev.chk_z = put(h_cz);
  p->dev.chk_x = put(h_cx);
  p->dev.n_chk_z = n_chk_z;
  p->dev.n_chk_x = n_chk_x;
  p->dev.lx = put(h_lx);
  p->dev.lz = put(h_lz);
  cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
  if (cudaGetLastError() != cudaSuccess) {
    tqec_patterns_destroy(p);
    return pfail(TQEC_ERR_CUDA, "pattern setup");
  }
  *out = p;
  return TQEC_OK;
}

int tqec_patterns_destroy(tqec_patterns* p) {
  if (!p) return TQEC_OK;
  cudaSetDevice(p->device);
  if (p->stream) cudaStreamSynchronize(p->stream);
  cudaFree(p->buf);
  cudaFree(p->stage);
  if (p->stream) cudaStreamDestroy(p->stream);
  delete p;
  return TQEC_OK;
}

int tqec_patterns_decode(tqec_patterns* p, const uint8_t* syndromes, const int32_t* classes, int64_t n,
                         uint8_t* ex_out, uint8_t* ez_out, uint8_t* ok_out, void* stream) {
  if (!p || n < 0 || (n > 0 && (!syndromes || !classes || !ex_out || !ez_out)))
    return pfail(TQEC_ERR_INVALID, "bad argument");
  if (n == 0) return TQEC_OK;
  if (cudaSetDevice(p->device) != cudaSuccess) return pfail(TQEC_ERR_CUDA, "cudaSetDevice");
  cudaStream_t st = stream ? (cudaStream_t)stream : p->stream;
  const int sb = (p->dev.nsx + p->dev.nsz + 7) / 8;
  const int qb = (p->dev.nq + 7) / 8;
  const bool dev_all = on_device(syndromes) && on_device(classes) && on_device(ex_out) && on_device(ez_out) &&
                       (!ok_out || on_device(ok_out));
  const uint8_t* s = syndromes;
  const int32_t* c = classes;
  uint8_t *ex = ex_out, *ez = ez_out, *ok = ok_out;
  if (!dev_all) {
    // stage everything through one device buffer
    const size_t need = size_t(n) * (sb + 4 + 2 * qb + 1) + 64;
    if (need > p->stage_bytes) {
      cudaFree(p->stage);
      p->stage = nullptr;
      p->stage_bytes = 0;
      if (cudaMalloc(&p->stage, need) != cudaSuccess) return pfail(TQEC_ERR_OOM, "pattern staging");
      p->stage_bytes = need;
    }
    uint8_t* b = static_cast<uint8_t*>(p->stage);
    int32_t* dc = reinterpret_cast<int32_t*>(b);
    uint8_t* ds = b + size_t(n) * 4;
    ex = ds + size_t(n) * sb;
    ez = ex + size_t(n) * qb;
    ok = ez + size_t(n) * qb;
    cudaMemcpyAsync(dc, classes, size_t(n) * 4, cudaMemcpyDefault, st);
    cudaMemcpyAsync(ds, syndromes, size_t(n) * sb, cudaMemcpyDefault, st);
    s = ds;
    c = dc;
  }
  patterns_kernel<<<unsigned((n + 127) / 128), 128, 0, st>>>(p->dev, s, sb, c, n, ex, ez, qb, ok);
  if (cudaGetLastError() != cudaSuccess) return pfail(TQEC_ERR_CUDA, "pattern kernel launch");
  if (!dev_all) {
    cudaMemcpyAsync(ex_out, ex, size_t(n) * qb, cudaMemcpyDefault, st);
    cudaMemcpyAsync(ez_out, ez, size_t(n) * qb, cudaMemcpyDefault, st);
    if (ok_out) cudaMemcpyAsync(ok_out, ok, size_t(n), cudaMemcpyDefault, st);
  }
  if (!stream || !dev_all) {
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return pfail(TQEC_ERR_CUDA, cudaGetErrorString(e));
  }
  return TQEC_OK;
}

}  // extern "C"
