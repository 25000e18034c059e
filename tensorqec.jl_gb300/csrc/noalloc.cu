// noalloc.cu -- a float64 batch decode that performs no device allocation.
//
// Some callers of this library cannot allocate device memory while they
// decode: a real-time decoding loop that runs beside the quantum hardware
// must not stall or fail on an allocation, and a process whose device memory
// is already reserved in full by another allocator (a framework's caching
// pool, for example) has none left for cudaMalloc.  tqec_decode_batch may
// allocate (staging buffers, the per-block arena of programs whose working
// set does not fit shared memory), so those callers use
// tqec_decode_batch_noalloc instead.  Its only scratch memory is the
// file-scope device array below: kNoallocScratchBytes (32 MiB), which every
// GPU that loads this library holds until the process exits.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "../../include/tqec_gb300.h"
#include "contract.cuh"
#include "program_view.h"

namespace tqec {
std::string& last_error_ref();
}  // namespace tqec

namespace {

constexpr size_t kNoallocScratchBytes = size_t(32) << 20;

// The per-block contraction arenas of tqec_decode_batch_noalloc.  Host code
// must not pass this symbol to a kernel: on the host it names a stand-in, not
// the device array.  Its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices] = {};

int nfail(int code, const std::string& m) {
  tqec::last_error_ref() = m;
  return code;
}

// Device address of the scratch array on `device`, which must be current.
// Resolved once per device and cached for the life of the process: a
// cudaDeviceReset by the caller destroys the context the address belongs to,
// so this entry point must not be called on that device after such a reset.
int scratch_address(int device, void** out) {
  if (device < 0 || device >= kMaxDevices) return nfail(TQEC_ERR_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return nfail(TQEC_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_scratch_addr[device] = p;
  }
  *out = g_scratch_addr[device];
  return TQEC_OK;
}

// True when p is device (or managed) memory of `device`: a buffer on another
// GPU would be dereferenced directly by the kernel, which faults without peer
// access, so it is rejected like a host pointer.
bool on_device(const void* p, int device) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) && at.device == device;
}

}  // namespace

extern "C" int tqec_decode_batch_noalloc(tqec_program* prog, const uint8_t* syndromes, int64_t n,
                                         int32_t* class_out, double* logp_out, void* stream) {
  if (!prog || n < 0 || (n > 0 && (!syndromes || !class_out)))
    return nfail(TQEC_ERR_INVALID, "bad argument");
  tqec::ProgramF64View v;
  int rc = tqec::program_f64_view(prog, &v);
  if (rc) return nfail(rc, "bad program");
  // a most-probable-configuration program returns assignments, not classes
  // (tqec_map_decode_batch); tqec_decode_batch rejects it the same way
  if (v.args.map_mode)
    return nfail(TQEC_ERR_INVALID, "a TQEC_FLAG_MAP program decodes with tqec_map_decode_batch");
  std::lock_guard<std::mutex> lk(*v.mu);
  cudaError_t e = cudaSetDevice(v.device);
  if (e != cudaSuccess) return nfail(TQEC_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  void* scratch = nullptr;
  if ((rc = scratch_address(v.device, &scratch))) return rc;
  if (n == 0) return TQEC_OK;
  if (!on_device(syndromes, v.device) || !on_device(class_out, v.device) ||
      (logp_out && !on_device(logp_out, v.device)))
    return nfail(TQEC_ERR_INVALID,
                 "tqec_decode_batch_noalloc takes device pointers only, on the program's device");
  const size_t per_syndrome = size_t(v.args.arena_elems) * sizeof(double);
  if (per_syndrome > kNoallocScratchBytes)
    return nfail(TQEC_ERR_UNSUPPORTED,
                 "the program's float64 working set of " + std::to_string(per_syndrome) +
                     " bytes per syndrome exceeds the 33554432-byte scratch of tqec_decode_batch_noalloc");
  // syndromes per block: the program's float64 group, halved until one block fits
  int G = std::max(1, v.group);
  while (G > 1 && size_t(G) * per_syndrome > kNoallocScratchBytes) G >>= 1;
  int lg = 0;
  while ((1 << lg) < G) ++lg;
  const size_t smem = tqec::contract_smem_bytes(TQEC_F64, v.args.n_steps, v.args.syn_words, G, v.args.arena_elems,
                                                false, v.args.var_words);
  const int occ = tqec::contract_occupancy(TQEC_F64, v.threads, smem, v.args.map_mode != 0);
  if (occ < 1) return nfail(TQEC_ERR_UNSUPPORTED, "launch shape cannot be resident on this device");
  const int64_t by_scratch = int64_t(kNoallocScratchBytes / (size_t(G) * per_syndrome));
  const int64_t by_rows = (n + G - 1) / G;
  const int grid = int(std::max<int64_t>(1, std::min<int64_t>({by_rows, by_scratch, int64_t(occ) * v.sm_count})));
  tqec::KArgs a = v.args;
  a.G = G;
  a.lg = lg;
  a.syn = syndromes;
  a.n = n;
  a.row_offset = 0;
  a.list = nullptr;
  a.list_count = nullptr;
  a.arena_global = scratch;  // every arena element is written before it is read
  a.class_out = class_out;
  a.logp_out = logp_out;
  a.err_out = nullptr;
  a.recheck_margin = -1.0;
  a.recheck_list = nullptr;
  a.recheck_count = nullptr;
  e = tqec::contract_launch(TQEC_F64, a, grid, v.threads, smem, (cudaStream_t)stream);
  if (e != cudaSuccess) return nfail(TQEC_ERR_CUDA, std::string("contraction launch: ") + cudaGetErrorString(e));
  if (!stream) {
    e = cudaStreamSynchronize(nullptr);
    if (e != cudaSuccess) return nfail(TQEC_ERR_CUDA, std::string("synchronize: ") + cudaGetErrorString(e));
  }
  return TQEC_OK;
}
