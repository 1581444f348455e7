// Allocation-free application of the bond operator (the derivative operator of a
// bond tensor, y = GL . x . GR) for callers that cannot allocate device memory.
//
// Who needs it: a caller that owns every byte of device memory through its own pool --
// an external Krylov solver running on CUDA.jl arrays, or code that records its launches
// into a CUDA graph, where a cudaMalloc inside the library is not allowed -- can still
// pass its own input and output buffers.  The one intermediate of the contraction,
// T = x . GR (Dl x w x Dr elements), lives in a file-scope device array instead of the
// context's scratch pool.
//
// Limits and rules:
//   * the array holds GB_NOALLOC_SCRATCH_BYTES (64 MiB); larger problems are rejected;
//   * every GPU that loads the library holds the array until the process exits;
//   * all calls share the array and it keeps the last call's contents; the first GEMM
//     overwrites all of T before the second reads it, so nothing has to start at zero;
//   * calls that overlap on the GPU (two streams, or two threads) race on the array;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current -- make that first call before
//     any stream capture begins;
//   * the address is cached for the life of the process; cudaDeviceReset unloads the
//     module and its array, so after a reset of a device this entry point must not be
//     called on that device again in the same process.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "gb_common.h"

namespace gb {
cudaError_t gemm_fp64_on_stream(cudaStream_t stream, int dtype, char opA, char opB, int64_t M,
                                int64_t N, int64_t K, cplx alpha, const void* A, int64_t lda,
                                const void* B, int64_t ldb, cplx beta, void* C, int64_t ldc);
}

namespace {

constexpr size_t GB_NOALLOC_SCRATCH_BYTES = size_t(64) << 20;

// In host code this name is only a stand-in for the symbol, not a device address: the
// device address is obtained once per device with cudaGetSymbolAddress below.
static __device__ __align__(256) double g_noalloc_scratch[GB_NOALLOC_SCRATCH_BYTES / sizeof(double)];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

// set-up, once per device, with that device current
cudaError_t scratch_address(int dev, void** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" int gb_c_apply_noalloc(const void* GL, const void* GR, const void* x, void* y,
                                  int64_t Dl, int64_t Dr, int64_t w, int dtype, void* stream) {
  if (!GL || !GR || !x || !y) {
    gb::set_last_error("gb_c_apply_noalloc: null buffer");
    return GB_ERR_ARG;
  }
  if (dtype != GB_F64 && dtype != GB_C128) {
    gb::set_last_error("gb_c_apply_noalloc: dtype must be GB_F64 or GB_C128");
    return GB_ERR_ARG;
  }
  if (Dl <= 0 || Dr <= 0 || w <= 0) {
    gb::set_last_error("gb_c_apply_noalloc: dimensions must be positive");
    return GB_ERR_ARG;
  }
  const size_t es = gb::elem_size(dtype);
  const double need = (double)Dl * (double)w * (double)Dr * (double)es;
  if (need > (double)GB_NOALLOC_SCRATCH_BYTES) {
    gb::set_last_error("gb_c_apply_noalloc: the intermediate needs " +
                       std::to_string((unsigned long long)need) +
                       " bytes but the static scratch holds " +
                       std::to_string((unsigned long long)GB_NOALLOC_SCRATCH_BYTES) +
                       " bytes (Dl*w*Dr*elem_size too large)");
    return GB_ERR_ARG;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess && (dev < 0 || dev >= kMaxDevices)) e = cudaErrorInvalidDevice;
  void* T = nullptr;
  if (e == cudaSuccess) e = scratch_address(dev, &T);
  if (e != cudaSuccess) {
    gb::set_last_error(std::string("gb_c_apply_noalloc: scratch address lookup failed: ") +
                       cudaGetErrorString(e));
    return GB_ERR_CUDA;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const gb::cplx one{1.0, 0.0}, zero{0.0, 0.0};
  // T[l', (w r)] = x[l', r'] GR[r', (w r)]
  e = gb::gemm_fp64_on_stream(s, dtype, 'N', 'N', Dl, w * Dr, Dr, one, x, Dl, GR, Dr, zero, T, Dl);
  // y[l, r] = GL[l, (l' w)] T[(l' w), r]
  if (e == cudaSuccess)
    e = gb::gemm_fp64_on_stream(s, dtype, 'N', 'N', Dl, Dr, Dl * w, one, GL, Dl, T, Dl * w, zero,
                                y, Dl);
  if (e != cudaSuccess) {
    gb::set_last_error(std::string("gb_c_apply_noalloc: launch failed: ") + cudaGetErrorString(e));
    return GB_ERR_CUDA;
  }
  return GB_OK;
}
