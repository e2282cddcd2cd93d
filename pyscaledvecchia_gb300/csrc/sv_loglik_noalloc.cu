// sv_vecchia_loglik_noalloc: the likelihood / score / Fisher evaluation of
// sv_vecchia_loglik for callers that cannot allocate device memory.
//
// Who needs it: an application that owns the GPU's memory through its own
// fixed pool (a serving process that reserves the device memory up front and
// grants libraries no allocation rights), or a caller that must not call
// cudaMalloc inside its loop because cudaMalloc synchronises the device and
// can fail under memory pressure at a point where the failure cannot be
// handled.  Such callers still pass their inputs and outputs; the scratch
// memory that sv_vecchia_loglik takes as a caller-provided workspace comes
// instead from a fixed array compiled into this library.
//
// The scratch is a file-scope static __device__ array of
// SV_NOALLOC_SCRATCH_BYTES (32 MiB): every GPU that loads the library holds
// it until the process exits.  Host code cannot use the array's name as a
// device address, so the first call on each device (with that device
// current) looks the address up with cudaGetSymbolAddress and keeps it; that
// first call should come before any stream capture.  Problems whose workspace
// (sv_loglik_workspace_bytes) exceeds the array are rejected with SV_ENOSPC
// before anything is launched.  Nothing here calls cudaMalloc, cudaFree or an
// allocating library routine.
//
// All calls share the one array and it keeps the last call's contents; the
// evaluation re-initialises everything that must start at zero (jitter flags,
// chunk maxima) and overwrites every per-block record before reading it.
// Calls that overlap on the GPU (different streams, or host threads issuing
// concurrently) race on the array and must be serialised by the caller.
#include <mutex>

#include "sv_common.cuh"

namespace {

static __device__ __align__(256) unsigned char sv_noalloc_scratch[SV_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set up once per
// device); returns SV_OK or a status.
int scratch_address(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return sv_record_cuda_error(e);
  if (dev < 0 || dev >= kMaxDevices) return SV_EINVAL;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, sv_noalloc_scratch);
    if (e != cudaSuccess) return sv_record_cuda_error(e);
    if (!p) return SV_ECUDA;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return SV_OK;
}

}  // namespace

extern "C" int sv_vecchia_loglik_noalloc(const sv_loglik_desc* desc, const double* theta,
                                         const double* X, const double* y, const double* Z,
                                         const int32_t* rowb, const int32_t* kb,
                                         const int32_t* nbr, const int32_t* chunk, double* out,
                                         int32_t* info, sv_stream_t stream) {
  if (!desc) return SV_EINVAL;
  const size_t need = sv_loglik_workspace_bytes(desc);
  if (need > (size_t)SV_NOALLOC_SCRATCH_BYTES) return SV_ENOSPC;
  void* scratch = nullptr;
  const int st = scratch_address(&scratch);
  if (st != SV_OK) return st;
  return sv_vecchia_loglik(desc, theta, X, y, Z, rowb, kb, nbr, chunk, out, info, scratch,
                           (size_t)SV_NOALLOC_SCRATCH_BYTES, stream);
}
