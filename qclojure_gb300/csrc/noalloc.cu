// Fixed device scratch for qg_state_sample_noalloc.
//
// The shot sampler needs per-chunk and per-block integer prefix data plus a
// compensated FP64 total (sampler_scratch_bytes). qg_state_sample takes that
// from the stream-ordered pool on every call; the no-allocation entry point
// uses this file-scope array instead, so its size bounds the state it can
// sample: 2^24 amplitudes (kNoAllocSampleMaxQubits). Its size comes from the
// sampler's own layout function (sampler_scratch_bytes_at, qgpu_internal.h), so a
// change of the sampler geometry resizes it.
#include <cuda_runtime.h>

#include <mutex>

#include "qgpu_internal.h"

namespace qg {

// Sampler region, then 256 bytes that hold the FP64 total probability.
constexpr size_t kScratchBytes =
    (sampler_scratch_bytes_at(kNoAllocSampleMaxQubits) + 255) / 256 * 256 + 256;
static_assert(sampler_scratch_bytes_at(kNoAllocSampleMaxQubits) + 256 <= kScratchBytes,
              "the fixed sampler scratch must cover a state of kNoAllocSampleMaxQubits qubits");

namespace {

static __device__ __align__(256) unsigned char g_sample_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
// Per device: the array's address and the CUDA context it was resolved in. A device
// reset (cudaDeviceReset, or a library tearing the primary context down) gives the
// device a new context in which the array may live elsewhere, so the address is
// resolved again whenever the current context differs from the recorded one.
void* g_addr[kMaxDevices] = {};
void* g_ctx[kMaxDevices] = {};

typedef int (*CtxGetCurrentFn)(void** ctx);
CtxGetCurrentFn ctx_get_current() {
  static CtxGetCurrentFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return (CtxGetCurrentFn)f;
  }();
  return fn;
}

}  // namespace

cudaError_t noalloc_sample_scratch(int device, void** ptr, size_t* bytes) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  // The caller has made `device` current: make sure its context exists, then note it.
  cudaError_t e = cudaFree(nullptr);
  if (e != cudaSuccess) return e;
  void* cur = nullptr;
  if (CtxGetCurrentFn f = ctx_get_current()) {
    if (f(&cur) != 0) cur = nullptr;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[device] || !cur || cur != g_ctx[device]) {
    // The symbol resolves in the current context of `device`.
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_sample_scratch);
    if (e != cudaSuccess) return e;
    g_addr[device] = p;
    g_ctx[device] = cur;
  }
  *ptr = g_addr[device];
  *bytes = kScratchBytes;
  return cudaSuccess;
}

}  // namespace qg
