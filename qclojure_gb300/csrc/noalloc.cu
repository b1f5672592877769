// Fixed device scratch for qg_state_sample_noalloc.
//
// The shot sampler needs per-chunk and per-block integer prefix data plus a
// compensated FP64 total (sampler_scratch_bytes). qg_state_sample takes that
// from the stream-ordered pool on every call; the no-allocation entry point
// uses this file-scope array instead, so its size bounds the state it can
// sample: 2^24 amplitudes (kNoAllocSampleMaxQubits).
#include <cuda_runtime.h>

#include <mutex>

#include "qgpu_internal.h"

namespace qg {
namespace {

// Sampler geometry for n >= 13 qubits: 32 amplitudes per chunk, 256 chunks per
// block, so 2^(n-5) chunk sums and 2^(n-13) block sums / prefixes / FP64 block sums.
constexpr size_t sampler_bytes_at(int n) {
  return sizeof(unsigned long long) * ((1ULL << (n - 5)) + (1ULL << (n - 13)) + (1ULL << (n - 13)) + 1) +
         sizeof(double) * ((1ULL << (n - 13)) + 2) + 256;
}
// Sampler region, then 256 bytes that hold the FP64 total probability.
constexpr size_t kScratchBytes = (sampler_bytes_at(kNoAllocSampleMaxQubits) + 255) / 256 * 256 + 256;

static __device__ __align__(256) unsigned char g_sample_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

}  // namespace

cudaError_t noalloc_sample_scratch(int device, void** ptr, size_t* bytes) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[device]) {
    // The caller has made `device` current; the symbol resolves in that device's context.
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_sample_scratch);
    if (e != cudaSuccess) return e;
    g_addr[device] = p;
  }
  *ptr = g_addr[device];
  *bytes = kScratchBytes;
  return cudaSuccess;
}

}  // namespace qg
