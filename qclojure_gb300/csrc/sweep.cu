// Kernels of the batched parameter sweep: many states of equal size run the same
// pass structure together (QAOA / VQE parameter sweeps, the loop of
// src/org/soulspace/qclojure/application/algorithm/variational_algorithm.clj:310-363).
//
//   k_batch_zero       every state of a slab to |0...0>
//   k_diag_expect      per (state, chunk of 4096 amplitudes): sum_i p_i f_g(i) for each
//                      coefficient group g of a diagonal Hamiltonian, where
//                      f_g(i) = sum_{t in g} (-1)^popc(i & z_t) is an integer (identity
//                      strings, z_t = 0, only add their count), so the
//                      energy is sum_g c_g * sum_i p_i f_g(i); partials are FP64
//                      (FP32 within 32-amplitude runs) and written per work item
//   k_diag_reduce      fixed-order FP64 (TwoSum) reduction of the partials per state
#include <atomic>
#include <cstdio>

#include "qgpu_internal.h"

namespace qg {

void count_launch(int k);

namespace {

constexpr int kSMs = 152;
constexpr int kChunkBits = 12;
constexpr int kMaxGroups = 4;
constexpr int kCountBits = 7;  // bit-sliced odd counts: at most 127 Z-strings per coefficient group

template <typename V>
__global__ void k_batch_zero(unsigned char* slab, uint64_t per_state, int nstates) {
  const uint64_t total = per_state * (uint64_t)nstates;
  V* s = reinterpret_cast<V*>(slab);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
    V v;
    v.x = (i % per_state) == 0 ? 1 : 0;
    v.y = 0;
    s[i] = v;
  }
}

struct DiagState {
  uint64_t zoff;      // first z-mask of this state in the z array
  int32_t ngroups;    // coefficient groups (<= kMaxGroups)
  int32_t gcount[kMaxGroups];  // Z-strings with at least one Z per group (their masks are in the z array)
  int32_t nid[kMaxGroups];     // identity strings per group: each adds +1 to f_g(i) for every i
};

__device__ __forceinline__ double p_of(double2 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ float p_of(float2 a) { return a.x * a.x + a.y * a.y; }

// one CTA of 256 threads per work item (state, chunk); 16 amplitudes per thread,
// i = i0 + 256 q (q = 0..15), so bits 8-11 of i are q and i0 has none of them.
// A term's parity on amplitude q is parity(i0 & z) xor parity(q & z[8:12]); the
// second part is a 16-bit pattern over q (qmask, from the host). Odd counts are
// kept bit-sliced over the 16 amplitudes (bit q of slice k = bit k of the count
// of amplitude q), so a term costs one population count and a 16-lane ripple add
// instead of sixteen population counts.
template <typename V, typename R>
__global__ void __launch_bounds__(256) k_diag_expect(unsigned char* const* states, int n, const DiagState* __restrict__ ds,
                                                    const uint64_t* __restrict__ zmasks,
                                                    const uint32_t* __restrict__ qmasks, int nstates,
                                                    double* __restrict__ partial) {
  const uint64_t chunks = 1ULL << (n - kChunkBits);
  const uint64_t items = chunks * (uint64_t)nstates;
  __shared__ double red[kMaxGroups][8];
  for (uint64_t item = blockIdx.x; item < items; item += gridDim.x) {
    const int s = (int)(item / chunks);
    const uint64_t c = item - (uint64_t)s * chunks;
    const V* amps = reinterpret_cast<const V*>(states[s]);
    const DiagState d = ds[s];
    double acc[kMaxGroups] = {0, 0, 0, 0};
    const uint64_t i0 = (c << kChunkBits) + threadIdx.x;
    R p[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) p[q] = p_of(amps[i0 + (uint64_t)q * 256]);
    uint64_t zo = d.zoff;
    for (int g = 0; g < d.ngroups && g < kMaxGroups; ++g) {
      uint32_t sl[kCountBits];
#pragma unroll
      for (int k = 0; k < kCountBits; ++k) sl[k] = 0;
      for (int t = 0; t < d.gcount[g]; ++t) {
        const uint32_t m = qmasks[zo + t];
        uint32_t carry = (__popcll(i0 & zmasks[zo + t]) & 1) ? (~m & 0xFFFFu) : m;
#pragma unroll
        for (int k = 0; k < kCountBits; ++k) {
          const uint32_t nc = sl[k] & carry;
          sl[k] ^= carry;
          carry = nc;
        }
      }
      zo += d.gcount[g];
      // odd count of amplitude q from the slices (integer work), then one
      // multiply-add per amplitude: sum_q p_q (count_g - 2 odd_q)
      R run = 0;  // FP32 for complex64 within one 16-amplitude run, FP64 afterwards
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        int odd = 0;
#pragma unroll
        for (int k = 0; k < kCountBits; ++k) odd |= (int)((sl[k] >> q) & 1u) << k;
        run += p[q] * (R)(d.gcount[g] + d.nid[g] - 2 * odd);
      }
      acc[g] = (double)run;
    }
    // block reduction per group (fixed order)
#pragma unroll
    for (int g = 0; g < kMaxGroups; ++g) {
      double v = acc[g];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      if ((threadIdx.x & 31) == 0) red[g][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < kMaxGroups) {
      double t = 0;
      for (int w = 0; w < 8; ++w) t += red[threadIdx.x][w];
      partial[item * kMaxGroups + threadIdx.x] = t;
    }
    __syncthreads();
  }
}

// per state: sum of its chunks' partials in chunk order (TwoSum), then sum_g c_g * S_g
__global__ void k_diag_reduce(const double* __restrict__ partial, uint64_t chunks, int nstates,
                              const double* __restrict__ gcoef, double* __restrict__ energies) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nstates) return;
  double e = 0;
  for (int g = 0; g < kMaxGroups; ++g) {
    double hi = 0, lo = 0;
    for (uint64_t c = 0; c < chunks; ++c) {
      const double x = partial[((uint64_t)s * chunks + c) * kMaxGroups + g];
      const double t = hi + x, bp = t - hi;
      lo += (hi - (t - bp)) + (x - bp);
      hi = t;
    }
    e += gcoef[s * kMaxGroups + g] * (hi + lo);
  }
  energies[s] = e;
}

// Several slabs at once (one launch for every group of a sweep): slab g holds
// nstates[g] states of per[g] amplitudes; items are laid end to end.
template <typename V>
__global__ void k_multi_zero(const MultiZero z) {
  uint64_t total = 0;
  for (int g = 0; g < z.ngroups; ++g) total += z.per[g] * (uint64_t)z.nstates[g];
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t j = i;
    int g = 0;
    while (g + 1 < z.ngroups && j >= z.per[g] * (uint64_t)z.nstates[g]) {
      j -= z.per[g] * (uint64_t)z.nstates[g];
      ++g;
    }
    V v;
    v.x = (j % z.per[g]) == 0 ? 1 : 0;
    v.y = 0;
    reinterpret_cast<V*>(z.slab[g])[j] = v;
  }
}

}  // namespace

cudaError_t launch_multi_zero(const MultiZero& z, int precision, cudaStream_t st) {
  if (z.ngroups < 1 || z.ngroups > kMaxZeroGroups) return cudaErrorInvalidValue;
  uint64_t total = 0;
  for (int g = 0; g < z.ngroups; ++g) total += z.per[g] * (uint64_t)z.nstates[g];
  uint64_t grid = (total + 255) / 256;
  if (grid > (uint64_t)kSMs * 8) grid = (uint64_t)kSMs * 8;
  if (precision == QG_C64) k_multi_zero<float2><<<(unsigned)grid, 256, 0, st>>>(z);
  else k_multi_zero<double2><<<(unsigned)grid, 256, 0, st>>>(z);
  count_launch(1);
  return cudaGetLastError();
}

int diag_max_groups() { return kMaxGroups; }
size_t diag_state_bytes() { return sizeof(DiagState); }

cudaError_t launch_batch_zero(void* slab, int precision, int n, int nstates, cudaStream_t st) {
  const uint64_t per = 1ULL << n;
  const uint64_t total = per * (uint64_t)nstates;
  uint64_t grid = (total + 255) / 256;
  if (grid > (uint64_t)kSMs * 8) grid = (uint64_t)kSMs * 8;
  if (precision == QG_C64) k_batch_zero<float2><<<(unsigned)grid, 256, 0, st>>>((unsigned char*)slab, per, nstates);
  else k_batch_zero<double2><<<(unsigned)grid, 256, 0, st>>>((unsigned char*)slab, per, nstates);
  count_launch(1);
  return cudaGetLastError();
}

// host layout of DiagState: zoff, ngroups, gcount[kMaxGroups]
void fill_diag_state(void* out, uint64_t zoff, int ngroups, const int* gcount, const int* nid) {
  DiagState d{};
  d.zoff = zoff;
  d.ngroups = ngroups;
  for (int g = 0; g < kMaxGroups; ++g) {
    d.gcount[g] = g < ngroups ? gcount[g] : 0;
    d.nid[g] = g < ngroups ? nid[g] : 0;
  }
  *reinterpret_cast<DiagState*>(out) = d;
}

int diag_max_terms_per_group() { return (1 << kCountBits) - 1; }

uint32_t diag_qmask(uint64_t z) {
  const uint32_t zq = (uint32_t)(z >> 8) & 15u;
  uint32_t m = 0;
  for (uint32_t q = 0; q < 16; ++q) m |= (uint32_t)(__builtin_popcount(q & zq) & 1) << q;
  return m;
}

cudaError_t launch_diag_expect(void* const* d_states, int precision, int n, const void* d_diag, const uint64_t* d_z,
                               const uint32_t* d_qm, int nstates, double* d_partial, const double* d_gcoef,
                               double* d_energies, cudaStream_t st) {
  if (n < kChunkBits) return cudaErrorInvalidValue;
  const uint64_t chunks = 1ULL << (n - kChunkBits);
  uint64_t items = chunks * (uint64_t)nstates;
  uint64_t grid = items < (uint64_t)kSMs * 8 ? items : (uint64_t)kSMs * 8;
  if (precision == QG_C64)
    k_diag_expect<float2, float><<<(unsigned)grid, 256, 0, st>>>((unsigned char* const*)d_states, n,
                                                                 (const DiagState*)d_diag, d_z, d_qm, nstates,
                                                                 d_partial);
  else
    k_diag_expect<double2, double><<<(unsigned)grid, 256, 0, st>>>((unsigned char* const*)d_states, n,
                                                                   (const DiagState*)d_diag, d_z, d_qm, nstates,
                                                                   d_partial);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_diag_reduce<<<(nstates + 127) / 128, 128, 0, st>>>(d_partial, chunks, nstates, d_gcoef, d_energies);
  count_launch(2);
  return cudaGetLastError();
}

}  // namespace qg
