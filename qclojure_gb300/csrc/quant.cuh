// Probabilities and their 2^-62 quantisation on the integer pipes.
//
// The sampler, the marginals and the reductions work with p = re^2 + im^2 in FP64
// (the oracle's arithmetic) and with floor(p 2^62), the integer the sampler sums. On
// this part the FP64 pipe runs at about 1/58 of the FP32 rate, and five FP64
// instructions per amplitude (two conversions, two squares, the sum; then the scaling
// and the conversion of the quantisation) bound the whole sampler by it. Two of them
// need no floating point at all:
//   * qg_quant62(p): p 2^62 is exact (a power of two), and the conversion truncates, so
//     floor(p 2^62) is the double's significand shifted by its exponent;
//   * qg_sq_float(x): (double)x * (double)x for a float x is exact (a 24-bit significand
//     squared fits in 53 bits), so the double is assembled from the integer square.
// For complex64 that leaves one FP64 instruction per amplitude (the rounded sum);
// every value is bit-identical to the FP64 expressions (tests/test_quant.py checks
// them against those expressions over random and edge-case inputs).
//
// Host and device: the CPU test compiles this header with a host compiler.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define QG_QHD __host__ __device__ __forceinline__
#else
#define QG_QHD inline
#endif

QG_QHD uint64_t qg_bits_of(double d) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t b;
  std::memcpy(&b, &d, 8);
  return b;
#endif
}
QG_QHD double qg_double_of(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double d;
  std::memcpy(&d, &b, 8);
  return d;
#endif
}
QG_QHD uint32_t qg_bits_of(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t b;
  std::memcpy(&b, &f, 4);
  return b;
#endif
}
QG_QHD int qg_clz64(uint64_t v) {  // v != 0
#if defined(__CUDA_ARCH__)
  return __clzll((long long)v);
#else
  return __builtin_clzll(v);
#endif
}

// floor(p 2^62) for p >= 0, as (unsigned long long)(p * 2^62) for 0 <= p < 4, 0 for
// NaN, saturated above (where the conversion saturates too).
QG_QHD uint64_t qg_quant62(double p) {
  const uint64_t b = qg_bits_of(p);
  const int e = (int)((b >> 52) & 0x7FF);
  const uint64_t frac = b & 0xFFFFFFFFFFFFFull;
  if (b >> 63) return 0ull;                     // negative (and -0, -infinity)
  if (e == 0x7FF) return frac ? 0ull : ~0ull;   // NaN, infinity
  if (e < 1013 - 52) return 0ull;               // p 2^62 < 1 (zero, subnormals)
  const uint64_t m = frac | (1ull << 52);       // p = m 2^(e - 1075), p 2^62 = m 2^(e - 1013)
  const int sh = e - 1013;
  if (sh > 11) return ~0ull;
  return sh >= 0 ? (m << sh) : (m >> -sh);
}

// (double)x * (double)x, exactly, without an FP64 instruction
QG_QHD double qg_sq_float(float x) {
  const uint32_t u = qg_bits_of(x) & 0x7FFFFFFFu;
  const uint32_t ef = u >> 23;
  if (ef == 0xFF) {  // NaN or infinity: the FP64 square of the same
    const double d = (double)x;
    return d * d;
  }
  const uint32_t m = ef ? ((u & 0x7FFFFFu) | 0x800000u) : (u & 0x7FFFFFu);
  if (m == 0) return 0.0;
  const int E = (ef ? (int)ef : 1) - 150;  // |x| = m 2^E
  const uint64_t M = (uint64_t)m * m;      // < 2^48, x^2 = M 2^(2E)
  const int nb = 64 - qg_clz64(M);         // significant bits of M
  const uint64_t mant = M << (53 - nb);    // leading one at bit 52 (exact: nb <= 48)
  const int exp = 2 * E + nb - 1;          // x^2 = 1.f 2^exp, within the normal range
  return qg_double_of(((uint64_t)(exp + 1023) << 52) | (mant & 0xFFFFFFFFFFFFFull));
}
