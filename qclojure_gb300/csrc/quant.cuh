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
// For complex64 that leaves one FP64 instruction per amplitude (the rounded sum).
// qg_quant62_sq_fast removes the rest for the amplitudes of large states: it forms
// floor(p 2^62) from fixed-point squares whenever a guard shows that the roundings of
// the FP64 expression cannot move the result (below). Every value is bit-identical
// to the FP64 expressions (tests/test_quant.py checks them against those expressions
// over random and edge-case inputs).
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

// ---------------------------------------------------------------------------
// floor(p 2^62) of p = re^2 + im^2 (the FP64 expression: for complex64 parts the
// squares are exact and only the sum rounds; for complex128 both squares and the sum
// round) without any floating-point instruction, for amplitudes with |re|, |im| below
// about 2^-10 (p below about 2^-19: every amplitude of a state of more than about 20
// qubits that is not concentrated on a few basis states).
//
// Each square is taken in fixed point with kQgFix = 20 bits below the 2^-62 grid,
// truncated: Xf <= x^2 2^82 < Xf + 1. With Sf = Xf + Yf the exact sum S satisfies
// Sf <= S 2^82 < Sf + 2, and the rounded FP64 value P differs from S by at most
// 2^-52 S (three roundings of relative size 2^-53 for complex128, one for complex64),
// which is below hb = (Sf >> 53) + 2 units. So when the fraction fr = Sf mod 2^20
// keeps 2 hb + 2 units from both ends of its range, P 2^62 lies strictly inside
// [Sf >> 20, (Sf >> 20) + 1) and floor(P 2^62) = Sf >> 20. The lower margin is not
// needed when Sf >> 20 is 0 (P >= 0; zero amplitudes take this case), nor for
// complex64 (qg_quant62_fix). Otherwise (large parts,
// NaN or infinity, or a sum within about 2^-18 of a grid point) the caller evaluates
// the FP64 expression instead. tests/test_quant.py checks the fast values against the
// FP64 expressions bit for bit.
// ---------------------------------------------------------------------------
constexpr int kQgFix = 20;

QG_QHD uint64_t qg_umulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// floor(x^2 2^82) for a float with |x| < 2^-10 (*big set otherwise). x = m 2^(ef - 150)
// with m the 24-bit significand; (m 2^7)^2 < 2^62 is the square 2^14 m^2, and
// x^2 2^82 = (m 2^7)^2 2^(2 ef - 232). Zeros and subnormals shift out entirely.
QG_QHD uint64_t qg_sq_fix(float x, bool* big) {
  const uint32_t u = qg_bits_of(x) & 0x7FFFFFFFu;
  *big = u >= (117u << 23);
  const uint32_t m7 = ((u << 7) & 0x3FFFFF80u) | 0x40000000u;
  const uint64_t M = (uint64_t)m7 * m7;
  const unsigned r = 232u - 2u * (u >> 23);  // wraps above 63 when *big: any value then
  return M >> (r < 63u ? r : 63u);           // M < 2^62: a shift by 63 leaves 0
}

// floor(x^2 2^82) for a double with |x| < 2^-10 (*big set otherwise), truncated from
// the high word of the 128-bit square of the significand: x = m 2^(e - 1075), m11 = m 2^11,
// x^2 2^82 = (m11^2 / 2^64) 2^(2 e - 2026).
QG_QHD uint64_t qg_sq_fix(double x, bool* big) {
  const uint64_t b = qg_bits_of(x) & 0x7FFFFFFFFFFFFFFFull;
  const int e = (int)(b >> 52);
  *big = e > 1012;
  const uint64_t m11 = (b << 11) | 0x8000000000000000ull;
  const uint64_t hi = qg_umulhi(m11, m11);
  const unsigned r = 2026u - 2u * (unsigned)e;  // wraps above 63 when *big: any value then
  return r > 63u ? 0ull : (hi >> r);             // hi >= 2^62: shifts of 64 and more give 0
}

// The fixed-point sum and its guard: *q = floor(p 2^62) when the result is true.
// EXACT_SQUARES (complex64 parts): the sum is the only rounding, and rounding is
// monotone, so P >= (Sf >> 20) 2^-62 (a double: below 2^53 units) holds without the
// lower margin.
template <bool EXACT_SQUARES>
QG_QHD bool qg_quant62_fix(uint64_t xf, uint64_t yf, uint64_t* q) {
  const uint64_t s = xf + yf;                                  // each below 2^62 on the fast path
  const uint32_t t = (uint32_t)(s >> 52);                      // 2 hb - 4
  const uint32_t fr = (uint32_t)s & ((1u << kQgFix) - 1u);
  *q = s >> kQgFix;
  const bool upper = fr + t <= (1u << kQgFix) - 6u;
  if (EXACT_SQUARES) return upper;
  return upper && (fr >= t + 4u || *q == 0);
}

// True when a part is at least 2^-10 in magnitude (outside the fast path's range): a
// cheap test a warp uses to send a group of amplitudes straight to the FP64 expression.
// Integer compares only (NaN parts are left to qg_sq_fix's own flag).
QG_QHD bool qg_part_big(float x) { return (qg_bits_of(x) & 0x7FFFFFFFu) >= (117u << 23); }
QG_QHD bool qg_part_big(double x) { return (qg_bits_of(x) & 0x7FFFFFFFFFFFFFFFull) >= (1013ull << 52); }

// floor(p 2^62) for p = re^2 + im^2 when the fast path applies (true), else false
template <typename R>
QG_QHD bool qg_quant62_sq_fast(R re, R im, uint64_t* q) {
  bool b0, b1;
  const uint64_t xf = qg_sq_fix(re, &b0), yf = qg_sq_fix(im, &b1);
  const bool ok = qg_quant62_fix<sizeof(R) == 4>(xf, yf, q);
  return ok && !b0 && !b1;
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
