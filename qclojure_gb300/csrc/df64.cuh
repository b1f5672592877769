// Double-float arithmetic for complex128 gate passes on GB300.
//
// On this part the FP64 pipe delivers about 1/58 of the FP32 FMA rate (a DFMA
// probe measured 1.19 TFLOP/s against 69 TFLOP/s for FFMA), so a c128 gate
// pass written in FP64 is bound by the FP64 pipe long before HBM. Here every
// real number is an unevaluated sum hi + lo of two floats (about 48 significand
// bits), every product is formed exactly with an FMA error term (Dekker /
// Ogita-Rump-Oishi TwoProduct), and every sum keeps its rounding error with
// Knuth's TwoSum. The conversions between IEEE doubles in memory and float pairs
// use integer operations only, so a pass issues no FP64 instruction at all.
//
// Accuracy: each product-sum carries a relative error of a few 2^-48 of the
// magnitudes involved; amplitudes are bounded by 1, so the absolute error per
// gate is below 1e-14. Inputs must satisfy |x| < 2^127 (float exponent range);
// magnitudes below 2^-126 are flushed to zero (absolute error < 1e-38).
#pragma once

#ifndef __CUDACC_RTC__
#include <cstdint>
#endif

namespace qg {

struct dfc {  // complex double-float: (re.hi, re.lo, im.hi, im.lo)
  float rh, rl, ih, il;
};

// IEEE double -> (hi, lo): hi keeps the leading 24 significand bits (truncated),
// lo the remaining 29 bits rounded to a float. Integer operations plus one
// int->float conversion; no FP64 instruction.
__device__ __forceinline__ void d2f2(double d, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
  const unsigned e = (hw >> 20) & 0x7FFu;
  const unsigned t = __funnelshift_l(lw, hw, 3);  // upper word of (hw:lw) << 3
  const unsigned hib = ((t + 0x40000000u) & 0x7FFFFFFFu) | (hw & 0x80000000u);
  hi = (e > 896u) ? __uint_as_float(hib) : 0.0f;
  const float r = __uint2float_rn(lw & 0x1FFFFFFFu);
  const unsigned sb = ((e - 948u) << 23) | (hw & 0x80000000u);  // +-2^(e-1075)
  lo = (e > 948u) ? r * __uint_as_float(sb) : 0.0f;
}

// (hi, lo) with |lo| <= ulp(hi)/2 -> nearest IEEE double. The double is built
// from hi's bits; lo is added as an integer number of double ulps of hi (the
// ulp of the lower binade when hi is a power of two and lo points to zero).
__device__ __forceinline__ double f22d(float h, float l) {
  const unsigned hb = __float_as_uint(h);
  const unsigned eh = (hb >> 23) & 0xFFu;
  const unsigned hw = (hb & 0x80000000u) | (((hb & 0x7FFFFFFFu) >> 3) + (896u << 20));
  const unsigned lw = hb << 29;
  const long long bits = (long long)(((unsigned long long)hw << 32) | lw);
  const bool opp = ((__float_as_uint(l) ^ hb) >> 31) != 0;
  const bool pow2 = (hb & 0x7FFFFFu) == 0u;
  const int se = 306 - (int)eh + ((pow2 && opp) ? 1 : 0);  // biased exponent of 2^(179-eh[+1])
  const float c = (se >= 1 && se <= 254) ? l * __int_as_float(se << 23) : 0.0f;
  const long long ci = (long long)__float2int_rn(c);
  const long long delta = (hb >> 31) ? -ci : ci;
  return (eh == 0u) ? 0.0 : __longlong_as_double(bits + delta);
}

__device__ __forceinline__ dfc load_dfc(double2 v) {
  dfc r;
  d2f2(v.x, r.rh, r.rl);
  d2f2(v.y, r.ih, r.il);
  return r;
}
__device__ __forceinline__ double2 store_dfc(const dfc& v) { return make_double2(f22d(v.rh, v.rl), f22d(v.ih, v.il)); }

// a*u + b*v for double-float a, b, u, v; result normalised (|lo| <= ulp(hi)/2).
__device__ __forceinline__ void lin2(float ah, float al, float uh, float ul, float bh, float bl, float vh, float vl,
                                     float& yh, float& yl) {
  const float p1 = ah * uh;
  float e1 = fmaf(ah, uh, -p1);
  e1 = fmaf(ah, ul, e1);
  e1 = fmaf(al, uh, e1);
  const float p2 = bh * vh;
  float e2 = fmaf(bh, vh, -p2);
  e2 = fmaf(bh, vl, e2);
  e2 = fmaf(bl, vh, e2);
  const float s = p1 + p2;  // TwoSum(p1, p2)
  const float bb = s - p1;
  const float err = (p1 - (s - bb)) + (p2 - bb);
  const float t = (e1 + e2) + err;
  yh = s + t;  // Fast2Sum renormalisation
  yl = t - (yh - s);
}

// a*u for double-float a, u (normalised result)
__device__ __forceinline__ void mul1(float ah, float al, float uh, float ul, float& yh, float& yl) {
  const float p = ah * uh;
  float e = fmaf(ah, uh, -p);
  e = fmaf(ah, ul, e);
  e = fmaf(al, uh, e);
  yh = p + e;
  yl = e - (yh - p);
}

// (xh + xl) + (yh + yl), normalised
__device__ __forceinline__ void add2(float xh, float xl, float yh, float yl, float& zh, float& zl) {
  const float s = xh + yh;
  const float bb = s - xh;
  const float err = (xh - (s - bb)) + (yh - bb);
  const float t = (xl + yl) + err;
  zh = s + t;
  zl = t - (zh - s);
}

// complex g*x, g given as (re.hi, re.lo, im.hi, im.lo)
__device__ __forceinline__ dfc cmul_df(float grh, float grl, float gih, float gil, const dfc& x) {
  dfc y;
  lin2(grh, grl, x.rh, x.rl, -gih, -gil, x.ih, x.il, y.rh, y.rl);
  lin2(grh, grl, x.ih, x.il, gih, gil, x.rh, x.rl, y.ih, y.il);
  return y;
}

}  // namespace qg
