// Device prelude of the specialised pass kernels (pass_kernels.cpp).
//
// A tiled pass (one HBM read and write of the state that applies a run of
// gates, see tile.cu) is compiled into its own kernel: the generated code
// names every gate with its matrix entries as literals, its register slots and
// its conditions, so the gate run is straight-line code with no op dispatch.
// This file holds what every such kernel shares:
//   - run_pass<P>: the tile loop (cp.async double-buffered 16-byte copies into
//     an XOR-swizzled shared-memory tile, P::body applied to the tile, coalesced
//     16-byte stores), with the pass geometry supplied by P;
//   - the complex arithmetic of the two policies the generator emits:
//       complex128 as double-float pairs (hi + lo floats, about 48 bits) on the
//       FP32 pipes, with error-free products (FMA) and sums (TwoSum); results
//       are left unnormalised (the pair (s, t) of a rounded sum and its
//       collected error) and renormalised by the generated code after a few
//       operations on a register and before it is stored;
//       complex64 in FP32 with FMA contraction.
// It is compiled by NVRTC together with df64.cuh; it includes no system header.
#pragma once

#include "df64.cuh"

// Powers of w = exp(2 pi i / 2^30) in three tables of 1024 (w^(a 2^20), w^(b 2^10),
// w^c), double-float (re.hi, re.lo, im.hi, im.lo); filled by the host after the
// module is loaded. Runs of phases that are all such powers (the controlled
// phases of a QFT) add integer exponents and look the product up here.
__device__ float4 qgp_roots[3072];

namespace qgp {

using qg::dfc;
typedef unsigned long long u64;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// XOR swizzle of the shared-memory tile (16-byte units, 8 per 128-byte row);
// 8-byte amplitudes move in 16-byte pairs.
template <int E>
__device__ __forceinline__ int swz(int l) {
  if (E == 16) return l ^ ((l >> 3) & 7);
  return l ^ (((l >> 4) & 7) << 1);
}

// ---------------------------------------------------------------------------
// double-float scalars. A value is the unevaluated sum h + l of two floats.
// tprod: a * x with a a constant pair (ah, al) -> (p, e), p = fl(ah*xh) and e
// its exact error plus the cross terms ah*xl and al*xh (AL = false: al == 0).
// ---------------------------------------------------------------------------
template <bool AL>
__device__ __forceinline__ void tprod(float ah, float al, float xh, float xl, float& p, float& e) {
  p = ah * xh;
  e = fmaf(ah, xh, -p);
  e = fmaf(ah, xl, e);
  if (AL) e = fmaf(al, xh, e);
}
// Knuth's TwoSum: s = fl(a + b), e = (a + b) - s exactly.
__device__ __forceinline__ void tsum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
// a*x + b*y, unnormalised
template <bool AL, bool BL>
__device__ __forceinline__ void dot2(float ah, float al, float xh, float xl, float bh, float bl, float yh, float yl,
                                     float& sh, float& sl) {
  float p1, e1, p2, e2, err;
  tprod<AL>(ah, al, xh, xl, p1, e1);
  tprod<BL>(bh, bl, yh, yl, p2, e2);
  tsum(p1, p2, sh, err);
  sl = (e1 + e2) + err;
}
// x + y, unnormalised
__device__ __forceinline__ void add2(float xh, float xl, float yh, float yl, float& sh, float& sl) {
  float err;
  tsum(xh, yh, sh, err);
  sl = (xl + yl) + err;
}
// Fast2Sum: bring the collected error back under the leading float. The
// generated code applies it to a register after a few products (and before a
// register goes to shared memory): left to grow, the low float random-walks to
// a sizeable fraction of the high one and its roundings no longer average out
// (the state's norm then drifts by ~1e-11 over a thousand gates).
__device__ __forceinline__ void fast2(float& h, float& l) {
  const float s = h + l;
  l = l - (s - h);
  h = s;
}
// normalised pair (|l| <= ulp(h)/2) for the conversion to IEEE doubles
__device__ __forceinline__ void norm2(float& h, float& l) {
  float s, e;
  tsum(h, l, s, e);
  h = s;
  l = e;
}

// ---- complex double-float ------------------------------------------------
struct DF {
  typedef dfc V;
  static constexpr int E = 16;
  static __device__ __forceinline__ V ld_work(const unsigned char* b, int pos) {
    const float4 v = reinterpret_cast<const float4*>(b)[pos];
    return dfc{v.x, v.y, v.z, v.w};
  }
  static __device__ __forceinline__ void st_work(unsigned char* b, int pos, const V& v) {
    reinterpret_cast<float4*>(b)[pos] = make_float4(v.rh, v.rl, v.ih, v.il);
  }
  static __device__ __forceinline__ V ld_doubles(const unsigned char* b, int pos) {
    return qg::load_dfc(reinterpret_cast<const double2*>(b)[pos]);
  }
  static __device__ __forceinline__ void st_doubles(unsigned char* b, int pos, V v) {
    norm2(v.rh, v.rl);
    norm2(v.ih, v.il);
    reinterpret_cast<double2*>(b)[pos] = qg::store_dfc(v);
  }
  static __device__ __forceinline__ V renorm(V v) {
    fast2(v.rh, v.rl);
    fast2(v.ih, v.il);
    return v;
  }
  static __device__ __forceinline__ V zero() { return dfc{0.f, 0.f, 0.f, 0.f}; }
  static __device__ __forceinline__ V neg(const V& x) { return dfc{-x.rh, -x.rl, -x.ih, -x.il}; }
  static __device__ __forceinline__ V mul_i(const V& x) { return dfc{-x.ih, -x.il, x.rh, x.rl}; }
  static __device__ __forceinline__ V mul_mi(const V& x) { return dfc{x.ih, x.il, -x.rh, -x.rl}; }
};

// (gr + i gi) * x
template <bool RL, bool IL>
__device__ __forceinline__ dfc df_cmul(float grh, float grl, float gih, float gil, const dfc& x) {
  dfc y;
  dot2<RL, IL>(grh, grl, x.rh, x.rl, -gih, -gil, x.ih, x.il, y.rh, y.rl);
  dot2<RL, IL>(grh, grl, x.ih, x.il, gih, gil, x.rh, x.rl, y.ih, y.il);
  return y;
}
// (a + i a) x (NEG = false) or (a - i a) x (NEG = true), a a constant pair: the sum and
// the difference of x's parts first, then one product each (a T-gate phase)
template <bool AL, bool NEG>
__device__ __forceinline__ dfc df_cmul_diag(float ah, float al, const dfc& x) {
  float dh, dl, sh, sl;
  dfc y;
  if (!NEG) {  // a (xr - xi) + i a (xr + xi)
    add2(x.rh, x.rl, -x.ih, -x.il, dh, dl);
    add2(x.rh, x.rl, x.ih, x.il, sh, sl);
  } else {  // a (xr + xi) + i a (xi - xr)
    add2(x.rh, x.rl, x.ih, x.il, dh, dl);
    add2(x.ih, x.il, -x.rh, -x.rl, sh, sl);
  }
  tprod<AL>(ah, al, dh, dl, y.rh, y.rl);
  tprod<AL>(ah, al, sh, sl, y.ih, y.il);
  return y;
}
// a real scalar times x
template <bool AL>
__device__ __forceinline__ dfc df_scale(float ah, float al, const dfc& x) {
  dfc y;
  tprod<AL>(ah, al, x.rh, x.rl, y.rh, y.rl);
  tprod<AL>(ah, al, x.ih, x.il, y.ih, y.il);
  return y;
}
// y = a*x0 + b*x1 for complex constants a, b (8 floats: a.re h/l, a.im h/l, b.re h/l, b.im h/l)
__device__ __forceinline__ dfc df_row(float arh, float arl, float aih, float ail, float brh, float brl, float bih,
                                      float bil, const dfc& x0, const dfc& x1) {
  dfc y;
  float uh, ul, vh, vl;
  dot2<true, true>(arh, arl, x0.rh, x0.rl, -aih, -ail, x0.ih, x0.il, uh, ul);
  dot2<true, true>(brh, brl, x1.rh, x1.rl, -bih, -bil, x1.ih, x1.il, vh, vl);
  add2(uh, ul, vh, vl, y.rh, y.rl);
  dot2<true, true>(arh, arl, x0.ih, x0.il, aih, ail, x0.rh, x0.rl, uh, ul);
  dot2<true, true>(brh, brl, x1.ih, x1.il, bih, bil, x1.rh, x1.rl, vh, vl);
  add2(uh, ul, vh, vl, y.ih, y.il);
  return y;
}
// real 2x2 [[a, b], [c, d]]
template <bool AL, bool BL, bool CL, bool DL>
__device__ __forceinline__ void df_real(float ah, float al, float bh, float bl, float ch, float cl, float dh, float dl,
                                        dfc& x0, dfc& x1) {
  dfc y0, y1;
  dot2<AL, BL>(ah, al, x0.rh, x0.rl, bh, bl, x1.rh, x1.rl, y0.rh, y0.rl);
  dot2<AL, BL>(ah, al, x0.ih, x0.il, bh, bl, x1.ih, x1.il, y0.ih, y0.il);
  dot2<CL, DL>(ch, cl, x0.rh, x0.rl, dh, dl, x1.rh, x1.rl, y1.rh, y1.rl);
  dot2<CL, DL>(ch, cl, x0.ih, x0.il, dh, dl, x1.ih, x1.il, y1.ih, y1.il);
  x0 = y0;
  x1 = y1;
}
// [[c, c], [c, -c]] (Hadamard-shaped): the sum and difference first, one product each
template <bool CL>
__device__ __forceinline__ void df_hadamard(float ch, float cl, dfc& x0, dfc& x1) {
  float sh, sl, dh, dl;
  dfc y0, y1;
  add2(x0.rh, x0.rl, x1.rh, x1.rl, sh, sl);
  add2(x0.rh, x0.rl, -x1.rh, -x1.rl, dh, dl);
  tprod<CL>(ch, cl, sh, sl, y0.rh, y0.rl);
  tprod<CL>(ch, cl, dh, dl, y1.rh, y1.rl);
  add2(x0.ih, x0.il, x1.ih, x1.il, sh, sl);
  add2(x0.ih, x0.il, -x1.ih, -x1.il, dh, dl);
  tprod<CL>(ch, cl, sh, sl, y0.ih, y0.il);
  tprod<CL>(ch, cl, dh, dl, y1.ih, y1.il);
  x0 = y0;
  x1 = y1;
}
// [[1, 1], [1, -1]]: a Hadamard whose 1/sqrt 2 is applied later with the global factors
__device__ __forceinline__ void df_sumdiff(dfc& x0, dfc& x1) {
  dfc y0, y1;
  add2(x0.rh, x0.rl, x1.rh, x1.rl, y0.rh, y0.rl);
  add2(x0.rh, x0.rl, -x1.rh, -x1.rl, y1.rh, y1.rl);
  add2(x0.ih, x0.il, x1.ih, x1.il, y0.ih, y0.il);
  add2(x0.ih, x0.il, -x1.ih, -x1.il, y1.ih, y1.il);
  x0 = y0;
  x1 = y1;
}
// x + k*y for a constant pair k, unnormalised
template <bool KL>
__device__ __forceinline__ void axpy(float kh, float kl, float xh, float xl, float yh, float yl, float& zh, float& zl) {
  float p, e, err;
  tprod<KL>(kh, kl, yh, yl, p, e);
  tsum(xh, p, zh, err);
  zl = (xl + e) + err;
}
// [[1, b], [c, S]] (S = +-1): a real rotation with its diagonal factored out
template <bool BL, bool CL, bool NEG>
__device__ __forceinline__ void df_realunit(float bh, float bl, float ch, float cl, dfc& x0, dfc& x1) {
  dfc y0, y1;
  axpy<BL>(bh, bl, x0.rh, x0.rl, x1.rh, x1.rl, y0.rh, y0.rl);
  axpy<BL>(bh, bl, x0.ih, x0.il, x1.ih, x1.il, y0.ih, y0.il);
  if (NEG) {
    axpy<CL>(ch, cl, -x1.rh, -x1.rl, x0.rh, x0.rl, y1.rh, y1.rl);
    axpy<CL>(ch, cl, -x1.ih, -x1.il, x0.ih, x0.il, y1.ih, y1.il);
  } else {
    axpy<CL>(ch, cl, x1.rh, x1.rl, x0.rh, x0.rl, y1.rh, y1.rl);
    axpy<CL>(ch, cl, x1.ih, x1.il, x0.ih, x0.il, y1.ih, y1.il);
  }
  x0 = y0;
  x1 = y1;
}
// [[1, i b], [i c, 1]]: an RX-shaped rotation with its diagonal factored out
template <bool BL, bool CL>
__device__ __forceinline__ void df_rxunit(float bh, float bl, float ch, float cl, dfc& x0, dfc& x1) {
  dfc y0, y1;
  axpy<BL>(-bh, -bl, x0.rh, x0.rl, x1.ih, x1.il, y0.rh, y0.rl);
  axpy<BL>(bh, bl, x0.ih, x0.il, x1.rh, x1.rl, y0.ih, y0.il);
  axpy<CL>(-ch, -cl, x1.rh, x1.rl, x0.ih, x0.il, y1.rh, y1.rl);
  axpy<CL>(ch, cl, x1.ih, x1.il, x0.rh, x0.rl, y1.ih, y1.il);
  x0 = y0;
  x1 = y1;
}
// x * w^T, the chunks the run needs selected at compile time
template <bool A, bool B, bool C>
__device__ __forceinline__ dfc df_root_mul_impl(unsigned T, const dfc& x) {
  dfc g = dfc{1.0f, 0.0f, 0.0f, 0.0f};
  bool have = false;
  if (A) {
    const float4 v = qgp_roots[(T >> 20) & 1023u];
    g = dfc{v.x, v.y, v.z, v.w};
    have = true;
  }
  if (B) {
    const float4 v = qgp_roots[1024 + ((T >> 10) & 1023u)];
    g = have ? df_cmul<true, true>(v.x, v.y, v.z, v.w, g) : dfc{v.x, v.y, v.z, v.w};
    have = true;
  }
  if (C) {
    const float4 v = qgp_roots[2048 + (T & 1023u)];
    g = have ? df_cmul<true, true>(v.x, v.y, v.z, v.w, g) : dfc{v.x, v.y, v.z, v.w};
  }
  return df_cmul<true, true>(g.rh, g.rl, g.ih, g.il, x);
}
// x times a power of two (exact)
__device__ __forceinline__ dfc df_pow2(float c, const dfc& x) { return dfc{x.rh * c, x.rl * c, x.ih * c, x.il * c}; }
// [[a, i b], [i c, d]] with a, b, c, d real (RX-shaped)
template <bool AL, bool BL, bool CL, bool DL>
__device__ __forceinline__ void df_rxlike(float ah, float al, float bh, float bl, float ch, float cl, float dh, float dl,
                                          dfc& x0, dfc& x1) {
  dfc y0, y1;
  dot2<AL, BL>(ah, al, x0.rh, x0.rl, -bh, -bl, x1.ih, x1.il, y0.rh, y0.rl);
  dot2<AL, BL>(ah, al, x0.ih, x0.il, bh, bl, x1.rh, x1.rl, y0.ih, y0.il);
  dot2<DL, CL>(dh, dl, x1.rh, x1.rl, -ch, -cl, x0.ih, x0.il, y1.rh, y1.rl);
  dot2<CL, DL>(ch, cl, x0.rh, x0.rl, dh, dl, x1.ih, x1.il, y1.ih, y1.il);
  x0 = y0;
  x1 = y1;
}

// ---- complex64 -------------------------------------------------------------
struct F32 {
  typedef float2 V;
  static constexpr int E = 8;
  static __device__ __forceinline__ V ld_work(const unsigned char* b, int pos) {
    return reinterpret_cast<const float2*>(b)[pos];
  }
  static __device__ __forceinline__ void st_work(unsigned char* b, int pos, const V& v) {
    reinterpret_cast<float2*>(b)[pos] = v;
  }
  // two registers in the 16-byte slot pair (pos, pos + 1), pos even
  static __device__ __forceinline__ void ld_pair(const unsigned char* b, int pos, V& a, V& c) {
    const float4 v = *reinterpret_cast<const float4*>(b + pos * 8);
    a = make_float2(v.x, v.y);
    c = make_float2(v.z, v.w);
  }
  static __device__ __forceinline__ void st_pair(unsigned char* b, int pos, const V& a, const V& c) {
    *reinterpret_cast<float4*>(b + pos * 8) = make_float4(a.x, a.y, c.x, c.y);
  }
  static __device__ __forceinline__ V zero() { return make_float2(0.f, 0.f); }
  static __device__ __forceinline__ V neg(const V& x) { return make_float2(-x.x, -x.y); }
  static __device__ __forceinline__ V mul_i(const V& x) { return make_float2(-x.y, x.x); }
  static __device__ __forceinline__ V mul_mi(const V& x) { return make_float2(x.y, -x.x); }
};
__device__ __forceinline__ float2 f_cmul(float gr, float gi, float2 x) {
  return make_float2(fmaf(gr, x.x, -(gi * x.y)), fmaf(gr, x.y, gi * x.x));
}
__device__ __forceinline__ float2 f_scale(float a, float2 x) { return make_float2(a * x.x, a * x.y); }
__device__ __forceinline__ float2 f_row(float ar, float ai, float br, float bi, float2 x0, float2 x1) {
  return make_float2(fmaf(ar, x0.x, fmaf(-ai, x0.y, fmaf(br, x1.x, -(bi * x1.y)))),
                     fmaf(ar, x0.y, fmaf(ai, x0.x, fmaf(br, x1.y, bi * x1.x))));
}
__device__ __forceinline__ void f_real(float a, float b, float c, float d, float2& x0, float2& x1) {
  const float2 y0 = make_float2(fmaf(a, x0.x, b * x1.x), fmaf(a, x0.y, b * x1.y));
  const float2 y1 = make_float2(fmaf(c, x0.x, d * x1.x), fmaf(c, x0.y, d * x1.y));
  x0 = y0;
  x1 = y1;
}
__device__ __forceinline__ void f_hadamard(float c, float2& x0, float2& x1) {
  const float2 y0 = make_float2(c * (x0.x + x1.x), c * (x0.y + x1.y));
  const float2 y1 = make_float2(c * (x0.x - x1.x), c * (x0.y - x1.y));
  x0 = y0;
  x1 = y1;
}
__device__ __forceinline__ void f_sumdiff(float2& x0, float2& x1) {
  const float2 y0 = make_float2(x0.x + x1.x, x0.y + x1.y);
  const float2 y1 = make_float2(x0.x - x1.x, x0.y - x1.y);
  x0 = y0;
  x1 = y1;
}
__device__ __forceinline__ float2 f_pow2(float c, float2 x) { return make_float2(x.x * c, x.y * c); }
template <bool A, bool B, bool C>
__device__ __forceinline__ float2 f_root_mul_impl(unsigned T, float2 x) {
  float2 g = make_float2(1.0f, 0.0f);
  if (A) {
    const float4 v = qgp_roots[(T >> 20) & 1023u];
    g = f_cmul(v.x, v.z, g);
  }
  if (B) {
    const float4 v = qgp_roots[1024 + ((T >> 10) & 1023u)];
    g = f_cmul(v.x, v.z, g);
  }
  if (C) {
    const float4 v = qgp_roots[2048 + (T & 1023u)];
    g = f_cmul(v.x, v.z, g);
  }
  return f_cmul(g.x, g.y, x);
}
template <bool NEG>
__device__ __forceinline__ void f_realunit(float b, float c, float2& x0, float2& x1) {
  const float2 y0 = make_float2(fmaf(b, x1.x, x0.x), fmaf(b, x1.y, x0.y));
  const float2 y1 = NEG ? make_float2(fmaf(c, x0.x, -x1.x), fmaf(c, x0.y, -x1.y))
                        : make_float2(fmaf(c, x0.x, x1.x), fmaf(c, x0.y, x1.y));
  x0 = y0;
  x1 = y1;
}
__device__ __forceinline__ void f_rxunit(float b, float c, float2& x0, float2& x1) {
  const float2 y0 = make_float2(fmaf(-b, x1.y, x0.x), fmaf(b, x1.x, x0.y));
  const float2 y1 = make_float2(fmaf(-c, x0.y, x1.x), fmaf(c, x0.x, x1.y));
  x0 = y0;
  x1 = y1;
}
__device__ __forceinline__ void f_rxlike(float a, float b, float c, float d, float2& x0, float2& x1) {
  const float2 y0 = make_float2(fmaf(a, x0.x, -(b * x1.y)), fmaf(a, x0.y, b * x1.x));
  const float2 y1 = make_float2(fmaf(d, x1.x, -(c * x0.y)), fmaf(c, x0.x, d * x1.y));
  x0 = y0;
  x1 = y1;
}

// ---------------------------------------------------------------------------
// The tile loop. P supplies: E (bytes per amplitude in HBM), K_BITS, KLOW,
// R_BITS (each of the 2^(K_BITS - R_BITS) threads holds 2^R_BITS amplitudes),
// BUFS (1: one tile buffer, the SM's other CTAs overlap their copies with this
// one's arithmetic; 2 or 3: the next one or two tiles are prefetched), LM
// (mask of the local bit positions), hioff(h) (HBM offset, in amplitudes, of the
// h-th 2^KLOW-amplitude run of a tile), tile_base(t) (first amplitude of tile t)
// and body(buf, base, cs) (the gate run on the tile in shared memory; it ends
// with a barrier; cs holds the matrix entries when they come from a table). Each
// CTA walks a contiguous range of tiles.
// ---------------------------------------------------------------------------
template <class P>
__device__ __forceinline__ void run_pass(unsigned char* __restrict__ state, u64 ntiles) {
  constexpr int E = P::E, K = 1 << P::K_BITS, T = K >> P::R_BITS, PER = 16 / E, CPT = (K * E / 16) / T;
  extern __shared__ __align__(128) unsigned char smem[];
  u64 goff[CPT];
  unsigned soff[CPT];
#pragma unroll
  for (int i = 0; i < CPT; ++i) {
    const int l = ((int)threadIdx.x + i * T) * PER;
    goff[i] = ((u64)(l & ((1 << P::KLOW) - 1)) | P::hioff(l >> P::KLOW)) * E;
    soff[i] = (unsigned)swz<E>(l) * E;
  }
  const u64 w0 = ntiles * blockIdx.x / gridDim.x, w1 = ntiles * (blockIdx.x + 1) / gridDim.x;
  if (w0 >= w1) return;
  u64 base = P::tile_base(w0);
  if (P::BUFS == 1) {
    for (u64 t = w0; t < w1; ++t) {
#pragma unroll
      for (int i = 0; i < CPT; ++i) cp_async16(smem + soff[i], state + base * E + goff[i]);
      cp_commit();
      cp_wait<0>();
      __syncthreads();
      P::body(smem, base, nullptr);
#pragma unroll
      for (int i = 0; i < CPT; ++i)
        *reinterpret_cast<uint4*>(state + base * E + goff[i]) = *reinterpret_cast<const uint4*>(smem + soff[i]);
      __syncthreads();  // the buffer is refilled by the next tile
      base = ((base | P::LM) + 1) & ~P::LM;
    }
    return;
  }
  // a ring of BUFS buffers: the next BUFS - 1 tiles are in flight while one is worked
  // on; one copy group is committed per tile (empty ones past the range), so waiting
  // for all but the newest BUFS - 1 groups waits for the current tile
  u64 pb = base, pt = w0;
#pragma unroll
  for (int q = 0; q < P::BUFS - 1; ++q) {
    if (pt < w1) {
#pragma unroll
      for (int i = 0; i < CPT; ++i) cp_async16(smem + q * (K * E) + soff[i], state + pb * E + goff[i]);
      pb = ((pb | P::LM) + 1) & ~P::LM;
      ++pt;
    }
    cp_commit();
  }
  int cb = 0, nbuf = P::BUFS - 1;  // buffer of the current tile, of the next prefetch
  for (u64 t = w0; t < w1; ++t) {
    unsigned char* cur = smem + cb * (K * E);
    if (pt < w1) {
#pragma unroll
      for (int i = 0; i < CPT; ++i) cp_async16(smem + nbuf * (K * E) + soff[i], state + pb * E + goff[i]);
      pb = ((pb | P::LM) + 1) & ~P::LM;
      ++pt;
    }
    cp_commit();
    cp_wait<P::BUFS - 1>();
    __syncthreads();
    P::body(cur, base, nullptr);
#pragma unroll
    for (int i = 0; i < CPT; ++i)
      *reinterpret_cast<uint4*>(state + base * E + goff[i]) = *reinterpret_cast<const uint4*>(cur + soff[i]);
    __syncthreads();  // this buffer is refilled by the next prefetch
    base = ((base | P::LM) + 1) & ~P::LM;
    nbuf = cb;
    cb = cb + 1 == P::BUFS ? 0 : cb + 1;
  }
}

// The same pass over many states of one structure (a parameter sweep): work
// items are (state, tile) pairs; a CTA walks a contiguous range [w0, w1) of them
// and, whenever it reaches a new state, stages that state's matrix entries (ncoef
// floats at coefs + state * ncoef) into shared memory after the tile buffers.
template <class P>
__device__ __forceinline__ void run_pass_range(unsigned char* const* __restrict__ states,
                                               const float* __restrict__ coefs, int ncoef, u64 ntiles, u64 w0,
                                               u64 w1) {
  constexpr int E = P::E, K = 1 << P::K_BITS, T = K >> P::R_BITS, PER = 16 / E, CPT = (K * E / 16) / T;
  extern __shared__ __align__(128) unsigned char smem[];
  float* cs = reinterpret_cast<float*>(smem + P::BUFS * K * E);
  u64 goff[CPT];
  unsigned soff[CPT];
#pragma unroll
  for (int i = 0; i < CPT; ++i) {
    const int l = ((int)threadIdx.x + i * T) * PER;
    goff[i] = ((u64)(l & ((1 << P::KLOW) - 1)) | P::hioff(l >> P::KLOW)) * E;
    soff[i] = (unsigned)swz<E>(l) * E;
  }
  for (u64 w = w0; w < w1;) {
    const int si = (int)(w / ntiles);
    const u64 t0 = w - (u64)si * ntiles;
    const u64 t1 = (ntiles - t0 < w1 - w) ? ntiles : t0 + (w1 - w);
    unsigned char* state = states[si];
    __syncthreads();  // the previous state's readers of cs are done
    for (int q = (int)threadIdx.x; q < ncoef; q += T) cs[q] = coefs[(u64)si * ncoef + q];
    u64 base = P::tile_base(t0);
    // the ring of run_pass (one buffer: the next tile is loaded after the store)
    u64 pb = base, pt = t0;
#pragma unroll
    for (int q = 0; q < (P::BUFS > 1 ? P::BUFS - 1 : 1); ++q) {
      if (pt < t1) {
#pragma unroll
        for (int i = 0; i < CPT; ++i) cp_async16(smem + q * (K * E) + soff[i], state + pb * E + goff[i]);
        pb = ((pb | P::LM) + 1) & ~P::LM;
        ++pt;
      }
      cp_commit();
    }
    int cb = 0, nbuf = P::BUFS > 1 ? P::BUFS - 1 : 0;
    for (u64 t = t0; t < t1; ++t) {
      unsigned char* cur = smem + cb * (K * E);
      if (P::BUFS > 1) {
        if (pt < t1) {
#pragma unroll
          for (int i = 0; i < CPT; ++i) cp_async16(smem + nbuf * (K * E) + soff[i], state + pb * E + goff[i]);
          pb = ((pb | P::LM) + 1) & ~P::LM;
          ++pt;
        }
        cp_commit();
        cp_wait<(P::BUFS > 1 ? P::BUFS - 1 : 0)>();
      } else {
        cp_wait<0>();
      }
      __syncthreads();
      P::body(cur, base, cs);
#pragma unroll
      for (int i = 0; i < CPT; ++i)
        *reinterpret_cast<uint4*>(state + base * E + goff[i]) = *reinterpret_cast<const uint4*>(cur + soff[i]);
      __syncthreads();  // the buffer is refilled by a later tile
      if (P::BUFS == 1 && pt < t1) {
#pragma unroll
        for (int i = 0; i < CPT; ++i) cp_async16(smem + soff[i], state + pb * E + goff[i]);
        pb = ((pb | P::LM) + 1) & ~P::LM;
        ++pt;
        cp_commit();
      }
      base = ((base | P::LM) + 1) & ~P::LM;
      if (P::BUFS > 1) {
        nbuf = cb;
        cb = cb + 1 == P::BUFS ? 0 : cb + 1;
      }
    }
    w += t1 - t0;
  }
}

// One launch per pass over all states of a group: CTA b takes its share of the items.
template <class P>
__device__ __forceinline__ void run_pass_batch(unsigned char* const* __restrict__ states,
                                               const float* __restrict__ coefs, int ncoef, u64 ntiles, int nstates) {
  const u64 W = ntiles * (u64)nstates;
  run_pass_range<P>(states, coefs, ncoef, ntiles, W * blockIdx.x / gridDim.x, W * (blockIdx.x + 1) / gridDim.x);
}

// Sweeps of several sizes: one launch per pass level runs the pass of that level of
// every group (qubit count) that has one. Each CTA takes an equal share of every
// group's (state, tile) items, group after group, as if each group had its own launch
// of the same grid: a group of many small states spreads its state switches (each one
// stages that state's coefficients and cannot prefetch across states) over all CTAs.
struct GroupLevel {
  unsigned char* const* states;
  const float* coefs;  // this pass's rows: ncoef floats per state
  int ncoef, nstates;
  u64 ntiles, item0, items;
};
template <class P>
__device__ __forceinline__ void run_group_share(const GroupLevel& d) {
  const u64 a = d.items * blockIdx.x / gridDim.x, b = d.items * (blockIdx.x + 1) / gridDim.x;
  if (a < b) run_pass_range<P>(d.states, d.coefs, d.ncoef, d.ntiles, a, b);
}

}  // namespace qgp
