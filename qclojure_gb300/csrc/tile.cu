// Tiled gate-pass executor (one HBM pass applies a run of gates).
//
// A CTA owns tiles of 2^k amplitudes: the local bits of the pass (PassDesc.lbits)
// vary inside a tile, the other bits number the tiles. Per tile:
//   1. cp.async 16-byte copies bring the tile into an XOR-swizzled shared-memory
//      buffer; the next tile is prefetched into the second buffer while the
//      current one is computed (double buffering, commit/wait groups);
//   2. the op run is applied in registers: every thread holds 8 amplitudes whose
//      local indices differ in three "register bits"; a LAYOUT op writes the
//      registers back and reloads them with another choice of register bits, so
//      a barrier is paid per layout change and none per gate. Diagonal gates,
//      phases and controls need no particular layout: each register knows its
//      full basis index;
//   3. the tile goes back to HBM with coalesced 16-byte stores.
//
// Arithmetic policies:
//   PolD   complex128, exact FP64 with explicit _rn products and sums (no FMA):
//          the same rounded operations as the reference's complex multiply and
//          dense row sum (src/org/soulspace/qclojure/domain/gate.clj:384-395),
//          so results are bit-identical to the plain per-gate kernels;
//   PolF   complex64, FP32 with the same operation order;
//   PolDF  complex128 stored as IEEE doubles in HBM, computed as double-float
//          pairs on the FP32 pipes (df64.cuh); within 1e-14 per pass.
#include <cstdio>

#include "df64.cuh"
#include "qgpu_internal.h"

namespace qg {

void count_launch(int k);

namespace {

constexpr int kSMs = 152;
constexpr int kRegs = 8;  // amplitudes per thread (3 register bits)

__device__ __forceinline__ double mulD(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double addD(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double subD(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float mulD(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float addD(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float subD(float a, float b) { return __fsub_rn(a, b); }

// ---------------------------------------------------------------------------
// exact policies (FP64 / FP32), register type = double2 / float2
// ---------------------------------------------------------------------------
template <typename R, typename V>
struct PolExact {
  using Reg = V;
  static constexpr int kElem = sizeof(V);  // bytes per amplitude in HBM and shared memory
  static constexpr bool kDense = true;     // dense fused blocks supported
  struct Cst {
    R m[8];
  };
  __device__ static Cst cst(const TOp& op) {
    Cst c;
    if constexpr (sizeof(R) == 4) {
      // FP32 coefficients were rounded on the host: a double->float conversion
      // here would run on the FP64 pipe, once per op and thread
#pragma unroll
      for (int q = 0; q < 8; ++q) c.m[q] = op.mf[q];
    } else {
#pragma unroll
      for (int q = 0; q < 8; ++q) c.m[q] = op.m[q];
    }
    return c;
  }
  __device__ static V load_raw(const unsigned char* sm, int pos) { return reinterpret_cast<const V*>(sm)[pos]; }
  __device__ static V load_work(const unsigned char* sm, int pos) { return load_raw(sm, pos); }
  __device__ static void store_raw(unsigned char* sm, int pos, const V& v) { reinterpret_cast<V*>(sm)[pos] = v; }
  __device__ static void store_work(unsigned char* sm, int pos, const V& v) { store_raw(sm, pos, v); }
  __device__ static V cm(R gr, R gi, V x) {  // (gr x.re - gi x.im, gr x.im + gi x.re)
    V r;
    r.x = subD(mulD(gr, x.x), mulD(gi, x.y));
    r.y = addD(mulD(gr, x.y), mulD(gi, x.x));
    return r;
  }
  template <int CLS>
  __device__ static void u2(const Cst& c, V& x0, V& x1) {
    const R* m = c.m;
    V y0, y1;
    if (CLS == U2_GENERAL) {
      V a = cm(m[0], m[1], x0), b = cm(m[2], m[3], x1), d = cm(m[4], m[5], x0), e = cm(m[6], m[7], x1);
      y0.x = addD(a.x, b.x); y0.y = addD(a.y, b.y);
      y1.x = addD(d.x, e.x); y1.y = addD(d.y, e.y);
    } else if (CLS == U2_REAL) {
      y0.x = addD(mulD(m[0], x0.x), mulD(m[2], x1.x));
      y0.y = addD(mulD(m[0], x0.y), mulD(m[2], x1.y));
      y1.x = addD(mulD(m[4], x0.x), mulD(m[6], x1.x));
      y1.y = addD(mulD(m[4], x0.y), mulD(m[6], x1.y));
    } else if (CLS == U2_RXLIKE) {
      y0.x = subD(mulD(m[0], x0.x), mulD(m[3], x1.y));
      y0.y = addD(mulD(m[0], x0.y), mulD(m[3], x1.x));
      y1.x = subD(mulD(m[6], x1.x), mulD(m[5], x0.y));
      y1.y = addD(mulD(m[5], x0.x), mulD(m[6], x1.y));
    } else if (CLS == U2_DIAG) {
      y0 = cm(m[0], m[1], x0);
      y1 = cm(m[6], m[7], x1);
    } else if (CLS == U2_ANTIDIAG) {
      y0 = cm(m[2], m[3], x1);
      y1 = cm(m[4], m[5], x0);
    } else if (CLS == U2_X) {
      y0 = x1;
      y1 = x0;
    } else {  // U2_IMAG_ANTI
      if (m[3] > 0) { y0.x = -x1.y; y0.y = x1.x; } else { y0.x = x1.y; y0.y = -x1.x; }
      if (m[5] > 0) { y1.x = -x0.y; y1.y = x0.x; } else { y1.x = x0.y; y1.y = -x0.x; }
    }
    x0 = y0;
    x1 = y1;
  }
  template <int CLS>
  __device__ static V phase(const Cst& c, V x) {
    V r;
    if (CLS == PH_GENERAL) return cm(c.m[0], c.m[1], x);
    if (CLS == PH_NEG) { r.x = -x.x; r.y = -x.y; }
    else if (CLS == PH_I) { r.x = -x.y; r.y = x.x; }
    else { r.x = x.y; r.y = -x.x; }
    return r;
  }
  __device__ static V times_i(V x) { V r; r.x = -x.y; r.y = x.x; return r; }
  __device__ static V cmul_idx(const Cst& c, int which, V x) { return cm(c.m[2 * which], c.m[2 * which + 1], x); }
  __device__ static V scale(const Cst& c, V x) { V r; r.x = mulD(x.x, c.m[0]); r.y = mulD(x.y, c.m[0]); return r; }
  __device__ static V zero() { V r; r.x = 0; r.y = 0; return r; }
};

using PolD = PolExact<double, double2>;
using PolF = PolExact<float, float2>;

// ---------------------------------------------------------------------------
// double-float policy: HBM holds double2, registers and shared memory hold
// (re.hi, re.lo, im.hi, im.lo) after the first layout
// ---------------------------------------------------------------------------
struct PolDF {
  using Reg = dfc;
  static constexpr int kElem = 16;
  static constexpr bool kDense = false;  // dense fused blocks run with PolD
  struct Cst {
    float h[8], l[8];
  };
  __device__ static Cst cst(const TOp& op) {
    Cst c;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      c.h[q] = op.mf[q];
      c.l[q] = op.mf[8 + q];
    }
    return c;
  }
  __device__ static dfc load_raw(const unsigned char* sm, int pos) {
    return load_dfc(reinterpret_cast<const double2*>(sm)[pos]);
  }
  __device__ static dfc load_work(const unsigned char* sm, int pos) {
    float4 v = reinterpret_cast<const float4*>(sm)[pos];
    return dfc{v.x, v.y, v.z, v.w};
  }
  __device__ static void store_raw(unsigned char* sm, int pos, const dfc& v) {
    reinterpret_cast<double2*>(sm)[pos] = store_dfc(v);
  }
  __device__ static void store_work(unsigned char* sm, int pos, const dfc& v) {
    reinterpret_cast<float4*>(sm)[pos] = make_float4(v.rh, v.rl, v.ih, v.il);
  }
  __device__ static dfc cmk(const Cst& c, int k, const dfc& x) {  // matrix entry k (0..3) times x
    return cmul_df(c.h[2 * k], c.l[2 * k], c.h[2 * k + 1], c.l[2 * k + 1], x);
  }
  // a*x + b*y, complex, entries ka, kb
  __device__ static dfc lin_c(const Cst& c, int ka, const dfc& x, int kb, const dfc& y) {
    dfc p = cmk(c, ka, x), q = cmk(c, kb, y), r;
    add2(p.rh, p.rl, q.rh, q.rl, r.rh, r.rl);
    add2(p.ih, p.il, q.ih, q.il, r.ih, r.il);
    return r;
  }
  template <int CLS>
  __device__ static void u2(const Cst& c, dfc& x0, dfc& x1) {
    const float* h = c.h;
    const float* l = c.l;
    dfc y0, y1;
    if (CLS == U2_GENERAL) {
      y0 = lin_c(c, 0, x0, 1, x1);
      y1 = lin_c(c, 2, x0, 3, x1);
    } else if (CLS == U2_REAL) {
      lin2(h[0], l[0], x0.rh, x0.rl, h[2], l[2], x1.rh, x1.rl, y0.rh, y0.rl);
      lin2(h[0], l[0], x0.ih, x0.il, h[2], l[2], x1.ih, x1.il, y0.ih, y0.il);
      lin2(h[4], l[4], x0.rh, x0.rl, h[6], l[6], x1.rh, x1.rl, y1.rh, y1.rl);
      lin2(h[4], l[4], x0.ih, x0.il, h[6], l[6], x1.ih, x1.il, y1.ih, y1.il);
    } else if (CLS == U2_RXLIKE) {
      // m0=(a,0) m1=(0,b) m2=(0,c) m3=(d,0)
      lin2(h[0], l[0], x0.rh, x0.rl, -h[3], -l[3], x1.ih, x1.il, y0.rh, y0.rl);
      lin2(h[0], l[0], x0.ih, x0.il, h[3], l[3], x1.rh, x1.rl, y0.ih, y0.il);
      lin2(h[6], l[6], x1.rh, x1.rl, -h[5], -l[5], x0.ih, x0.il, y1.rh, y1.rl);
      lin2(h[5], l[5], x0.rh, x0.rl, h[6], l[6], x1.ih, x1.il, y1.ih, y1.il);
    } else if (CLS == U2_DIAG) {
      y0 = cmk(c, 0, x0);
      y1 = cmk(c, 3, x1);
    } else if (CLS == U2_ANTIDIAG) {
      y0 = cmk(c, 1, x1);
      y1 = cmk(c, 2, x0);
    } else if (CLS == U2_X) {
      y0 = x1;
      y1 = x0;
    } else {  // U2_IMAG_ANTI
      if (h[3] > 0) y0 = dfc{-x1.ih, -x1.il, x1.rh, x1.rl}; else y0 = dfc{x1.ih, x1.il, -x1.rh, -x1.rl};
      if (h[5] > 0) y1 = dfc{-x0.ih, -x0.il, x0.rh, x0.rl}; else y1 = dfc{x0.ih, x0.il, -x0.rh, -x0.rl};
    }
    x0 = y0;
    x1 = y1;
  }
  template <int CLS>
  __device__ static dfc phase(const Cst& c, const dfc& x) {
    if (CLS == PH_GENERAL) return cmk(c, 0, x);
    if (CLS == PH_NEG) return dfc{-x.rh, -x.rl, -x.ih, -x.il};
    if (CLS == PH_I) return dfc{-x.ih, -x.il, x.rh, x.rl};
    return dfc{x.ih, x.il, -x.rh, -x.rl};
  }
  __device__ static dfc times_i(const dfc& x) { return dfc{-x.ih, -x.il, x.rh, x.rl}; }
  __device__ static dfc cmul_idx(const Cst& c, int which, const dfc& x) { return cmk(c, which, x); }
  __device__ static dfc scale(const Cst& c, const dfc& x) {
    dfc r;
    mul1(c.h[0], c.l[0], x.rh, x.rl, r.rh, r.rl);
    mul1(c.h[0], c.l[0], x.ih, x.il, r.ih, r.il);
    return r;
  }
  __device__ static dfc zero() { return dfc{0.f, 0.f, 0.f, 0.f}; }
};

// XOR swizzle of the shared-memory tile: 16-byte units, 8 per 128-byte row.
template <int ELEM>
__device__ __forceinline__ int swz(int l) {
  if (ELEM == 16) return l ^ ((l >> 3) & 7);
  return l ^ (((l >> 4) & 7) << 1);  // 8-byte amplitudes: swizzle pairs, keep each 16-byte pair together
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

struct TileGeo {
  int k, K, klow, T;
};

__device__ __forceinline__ uint64_t tile_base(const PassDesc& pd, uint64_t tile) {
  uint64_t base = 0;
  for (int r = 0; r < pd.nruns; ++r)
    base |= ((tile >> pd.run_src[r]) & ((1ULL << pd.run_len[r]) - 1)) << pd.run_dst[r];
  return base;
}

// issue the copies of one tile (every thread: K*ELEM/16/T copies of 16 bytes)
template <int ELEM>
__device__ __forceinline__ void load_tile(unsigned char* buf, const unsigned char* gstate, uint64_t base,
                                          const uint64_t* hioff, const TileGeo& g) {
  constexpr int PER = 16 / ELEM;  // amplitudes per 16-byte copy
  const uint32_t lowmask = (1u << g.klow) - 1;
  const int ncopies = g.K / PER;
  for (int c = threadIdx.x; c < ncopies; c += g.T) {
    const int l = c * PER;
    const uint64_t gi = base | (l & lowmask) | hioff[l >> g.klow];
    cp_async16(buf + (size_t)swz<ELEM>(l) * ELEM, gstate + gi * ELEM);
  }
}

template <int ELEM>
__device__ __forceinline__ void store_tile(const unsigned char* buf, unsigned char* gstate, uint64_t base,
                                           const uint64_t* hioff, const TileGeo& g) {
  constexpr int PER = 16 / ELEM;
  const uint32_t lowmask = (1u << g.klow) - 1;
  const int ncopies = g.K / PER;
  for (int c = threadIdx.x; c < ncopies; c += g.T) {
    const int l = c * PER;
    const uint64_t gi = base | (l & lowmask) | hioff[l >> g.klow];
    const uint4 v = *reinterpret_cast<const uint4*>(buf + (size_t)swz<ELEM>(l) * ELEM);
    *reinterpret_cast<uint4*>(gstate + gi * ELEM) = v;
  }
}

// ---- register-level op application ----------------------------------------
template <class P, int CLS, int RP>
__device__ __forceinline__ void u2_regs(typename P::Reg (&r)[kRegs], const typename P::Cst& c, uint32_t lt,
                                        const uint32_t (&lj)[kRegs], uint32_t lc) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int j0 = ((q >> RP) << (RP + 1)) | (q & ((1 << RP) - 1));
    const int j1 = j0 | (1 << RP);
    if (((lt | lj[j0]) & lc) == lc) P::template u2<CLS>(c, r[j0], r[j1]);
  }
}

template <class P, int CLS>
__device__ __forceinline__ void u2_dispatch_rp(int rp, typename P::Reg (&r)[kRegs], const typename P::Cst& c,
                                               uint32_t lt, const uint32_t (&lj)[kRegs], uint32_t lc) {
  if (rp == 0) u2_regs<P, CLS, 0>(r, c, lt, lj, lc);
  else if (rp == 1) u2_regs<P, CLS, 1>(r, c, lt, lj, lc);
  else u2_regs<P, CLS, 2>(r, c, lt, lj, lc);
}

template <class P>
__device__ __forceinline__ void u2_dispatch(int cls, int rp, typename P::Reg (&r)[kRegs], const typename P::Cst& c,
                                            uint32_t lt, const uint32_t (&lj)[kRegs], uint32_t lc) {
  switch (cls) {
    case U2_GENERAL: u2_dispatch_rp<P, U2_GENERAL>(rp, r, c, lt, lj, lc); break;
    case U2_REAL: u2_dispatch_rp<P, U2_REAL>(rp, r, c, lt, lj, lc); break;
    case U2_RXLIKE: u2_dispatch_rp<P, U2_RXLIKE>(rp, r, c, lt, lj, lc); break;
    case U2_DIAG: u2_dispatch_rp<P, U2_DIAG>(rp, r, c, lt, lj, lc); break;
    case U2_ANTIDIAG: u2_dispatch_rp<P, U2_ANTIDIAG>(rp, r, c, lt, lj, lc); break;
    case U2_X: u2_dispatch_rp<P, U2_X>(rp, r, c, lt, lj, lc); break;
    default: u2_dispatch_rp<P, U2_IMAG_ANTI>(rp, r, c, lt, lj, lc); break;
  }
}

template <class P, int CLS>
__device__ __forceinline__ void phase_regs(typename P::Reg (&r)[kRegs], const typename P::Cst& c, uint32_t lt,
                                           const uint32_t (&lj)[kRegs], uint32_t lm) {
#pragma unroll
  for (int j = 0; j < kRegs; ++j)
    if (((lt | lj[j]) & lm) == lm) r[j] = P::template phase<CLS>(c, r[j]);
}

template <class P, int A, int B>  // swap register bits A < B: pairs with bit A = 1, bit B = 0
__device__ __forceinline__ void swap_regs(typename P::Reg (&r)[kRegs], uint32_t lt, const uint32_t (&lj)[kRegs],
                                          uint32_t lc, bool iswap) {
#pragma unroll
  for (int j = 0; j < kRegs; ++j) {
    if (((j >> A) & 1) && !((j >> B) & 1)) {
      const int p = j ^ (1 << A) ^ (1 << B);
      if (((lt | lj[j]) & lc) == lc) {
        typename P::Reg a = r[j], b = r[p];
        if (iswap) {
          r[j] = P::times_i(b);
          r[p] = P::times_i(a);
        } else {
          r[j] = b;
          r[p] = a;
        }
      }
    }
  }
}

// dense 2^dk block applied in shared memory (exact policies only)
template <class P>
__device__ void dense_smem(unsigned char* buf, const TOp& op, const double* dense, const TileGeo& g) {
  using V = typename P::Reg;
  constexpr int E = P::kElem;
  const int dk = op.dk, D = 1 << dk;
  const double* M = dense + 2 * op.doff;
  constexpr int kMaxItems = 16;
  V out[kMaxItems];
  int cnt = 0;
  for (int idx = threadIdx.x; idx < g.K; idx += g.T, ++cnt) {
    const int grp = idx >> dk, row = idx & (D - 1);
    uint32_t lg = grp;
    for (int j = 0; j < dk; ++j) {
      const int b = op.dbits[j];
      lg = ((lg >> b) << (b + 1)) | (lg & ((1u << b) - 1));
    }
    double ar = 0, ai = 0;
    for (int col = 0; col < D; ++col) {
      uint32_t lc = lg;
      for (int j = 0; j < dk; ++j)
        if ((col >> j) & 1) lc |= 1u << op.dbits[j];
      const V x = P::load_work(buf, swz<E>(lc));
      const double mr = M[2 * (row * D + col)], mi = M[2 * (row * D + col) + 1];
      ar = fma(mr, (double)x.x, fma(-mi, (double)x.y, ar));
      ai = fma(mr, (double)x.y, fma(mi, (double)x.x, ai));
    }
    V y;
    y.x = ar;
    y.y = ai;
    out[cnt] = y;
  }
  __syncthreads();
  cnt = 0;
  for (int idx = threadIdx.x; idx < g.K; idx += g.T, ++cnt) {
    const int grp = idx >> dk, row = idx & (D - 1);
    uint32_t lg = grp;
    for (int j = 0; j < dk; ++j) {
      const int b = op.dbits[j];
      lg = ((lg >> b) << (b + 1)) | (lg & ((1u << b) - 1));
    }
    for (int j = 0; j < dk; ++j)
      if ((row >> j) & 1) lg |= 1u << op.dbits[j];
    P::store_work(buf, swz<E>(lg), out[cnt]);
  }
  __syncthreads();
}

// Apply the pass's ops to the tile in buf. Returns with the tile in raw format.
template <class P>
__device__ void run_ops(unsigned char* buf, const PassDesc& pd, const TOp* __restrict__ ops,
                        const double* __restrict__ dense, uint64_t base, const TileGeo& g) {
  using Reg = typename P::Reg;
  constexpr int E = P::kElem;
  Reg r[kRegs];
  uint32_t lj[kRegs];
  uint32_t lt = 0;
  bool in_regs = false, raw = true;
  for (int64_t o = pd.op_begin; o < pd.op_end; ++o) {
    const TOp& op = ops[o];
    const int kind = op.kind;
    if (kind == OK_LAYOUT) {
      if (in_regs) {
#pragma unroll
        for (int j = 0; j < kRegs; ++j) P::store_work(buf, swz<E>(lt | lj[j]), r[j]);
        raw = false;
        __syncthreads();
      }
      // thread bits: local positions not in the register set, ascending
      const uint32_t rbmask = (1u << op.dbits[0]) | (1u << op.dbits[1]) | (1u << op.dbits[2]);
      lt = 0;
      int tb = 0;
      for (int b = 0; b < g.k; ++b) {
        if (rbmask & (1u << b)) continue;
        lt |= ((threadIdx.x >> tb) & 1u) << b;
        ++tb;
      }
#pragma unroll
      for (int j = 0; j < kRegs; ++j)
        lj[j] = ((j & 1) << op.dbits[0]) | (((j >> 1) & 1) << op.dbits[1]) | (((j >> 2) & 1) << op.dbits[2]);
      if (raw) {
#pragma unroll
        for (int j = 0; j < kRegs; ++j) r[j] = P::load_raw(buf, swz<E>(lt | lj[j]));
      } else {
#pragma unroll
        for (int j = 0; j < kRegs; ++j) r[j] = P::load_work(buf, swz<E>(lt | lj[j]));
      }
      in_regs = true;
      continue;
    }
    if (kind == OK_DENSE) {
      if (in_regs) {
#pragma unroll
        for (int j = 0; j < kRegs; ++j) P::store_work(buf, swz<E>(lt | lj[j]), r[j]);
        in_regs = false;
        raw = false;
        __syncthreads();
      }
      if constexpr (P::kDense) dense_smem<P>(buf, op, dense, g);
      continue;
    }
    const typename P::Cst c = P::cst(op);
    switch (kind) {
      case OK_U2:
        if ((base & op.gcmask) == op.gcmask) u2_dispatch<P>(op.cls, op.t2, r, c, lt, lj, op.lcmask);
        break;
      case OK_PHASE:
        if ((base & op.gmask) == op.gmask) {
          switch (op.cls) {
            case PH_GENERAL: phase_regs<P, PH_GENERAL>(r, c, lt, lj, op.lmask); break;
            case PH_NEG: phase_regs<P, PH_NEG>(r, c, lt, lj, op.lmask); break;
            case PH_I: phase_regs<P, PH_I>(r, c, lt, lj, op.lmask); break;
            default: phase_regs<P, PH_MINUS_I>(r, c, lt, lj, op.lmask); break;
          }
        }
        break;
      case OK_SWAP:
        if ((base & op.gcmask) == op.gcmask) {
          const int a = op.dbits[0], b = op.dbits[1];  // register positions, a < b
          const bool isw = op.flags & 1;
          if (a == 0 && b == 1) swap_regs<P, 0, 1>(r, lt, lj, op.lcmask, isw);
          else if (a == 0) swap_regs<P, 0, 2>(r, lt, lj, op.lcmask, isw);
          else swap_regs<P, 1, 2>(r, lt, lj, op.lcmask, isw);
        }
        break;
      case OK_BLOCKADE: {
        const int gc = __popcll(base & op.gmask);
        if (gc <= 1) {
#pragma unroll
          for (int j = 0; j < kRegs; ++j)
            if (gc + __popc((lt | lj[j]) & op.lmask) == 1) r[j] = P::cmul_idx(c, 0, r[j]);
        }
      } break;
      case OK_PARITY: {
        const int gp = __popcll(base & op.gmask) & 1;
#pragma unroll
        for (int j = 0; j < kRegs; ++j)
          r[j] = P::cmul_idx(c, gp ^ (__popc((lt | lj[j]) & op.lmask) & 1), r[j]);
      } break;
      case OK_COLLAPSE: {
        const bool gok = (base & op.gmask) == op.gval;
#pragma unroll
        for (int j = 0; j < kRegs; ++j)
          r[j] = (gok && (((lt | lj[j]) & op.lmask) == op.lval)) ? P::scale(c, r[j]) : P::zero();
      } break;
      default:
        break;
    }
  }
  if (in_regs) {
#pragma unroll
    for (int j = 0; j < kRegs; ++j) P::store_raw(buf, swz<E>(lt | lj[j]), r[j]);
  }
  __syncthreads();
}

template <class P>
__global__ void __launch_bounds__(512, 1) k_tile2(unsigned char* __restrict__ state, PassDesc pd,
                                                   const TOp* __restrict__ ops, const double* __restrict__ dense,
                                                   uint64_t ntiles) {
  constexpr int E = P::kElem;
  extern __shared__ __align__(128) unsigned char smem[];
  TileGeo g;
  g.k = pd.k;
  g.K = 1 << pd.k;
  g.klow = pd.klow;
  g.T = blockDim.x;
  const size_t tile_bytes = (size_t)g.K * E;
  uint64_t* hioff = reinterpret_cast<uint64_t*>(smem + 2 * tile_bytes);
  const int nhi = 1 << (g.k - g.klow);
  for (int h = threadIdx.x; h < nhi; h += g.T) {
    uint64_t off = 0;
    for (int j = g.klow; j < g.k; ++j)
      if ((h >> (j - g.klow)) & 1) off |= 1ULL << pd.lbits[j];
    hioff[h] = off;
  }
  __syncthreads();
  uint64_t tile = blockIdx.x;
  if (tile >= ntiles) return;
  load_tile<E>(smem, state, tile_base(pd, tile), hioff, g);
  cp_commit();
  for (int i = 0; tile < ntiles; ++i, tile += gridDim.x) {
    const uint64_t next = tile + gridDim.x;
    unsigned char* cur = smem + (i & 1) * tile_bytes;
    if (next < ntiles) {
      load_tile<E>(smem + ((i + 1) & 1) * tile_bytes, state, tile_base(pd, next), hioff, g);
      cp_commit();
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    __syncthreads();
    const uint64_t base = tile_base(pd, tile);
    run_ops<P>(cur, pd, ops, dense, base, g);
    store_tile<E>(cur, state, base, hioff, g);
    __syncthreads();  // the buffer is refilled two tiles later
  }
}

template <class P>
cudaError_t launch_t(void* s, int n, const PassDesc& pd, const TOp* d_tops, const double* d_dense,
                     cudaStream_t st) {
  constexpr int E = P::kElem;
  const int K = 1 << pd.k;
  const int threads = K / kRegs;
  if (threads < 1 || threads > 512 || (K * E) % 16 != 0 || K * E < 16 * threads) return cudaErrorInvalidValue;
  const size_t smem = 2 * (size_t)K * E + sizeof(uint64_t) * (1u << (pd.k - pd.klow));
  const uint64_t ntiles = 1ULL << (n - pd.k);
  int per_sm = (int)((220 * 1024) / smem);
  if (per_sm > 2048 / threads) per_sm = 2048 / threads;
  if (per_sm < 1) per_sm = 1;
  uint64_t grid = (uint64_t)kSMs * per_sm;
  if (grid > ntiles) grid = ntiles;
  cudaError_t e = cudaFuncSetAttribute(k_tile2<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_tile2<P><<<(unsigned)grid, threads, smem, st>>>((unsigned char*)s, pd, d_tops, d_dense, ntiles);
  count_launch(1);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_tile_pass(void* s, int precision, int arithmetic, int n, const PassDesc& pd, const TOp* d_tops,
                             const double* d_dense, cudaStream_t st) {
  if (pd.k < 3 || pd.k > kMaxTileBits) return cudaErrorInvalidValue;
  if (precision == QG_C64) return launch_t<PolF>(s, n, pd, d_tops, d_dense, st);
  if (arithmetic == QG_ARITH_DOUBLE_FLOAT) return launch_t<PolDF>(s, n, pd, d_tops, d_dense, st);
  return launch_t<PolD>(s, n, pd, d_tops, d_dense, st);
}

}  // namespace qg
