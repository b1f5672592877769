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
//   PolDFT complex128 computed as double-float pairs on the FP32 pipes
//          (df64.cuh), within 1e-14 per pass; HBM holds IEEE doubles at the
//          ends of a run of passes and float pairs between them.
#include <cstdio>
#include <cstring>
#include <type_traits>

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
  static constexpr bool kDF = false;
  // complex64 interprets two tiles per op dispatch (run_ops2); FP64 one
  static constexpr bool kTwoTiles = sizeof(R) == 4;
  static constexpr int kCst = sizeof(R) == 8 ? 0 : 1;
  static constexpr bool kInPairs = false, kOutPairs = false;
  struct Cst {
    R m[8];
  };
  __device__ static V load_raw(const unsigned char* sm, int pos) { return reinterpret_cast<const V*>(sm)[pos]; }
  __device__ static V load_work(const unsigned char* sm, int pos) { return load_raw(sm, pos); }
  __device__ static void store_raw(unsigned char* sm, int pos, const V& v) { reinterpret_cast<V*>(sm)[pos] = v; }
  __device__ static void store_work(unsigned char* sm, int pos, const V& v) { store_raw(sm, pos, v); }
  // FP64 keeps the reference's rounded products and sums (bit-identical to the oracle);
  // complex64, whose contract is a probability tolerance, contracts a product and a
  // sum into one FMA
  static constexpr bool kFMA = sizeof(R) == 4;
  __device__ static R mad(R a, R b, R c) {  // a b + c
    if constexpr (kFMA) return fmaf(a, b, c);
    else return addD(mulD(a, b), c);
  }
  __device__ static R msub(R a, R b, R c) {  // a b - c
    if constexpr (kFMA) return fmaf(a, b, -c);
    else return subD(mulD(a, b), c);
  }
  __device__ static V cm(R gr, R gi, V x) {  // (gr x.re - gi x.im, gr x.im + gi x.re)
    V r;
    r.x = msub(gr, x.x, mulD(gi, x.y));
    r.y = mad(gr, x.y, mulD(gi, x.x));
    return r;
  }
  template <int CLS>
  __device__ static void u2(const Cst& c, V& x0, V& x1) {
    const R* m = c.m;
    V y0, y1;
    if (CLS == U2_GENERAL) {
      if constexpr (kFMA) {  // y = m0 x0 + m1 x1, four FMAs per component
        y0.x = fmaf(m[0], x0.x, fmaf(-m[1], x0.y, fmaf(m[2], x1.x, -m[3] * x1.y)));
        y0.y = fmaf(m[0], x0.y, fmaf(m[1], x0.x, fmaf(m[2], x1.y, m[3] * x1.x)));
        y1.x = fmaf(m[4], x0.x, fmaf(-m[5], x0.y, fmaf(m[6], x1.x, -m[7] * x1.y)));
        y1.y = fmaf(m[4], x0.y, fmaf(m[5], x0.x, fmaf(m[6], x1.y, m[7] * x1.x)));
      } else {
        V a = cm(m[0], m[1], x0), b = cm(m[2], m[3], x1), d = cm(m[4], m[5], x0), e = cm(m[6], m[7], x1);
        y0.x = addD(a.x, b.x); y0.y = addD(a.y, b.y);
        y1.x = addD(d.x, e.x); y1.y = addD(d.y, e.y);
      }
    } else if (CLS == U2_REAL) {
      y0.x = mad(m[0], x0.x, mulD(m[2], x1.x));
      y0.y = mad(m[0], x0.y, mulD(m[2], x1.y));
      y1.x = mad(m[4], x0.x, mulD(m[6], x1.x));
      y1.y = mad(m[4], x0.y, mulD(m[6], x1.y));
    } else if (CLS == U2_RXLIKE) {
      y0.x = msub(m[0], x0.x, mulD(m[3], x1.y));
      y0.y = mad(m[0], x0.y, mulD(m[3], x1.x));
      y1.x = msub(m[6], x1.x, mulD(m[5], x0.y));
      y1.y = mad(m[5], x0.x, mulD(m[6], x1.y));
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
  // entry 0 or 1 of a phase pair (selected without indexing the constant array)
  __device__ static V cmul_idx(const Cst& c, int which, V x) {
    return which ? cm(c.m[2], c.m[3], x) : cm(c.m[0], c.m[1], x);
  }
  __device__ static V scale(const Cst& c, V x) { V r; r.x = mulD(x.x, c.m[0]); r.y = mulD(x.y, c.m[0]); return r; }
  __device__ static V zero() { V r; r.x = 0; r.y = 0; return r; }
};

using PolD = PolExact<double, double2>;
using PolF = PolExact<float, float2>;

// ---------------------------------------------------------------------------
// double-float policy: registers and shared memory hold (re.hi, re.lo, im.hi,
// im.lo). Between the passes of one program HBM holds the same pairs (IO bit 0:
// the input is in pair form, bit 1: the output is written in pair form); the
// first pass of a run converts from IEEE doubles and the last one back, so the
// passes in between convert nothing.
// ---------------------------------------------------------------------------
template <int IO, bool DENSE = false>
struct PolDFT {
  using Reg = dfc;
  static constexpr int kElem = 16;
  // dense fused blocks in double-float (dense_df), compiled only into the kernels of
  // programs that hold them
  static constexpr bool kDense = DENSE;
  static constexpr bool kDF = true;
  static constexpr bool kTwoTiles = false;
  static constexpr bool kInPairs = (IO & 1) != 0, kOutPairs = (IO & 2) != 0;
  static constexpr int kCst = 2;
  struct Cst {
    float h[8], l[8];
  };
  __device__ static dfc load_work(const unsigned char* sm, int pos) {
    float4 v = reinterpret_cast<const float4*>(sm)[pos];
    return dfc{v.x, v.y, v.z, v.w};
  }
  __device__ static dfc load_raw(const unsigned char* sm, int pos) {
    if constexpr (kInPairs) return load_work(sm, pos);
    else return load_dfc(reinterpret_cast<const double2*>(sm)[pos]);
  }
  __device__ static void store_raw(unsigned char* sm, int pos, const dfc& v) {
    if constexpr (kOutPairs) reinterpret_cast<float4*>(sm)[pos] = make_float4(v.rh, v.rl, v.ih, v.il);
    else reinterpret_cast<double2*>(sm)[pos] = store_dfc(v);
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
  __device__ static dfc cmul_idx(const Cst& c, int which, const dfc& x) {
    const bool w = which != 0;
    return cmul_df(w ? c.h[2] : c.h[0], w ? c.l[2] : c.l[0], w ? c.h[3] : c.h[1], w ? c.l[3] : c.l[1], x);
  }
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

// Each thread moves the same CPT 16-byte pieces of every tile: piece i of thread
// x is local copy c = x + i*T. Its byte offset from the tile base in HBM (goff)
// and its swizzled shared-memory offset (soff) are computed once per launch.
template <int ELEM>
struct CopyPlan {
  static constexpr int PER = 16 / ELEM;  // amplitudes per 16-byte copy
  static constexpr int CPT = ELEM / 2;   // copies per thread: (K*ELEM/16) / (K/8)
  uint64_t goff[CPT];
  uint32_t soff[CPT];
  __device__ void init(const uint64_t* hioff, const TileGeo& g) {
    const uint32_t lowmask = (1u << g.klow) - 1;
#pragma unroll
    for (int i = 0; i < CPT; ++i) {
      const int l = ((int)threadIdx.x + i * g.T) * PER;
      goff[i] = ((uint64_t)(l & lowmask) | hioff[l >> g.klow]) * ELEM;
      soff[i] = (uint32_t)swz<ELEM>(l) * ELEM;
    }
  }
  __device__ void load(unsigned char* buf, const unsigned char* gtile) const {
#pragma unroll
    for (int i = 0; i < CPT; ++i) cp_async16(buf + soff[i], gtile + goff[i]);
  }
  __device__ void store(const unsigned char* buf, unsigned char* gtile) const {
#pragma unroll
    for (int i = 0; i < CPT; ++i)
      *reinterpret_cast<uint4*>(gtile + goff[i]) = *reinterpret_cast<const uint4*>(buf + soff[i]);
  }
};

// ---- register-level op application ----------------------------------------
// ---------------------------------------------------------------------------
// Compact op records passed by value in kernel-parameter (constant-bank) space:
// every thread reads the same record, so the loads are uniform and cheap.
// ---------------------------------------------------------------------------
enum KCode : int32_t {
  KC_LAYOUT = 0,   // tmask/tval/rmr = register bits rb0/rb1/rb2, c[0..8) = lj (bit patterns)
  KC_DENSE = 1,    // tmask = dk, tval = doff, rmr = dbits (4 bits each)
  KC_U2 = 16,      // + cls * 4 + register position
  KC_PHASE = 128,  // + phase class * 8 + register mask (the registers whose bits must all be 1)
  KC_SWAP = 56,    // + register pair (0: {0,1}, 1: {0,2}, 2: {1,2}) + 3 * iswap
  KC_BLOCKADE = 62,
  KC_PARITY = 63,
  KC_COLLAPSE = 64,
  KF_COND = 0x100  // the op has control / mask conditions to evaluate
};

struct __align__(16) KOp {
  int32_t code;
  uint32_t tmask, tval, rmr;  // thread-bit mask/value, register mask | register value << 8
  uint64_t gmask, gval;       // non-local mask/value (controls of U2/SWAP: gval = gmask)
  float c[16];                // coefficients: float pairs (hi[8], lo[8]) or 8 doubles (FP64 policy)
};

constexpr int kMaxKOps = 320;

static_assert(sizeof(KOp) == 96, "KOp layout");

template <class P>
__device__ __forceinline__ typename P::Cst kcst(const KOp& op) {
  typename P::Cst c;
  if constexpr (P::kCst == 0) {  // 8 doubles
    const double* d = reinterpret_cast<const double*>(op.c);
#pragma unroll
    for (int q = 0; q < 8; ++q) c.m[q] = d[q];
  } else if constexpr (P::kCst == 1) {  // 8 floats
#pragma unroll
    for (int q = 0; q < 8; ++q) c.m[q] = op.c[q];
  } else {  // 8 float pairs: hi[8], lo[8]
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      c.h[q] = op.c[q];
      c.l[q] = op.c[8 + q];
    }
  }
  return c;
}

// Register slot j holds local index lt | lj[j]; bit q of j is register position q.
// A conditional op tests its thread bits once per thread and its register
// positions (cr, uniform) per slot with compile-time slot numbers.
__device__ __forceinline__ void csel_swap(bool c, float& a, float& b) {
  const float x = c ? b : a;
  b = c ? a : b;
  a = x;
}
__device__ __forceinline__ void csel_swap(bool c, double& a, double& b) {
  const double x = c ? b : a;
  b = c ? a : b;
  a = x;
}
__device__ __forceinline__ void csel_swap(bool c, float2& a, float2& b) {
  csel_swap(c, a.x, b.x);
  csel_swap(c, a.y, b.y);
}
__device__ __forceinline__ void csel_swap(bool c, double2& a, double2& b) {
  csel_swap(c, a.x, b.x);
  csel_swap(c, a.y, b.y);
}
__device__ __forceinline__ void csel_swap(bool c, dfc& a, dfc& b) {
  csel_swap(c, a.rh, b.rh);
  csel_swap(c, a.rl, b.rl);
  csel_swap(c, a.ih, b.ih);
  csel_swap(c, a.il, b.il);
}

// tc: the op's thread / tile condition. A conditional X (CNOT-like) swaps with
// selects instead of a divergent branch; other classes branch on tc.
template <class P, int CLS, int RP, bool COND>
__device__ __forceinline__ void u2_regs(typename P::Reg (&r)[kRegs], const typename P::Cst& c, uint32_t cr, bool tc) {
  if constexpr (COND && CLS == U2_X) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j0 = ((q >> RP) << (RP + 1)) | (q & ((1 << RP) - 1));
      const int j1 = j0 | (1 << RP);
      csel_swap(tc && (j0 & cr) == cr, r[j0], r[j1]);
    }
  } else {
    if (COND && !tc) return;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j0 = ((q >> RP) << (RP + 1)) | (q & ((1 << RP) - 1));
      const int j1 = j0 | (1 << RP);
      if (!COND || (j0 & cr) == cr) P::template u2<CLS>(c, r[j0], r[j1]);
    }
  }
}

// A phase touches only the registers whose bits include CR (compile time), so
// a phase conditioned on register bits costs its share of the registers.
template <class P, int CLS, int CR>
__device__ __forceinline__ void phase_regs(typename P::Reg (&r)[kRegs], const typename P::Cst& c) {
#pragma unroll
  for (int j = 0; j < kRegs; ++j)
    if ((j & CR) == CR) r[j] = P::template phase<CLS>(c, r[j]);
}

template <class P, int A, int B>  // swap register bits A < B: pairs with bit A = 1, bit B = 0
__device__ __forceinline__ void swap_regs(typename P::Reg (&r)[kRegs], uint32_t cr, bool iswap) {
#pragma unroll
  for (int j = 0; j < kRegs; ++j) {
    if (((j >> A) & 1) && !((j >> B) & 1)) {
      const int p = j ^ (1 << A) ^ (1 << B);
      if ((j & cr) == cr) {
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

// dense 2^dk block applied in shared memory (exact policies only). Each thread forms
// output amplitudes as row sums over the block's 2^dk inputs, visiting the columns in
// Gray-code order so that each step flips one tile bit of the input index. complex128
// multiplies in FP64 with the entries as doubles; complex64 in FP32 with the entries
// stored as float pairs.
template <class P>
__device__ void dense_smem(unsigned char* buf, const KOp& op, const double* dense, const TileGeo& g) {
  using V = typename P::Reg;
  using R = decltype(V{}.x);
  constexpr int E = P::kElem;
  const int dk = (int)op.tmask, D = 1 << dk;
  const uint32_t dbits = op.rmr;  // 4 bits per block bit
  constexpr int kMaxItems = 16;
  V out[kMaxItems];
  int cnt = 0;
  for (int idx = threadIdx.x; idx < g.K; idx += g.T, ++cnt) {
    const int grp = idx >> dk, row = idx & (D - 1);
    uint32_t lc = grp;
    for (int j = 0; j < dk; ++j) {
      const int b = (dbits >> (4 * j)) & 15;
      lc = ((lc >> b) << (b + 1)) | (lc & ((1u << b) - 1));
    }
    R ar = 0, ai = 0;
    for (int i = 0; i < D; ++i) {
      if (i) lc ^= 1u << ((dbits >> (4 * (__ffs(i) - 1))) & 15);
      const int e = row * D + (i ^ (i >> 1));
      R mr, mi;
      if constexpr (sizeof(R) == 8) {
        const double2 m = __ldg(reinterpret_cast<const double2*>(dense) + op.tval + e);
        mr = m.x;
        mi = m.y;
      } else {
        const float2 m = __ldg(reinterpret_cast<const float2*>(dense) + op.tval + e);
        mr = m.x;
        mi = m.y;
      }
      const V x = P::load_work(buf, swz<E>(lc));
      ar = fma(mr, x.x, fma(-mi, x.y, ar));
      ai = fma(mr, x.y, fma(mi, x.x, ai));
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
      const int b = (dbits >> (4 * j)) & 15;
      lg = ((lg >> b) << (b + 1)) | (lg & ((1u << b) - 1));
    }
    for (int j = 0; j < dk; ++j)
      if ((row >> j) & 1) lg |= 1u << ((dbits >> (4 * j)) & 15);
    P::store_work(buf, swz<E>(lg), out[cnt]);
  }
  __syncthreads();
}

// A dense 2^dk x 2^dk block in double-float: entries stored as (re.hi, re.lo, im.hi,
// im.lo) float quads (one 16-byte entry, the same offsets as the FP64 form), each output
// amplitude the double-float sum of its row's products with the block's columns, taken
// in the same Gray-code order as dense_smem. `raw`: the tile is still in the format the
// pass loaded (IEEE doubles unless the previous pass handed over float pairs); the
// result is always in the float-pair working format.
template <class P>
__device__ void dense_df(unsigned char* buf, const KOp& op, const double* dense, const TileGeo& g, bool raw) {
  const int dk = (int)op.tmask, D = 1 << dk;
  const uint32_t dbits = op.rmr;  // 4 bits per block bit
  constexpr int kMaxItems = 16;
  dfc out[kMaxItems];
  int cnt = 0;
  for (int idx = threadIdx.x; idx < g.K; idx += g.T, ++cnt) {
    const int grp = idx >> dk, row = idx & (D - 1);
    uint32_t lc = grp;
    for (int j = 0; j < dk; ++j) {
      const int b = (dbits >> (4 * j)) & 15;
      lc = ((lc >> b) << (b + 1)) | (lc & ((1u << b) - 1));
    }
    dfc acc{0.f, 0.f, 0.f, 0.f};
    for (int i = 0; i < D; ++i) {
      if (i) lc ^= 1u << ((dbits >> (4 * (__ffs(i) - 1))) & 15);
      const int e = row * D + (i ^ (i >> 1));
      const float4 m = __ldg(reinterpret_cast<const float4*>(dense) + op.tval + e);
      const dfc x = raw ? P::load_raw(buf, swz<16>(lc)) : P::load_work(buf, swz<16>(lc));
      const dfc pr = cmul_df(m.x, m.y, m.z, m.w, x);
      add2(acc.rh, acc.rl, pr.rh, pr.rl, acc.rh, acc.rl);
      add2(acc.ih, acc.il, pr.ih, pr.il, acc.ih, acc.il);
    }
    out[cnt] = acc;
  }
  __syncthreads();
  cnt = 0;
  for (int idx = threadIdx.x; idx < g.K; idx += g.T, ++cnt) {
    const int grp = idx >> dk, row = idx & (D - 1);
    uint32_t lg = grp;
    for (int j = 0; j < dk; ++j) {
      const int b = (dbits >> (4 * j)) & 15;
      lg = ((lg >> b) << (b + 1)) | (lg & ((1u << b) - 1));
    }
    for (int j = 0; j < dk; ++j)
      if ((row >> j) & 1) lg |= 1u << ((dbits >> (4 * j)) & 15);
    P::store_work(buf, swz<16>(lg), out[cnt]);
  }
  __syncthreads();
}

#define QG_U2_CASES(CLS)                                                                              \
  case KC_U2 + CLS * 4 + 0: u2_regs<P, CLS, 0, false>(r, kcst<P>(op), 0, true); break;               \
  case KC_U2 + CLS * 4 + 1: u2_regs<P, CLS, 1, false>(r, kcst<P>(op), 0, true); break;               \
  case KC_U2 + CLS * 4 + 2: u2_regs<P, CLS, 2, false>(r, kcst<P>(op), 0, true); break;               \
  case KF_COND | (KC_U2 + CLS * 4 + 0): u2_regs<P, CLS, 0, true>(r, kcst<P>(op), cr, tc); break;     \
  case KF_COND | (KC_U2 + CLS * 4 + 1): u2_regs<P, CLS, 1, true>(r, kcst<P>(op), cr, tc); break;     \
  case KF_COND | (KC_U2 + CLS * 4 + 2): u2_regs<P, CLS, 2, true>(r, kcst<P>(op), cr, tc); break;

#define QG_PHASE_CR(CLS, CR)                                                                 \
  case KC_PHASE + CLS * 8 + CR: phase_regs<P, CLS, CR>(r, kcst<P>(op)); break;               \
  case KF_COND | (KC_PHASE + CLS * 8 + CR): if (tc) phase_regs<P, CLS, CR>(r, kcst<P>(op)); break;
#define QG_PHASE_CASES(CLS) \
  QG_PHASE_CR(CLS, 0) QG_PHASE_CR(CLS, 1) QG_PHASE_CR(CLS, 2) QG_PHASE_CR(CLS, 3) \
  QG_PHASE_CR(CLS, 4) QG_PHASE_CR(CLS, 5) QG_PHASE_CR(CLS, 6) QG_PHASE_CR(CLS, 7)

// Apply the pass's ops to the tile in buf. Returns with the tile in raw format.
template <class P>
__device__ void run_ops(unsigned char* buf, const KOp* __restrict__ sops, int nops, const double* __restrict__ dense,
                        uint64_t base, const TileGeo& g) {
  using Reg = typename P::Reg;
  constexpr int E = P::kElem;
  Reg r[kRegs];
  int pos[kRegs];  // swizzled shared-memory slot of register j in the current layout
  uint32_t lt = 0;
  bool in_regs = false, raw = true;
  for (int o = 0; o < nops; ++o) {
    const KOp& op = sops[o];  // shared memory: a broadcast read
    const int code = op.code;
    if (code == KC_LAYOUT) {
      if (in_regs) {
#pragma unroll
        for (int j = 0; j < kRegs; ++j) P::store_work(buf, pos[j], r[j]);
        raw = false;
        __syncthreads();
      }
      // thread bits: insert zeros at the three register positions (ascending)
      lt = threadIdx.x;
      const uint32_t rb[3] = {op.tmask, op.tval, op.rmr};
#pragma unroll
      for (int q = 0; q < 3; ++q) lt = ((lt >> rb[q]) << (rb[q] + 1)) | (lt & ((1u << rb[q]) - 1));
#pragma unroll
      for (int j = 0; j < kRegs; ++j) pos[j] = swz<E>(lt | __float_as_uint(op.c[j]));
      if (raw) {
#pragma unroll
        for (int j = 0; j < kRegs; ++j) r[j] = P::load_raw(buf, pos[j]);
      } else {
#pragma unroll
        for (int j = 0; j < kRegs; ++j) r[j] = P::load_work(buf, pos[j]);
      }
      in_regs = true;
      continue;
    }
    if (code == KC_DENSE) {
      if (in_regs) {
#pragma unroll
        for (int j = 0; j < kRegs; ++j) P::store_work(buf, pos[j], r[j]);
        in_regs = false;
        raw = false;
        __syncthreads();
      }
      if constexpr (P::kDense) {
        if constexpr (P::kDF) {
          dense_df<P>(buf, op, dense, g, raw);
          raw = false;
        } else {
          dense_smem<P>(buf, op, dense, g);
        }
      }
      continue;
    }
    bool tc = true;
    uint32_t cr = 0;
    if (code & KF_COND) {
      tc = ((base & op.gmask) == op.gval) && ((lt & op.tmask) == op.tval);
      cr = op.rmr & 0xFFu;
    }
    switch (code) {
      QG_U2_CASES(U2_GENERAL)
      QG_U2_CASES(U2_REAL)
      QG_U2_CASES(U2_RXLIKE)
      QG_U2_CASES(U2_DIAG)
      QG_U2_CASES(U2_ANTIDIAG)
      QG_U2_CASES(U2_X)
      QG_U2_CASES(U2_IMAG_ANTI)
      QG_PHASE_CASES(PH_GENERAL)
      QG_PHASE_CASES(PH_NEG)
      QG_PHASE_CASES(PH_I)
      QG_PHASE_CASES(PH_MINUS_I)
      default: {
        const int k = code & 0xFF;
        if (k >= KC_SWAP && k < KC_SWAP + 6) {
          if (tc) {
            const int pr = (k - KC_SWAP) % 3;
            const bool isw = (k - KC_SWAP) >= 3;
            if (pr == 0) swap_regs<P, 0, 1>(r, cr, isw);
            else if (pr == 1) swap_regs<P, 0, 2>(r, cr, isw);
            else swap_regs<P, 1, 2>(r, cr, isw);
          }
        } else if (k == KC_BLOCKADE) {
          const int cnt = __popcll(base & op.gmask) + __popc(lt & op.tmask);
          if (cnt <= 1) {
            const typename P::Cst c = kcst<P>(op);
#pragma unroll
            for (int j = 0; j < kRegs; ++j)
              if (cnt + __popc(j & cr) == 1) r[j] = P::cmul_idx(c, 0, r[j]);
          }
        } else if (k == KC_PARITY) {
          const int par = (__popcll(base & op.gmask) + __popc(lt & op.tmask)) & 1;
          const typename P::Cst c = kcst<P>(op);
#pragma unroll
          for (int j = 0; j < kRegs; ++j) r[j] = P::cmul_idx(c, par ^ (__popc(j & cr) & 1), r[j]);
        } else if (k == KC_COLLAPSE) {
          const typename P::Cst c = kcst<P>(op);
          const uint32_t rv = (op.rmr >> 8) & 0xFFu;
#pragma unroll
          for (int j = 0; j < kRegs; ++j) r[j] = (tc && (j & cr) == rv) ? P::scale(c, r[j]) : P::zero();
        }
      } break;
    }
  }
  if (in_regs) {
#pragma unroll
    for (int j = 0; j < kRegs; ++j) P::store_raw(buf, pos[j], r[j]);
  } else if (!raw) {
    if constexpr (P::kDF && !P::kOutPairs) {  // a dense block left float pairs: to IEEE doubles
      for (int l = threadIdx.x; l < g.K; l += g.T) {
        const int p = swz<E>(l);
        P::store_raw(buf, p, P::load_work(buf, p));
      }
    }
  } else if constexpr (P::kInPairs != P::kOutPairs) {
    {  // no op loaded the tile: convert it in place (each thread its own slots)
      for (int l = threadIdx.x; l < g.K; l += g.T) {
        const int p = swz<E>(l);
        P::store_raw(buf, p, P::load_raw(buf, p));
      }
    }
  }
  __syncthreads();
}

#undef QG_U2_CASES
#undef QG_PHASE_CR
#undef QG_PHASE_CASES

// The interpreter on two tiles of one state at once, eight registers of each per
// thread: every op record is read, dispatched and its constants loaded once for sixteen
// amplitudes, which halves the per-op overhead per amplitude (the interpreter's cost:
// its gate arithmetic is a small share). Conditions on the tile index are evaluated per
// tile; everything else is shared. Used for complex64 (no pair formats).
#define QG_U2_PAIR(CLS, RP)                                                        \
  case KC_U2 + CLS * 4 + RP: {                                                     \
    const typename P::Cst c_ = kcst<P>(op);                                        \
    u2_regs<P, CLS, RP, false>(r0, c_, 0, true);                                   \
    u2_regs<P, CLS, RP, false>(r1, c_, 0, true);                                   \
  } break;                                                                         \
  case KF_COND | (KC_U2 + CLS * 4 + RP): {                                         \
    const typename P::Cst c_ = kcst<P>(op);                                        \
    u2_regs<P, CLS, RP, true>(r0, c_, cr, tc0);                                    \
    u2_regs<P, CLS, RP, true>(r1, c_, cr, tc1);                                    \
  } break;
#define QG_U2_CASES2(CLS) QG_U2_PAIR(CLS, 0) QG_U2_PAIR(CLS, 1) QG_U2_PAIR(CLS, 2)
#define QG_PHASE_CR2(CLS, CR)                                                      \
  case KC_PHASE + CLS * 8 + CR: {                                                  \
    const typename P::Cst c_ = kcst<P>(op);                                        \
    phase_regs<P, CLS, CR>(r0, c_);                                                \
    phase_regs<P, CLS, CR>(r1, c_);                                                \
  } break;                                                                         \
  case KF_COND | (KC_PHASE + CLS * 8 + CR): {                                      \
    const typename P::Cst c_ = kcst<P>(op);                                        \
    if (tc0) phase_regs<P, CLS, CR>(r0, c_);                                       \
    if (tc1) phase_regs<P, CLS, CR>(r1, c_);                                       \
  } break;
#define QG_PHASE_CASES2(CLS) \
  QG_PHASE_CR2(CLS, 0) QG_PHASE_CR2(CLS, 1) QG_PHASE_CR2(CLS, 2) QG_PHASE_CR2(CLS, 3) \
  QG_PHASE_CR2(CLS, 4) QG_PHASE_CR2(CLS, 5) QG_PHASE_CR2(CLS, 6) QG_PHASE_CR2(CLS, 7)

template <class P>
__device__ void run_ops2(unsigned char* buf0, unsigned char* buf1, const KOp* __restrict__ sops, int nops,
                         const double* __restrict__ dense, uint64_t base0, uint64_t base1, const TileGeo& g) {
  static_assert(!P::kDF && !P::kInPairs && !P::kOutPairs, "two-tile interpretation: one storage format");
  using Reg = typename P::Reg;
  constexpr int E = P::kElem;
  Reg r0[kRegs], r1[kRegs];
  int pos[kRegs];  // swizzled shared-memory slot of register j in the current layout (both tiles)
  uint32_t lt = 0;
  bool in_regs = false;
  for (int o = 0; o < nops; ++o) {
    const KOp& op = sops[o];
    const int code = op.code;
    if (code == KC_LAYOUT) {
      if (in_regs) {
#pragma unroll
        for (int j = 0; j < kRegs; ++j) {
          P::store_work(buf0, pos[j], r0[j]);
          P::store_work(buf1, pos[j], r1[j]);
        }
        __syncthreads();
      }
      lt = threadIdx.x;
      const uint32_t rb[3] = {op.tmask, op.tval, op.rmr};
#pragma unroll
      for (int q = 0; q < 3; ++q) lt = ((lt >> rb[q]) << (rb[q] + 1)) | (lt & ((1u << rb[q]) - 1));
#pragma unroll
      for (int j = 0; j < kRegs; ++j) pos[j] = swz<E>(lt | __float_as_uint(op.c[j]));
#pragma unroll
      for (int j = 0; j < kRegs; ++j) {
        r0[j] = P::load_work(buf0, pos[j]);
        r1[j] = P::load_work(buf1, pos[j]);
      }
      in_regs = true;
      continue;
    }
    if (code == KC_DENSE) {
      if (in_regs) {
#pragma unroll
        for (int j = 0; j < kRegs; ++j) {
          P::store_work(buf0, pos[j], r0[j]);
          P::store_work(buf1, pos[j], r1[j]);
        }
        in_regs = false;
        __syncthreads();
      }
      if constexpr (P::kDense) {
        dense_smem<P>(buf0, op, dense, g);
        dense_smem<P>(buf1, op, dense, g);
      }
      continue;
    }
    bool tc0 = true, tc1 = true;
    uint32_t cr = 0;
    if (code & KF_COND) {
      const bool tl = (lt & op.tmask) == op.tval;
      tc0 = tl && (base0 & op.gmask) == op.gval;
      tc1 = tl && (base1 & op.gmask) == op.gval;
      cr = op.rmr & 0xFFu;
    }
    switch (code) {
      QG_U2_CASES2(U2_GENERAL)
      QG_U2_CASES2(U2_REAL)
      QG_U2_CASES2(U2_RXLIKE)
      QG_U2_CASES2(U2_DIAG)
      QG_U2_CASES2(U2_ANTIDIAG)
      QG_U2_CASES2(U2_X)
      QG_U2_CASES2(U2_IMAG_ANTI)
      QG_PHASE_CASES2(PH_GENERAL)
      QG_PHASE_CASES2(PH_NEG)
      QG_PHASE_CASES2(PH_I)
      QG_PHASE_CASES2(PH_MINUS_I)
      default: {
        const int k = code & 0xFF;
        if (k >= KC_SWAP && k < KC_SWAP + 6) {
          const int pr = (k - KC_SWAP) % 3;
          const bool isw = (k - KC_SWAP) >= 3;
          if (pr == 0) {
            if (tc0) swap_regs<P, 0, 1>(r0, cr, isw);
            if (tc1) swap_regs<P, 0, 1>(r1, cr, isw);
          } else if (pr == 1) {
            if (tc0) swap_regs<P, 0, 2>(r0, cr, isw);
            if (tc1) swap_regs<P, 0, 2>(r1, cr, isw);
          } else {
            if (tc0) swap_regs<P, 1, 2>(r0, cr, isw);
            if (tc1) swap_regs<P, 1, 2>(r1, cr, isw);
          }
        } else if (k == KC_BLOCKADE) {
          const typename P::Cst c = kcst<P>(op);
          const int ct = __popc(lt & op.tmask);
          const int cnt0 = __popcll(base0 & op.gmask) + ct, cnt1 = __popcll(base1 & op.gmask) + ct;
#pragma unroll
          for (int j = 0; j < kRegs; ++j) {
            if (cnt0 <= 1 && cnt0 + __popc(j & cr) == 1) r0[j] = P::cmul_idx(c, 0, r0[j]);
            if (cnt1 <= 1 && cnt1 + __popc(j & cr) == 1) r1[j] = P::cmul_idx(c, 0, r1[j]);
          }
        } else if (k == KC_PARITY) {
          const typename P::Cst c = kcst<P>(op);
          const int pt = __popc(lt & op.tmask);
          const int par0 = (__popcll(base0 & op.gmask) + pt) & 1, par1 = (__popcll(base1 & op.gmask) + pt) & 1;
#pragma unroll
          for (int j = 0; j < kRegs; ++j) {
            r0[j] = P::cmul_idx(c, par0 ^ (__popc(j & cr) & 1), r0[j]);
            r1[j] = P::cmul_idx(c, par1 ^ (__popc(j & cr) & 1), r1[j]);
          }
        } else if (k == KC_COLLAPSE) {
          const typename P::Cst c = kcst<P>(op);
          const uint32_t rv = (op.rmr >> 8) & 0xFFu;
#pragma unroll
          for (int j = 0; j < kRegs; ++j) {
            r0[j] = (tc0 && (j & cr) == rv) ? P::scale(c, r0[j]) : P::zero();
            r1[j] = (tc1 && (j & cr) == rv) ? P::scale(c, r1[j]) : P::zero();
          }
        }
      } break;
    }
  }
  if (in_regs) {
#pragma unroll
    for (int j = 0; j < kRegs; ++j) {
      P::store_raw(buf0, pos[j], r0[j]);
      P::store_raw(buf1, pos[j], r1[j]);
    }
  }
  __syncthreads();
}

#undef QG_U2_PAIR
#undef QG_U2_CASES2
#undef QG_PHASE_CR2
#undef QG_PHASE_CASES2

// States processed by one launch: all share the pass structure (PassDesc, op
// kinds and count); op records may differ per state (ops_stride records apart).
struct BatchArgs {
  unsigned char* const* states;  // device array of nstates amplitude arrays
  const KOp* kops;               // op records of state 0
  int64_t ops_stride;            // records between consecutive states' lists (0: one shared list)
  int nstates;
};

template <class P>
__global__ void __launch_bounds__(512, 1) k_tile2(const PassDesc pd, const BatchArgs ba, int nops,
                                                  const double* __restrict__ dense, uint64_t ntiles, int pairs) {
  constexpr int E = P::kElem;
  extern __shared__ __align__(128) unsigned char smem[];
  TileGeo g;
  g.k = pd.k;
  g.K = 1 << pd.k;
  g.klow = pd.klow;
  g.T = blockDim.x;
  const size_t tile_bytes = (size_t)g.K * E;
  const int nhi = 1 << (g.k - g.klow);
  // pairs: four tile buffers (two pairs: one interpreted, one in flight), else two
  KOp* sops = reinterpret_cast<KOp*>(smem + (pairs ? 4 : 2) * tile_bytes);  // 16-byte aligned: tile_bytes % 16 == 0
  uint64_t* hioff = reinterpret_cast<uint64_t*>(sops + nops);
  for (int h = threadIdx.x; h < nhi; h += g.T) {
    uint64_t off = 0;
    for (int j = g.klow; j < g.k; ++j)
      if ((h >> (j - g.klow)) & 1) off |= 1ULL << pd.lbits[j];
    hioff[h] = off;
  }
  // mask of the local bit positions: the next tile's base is the deposit increment
  // ((base | lm) + 1) & ~lm, which carries through the local positions
  uint64_t lm = 0;
  for (int j = 0; j < g.k; ++j) lm |= 1ULL << pd.lbits[j];
  __syncthreads();  // hioff is complete
  CopyPlan<E> cp;
  cp.init(hioff, g);
  // contiguous range of (state, tile) work items for this CTA
  const uint64_t W = ntiles * (uint64_t)ba.nstates;
  const uint64_t w0 = W * blockIdx.x / gridDim.x, w1 = W * (blockIdx.x + 1) / gridDim.x;
  int staged = -1;
  for (uint64_t w = w0; w < w1;) {
    const int si = (int)(w / ntiles);
    const uint64_t t0 = w - (uint64_t)si * ntiles;
    const uint64_t t1 = (ntiles - t0 < w1 - w) ? ntiles : t0 + (w1 - w);
    unsigned char* state = ba.states[si];
    if (staged < 0 || (si != staged && ba.ops_stride != 0)) {
      __syncthreads();  // previous segment's readers of sops are done
      const uint4* src = reinterpret_cast<const uint4*>(ba.kops + (int64_t)si * ba.ops_stride);
      uint4* dst = reinterpret_cast<uint4*>(sops);
      const int words = nops * (int)(sizeof(KOp) / 16);
      for (int q = threadIdx.x; q < words; q += g.T) dst[q] = src[q];
    }
    staged = si;
    __syncthreads();
    uint64_t base = tile_base(pd, t0);
    if constexpr (P::kTwoTiles) {
      if (pairs) {
        // tiles two at a time (one op dispatch for both); the next pair loads into the
        // other two buffers meanwhile; an odd last tile runs alone
        auto next = [&](uint64_t b) { return ((b | lm) + 1) & ~lm; };
        auto buf = [&](int q) { return smem + q * tile_bytes; };
        cp.load(buf(0), state + base * E);
        if (t0 + 1 < t1) cp.load(buf(1), state + next(base) * E);
        cp_commit();
        int slot = 0;
        for (uint64_t tile = t0; tile < t1;) {
          const int cnt = (t1 - tile >= 2) ? 2 : 1;
          const uint64_t b0 = base, b1 = next(base);
          const uint64_t nb = cnt == 2 ? next(b1) : b1;
          const uint64_t ntile = tile + cnt;
          if (ntile < t1) {
            cp.load(buf(2 * (slot ^ 1)), state + nb * E);
            if (ntile + 1 < t1) cp.load(buf(2 * (slot ^ 1) + 1), state + next(nb) * E);
            cp_commit();
            cp_wait<1>();
          } else {
            cp_wait<0>();
          }
          __syncthreads();
          if (cnt == 2) {
            run_ops2<P>(buf(2 * slot), buf(2 * slot + 1), sops, nops, dense, b0, b1, g);
            cp.store(buf(2 * slot), state + b0 * E);
            cp.store(buf(2 * slot + 1), state + b1 * E);
          } else {
            run_ops<P>(buf(2 * slot), sops, nops, dense, b0, g);
            cp.store(buf(2 * slot), state + b0 * E);
          }
          __syncthreads();  // these buffers are refilled by the pair after next
          base = nb;
          tile = ntile;
          slot ^= 1;
        }
        w += t1 - t0;
        continue;
      }
    }
    cp.load(smem, state + base * E);
    cp_commit();
    int i = 0;
    for (uint64_t tile = t0; tile < t1; ++tile, ++i) {
      unsigned char* cur = smem + (i & 1) * tile_bytes;
      const uint64_t nbase = ((base | lm) + 1) & ~lm;
      if (tile + 1 < t1) {
        cp.load(smem + ((i + 1) & 1) * tile_bytes, state + nbase * E);
        cp_commit();
        cp_wait<1>();
      } else {
        cp_wait<0>();
      }
      __syncthreads();
      run_ops<P>(cur, sops, nops, dense, base, g);
      cp.store(cur, state + base * E);
      __syncthreads();  // the buffer is refilled two tiles later
      base = nbase;
    }
    w += t1 - t0;
  }
}

// Small jobs: a state of n <= 12 qubits is one tile, so one CTA runs a whole job.
// The state is loaded into shared memory once, every pass of the job's program
// (op records staged pass by pass) is applied to it there, and it is stored
// once. One launch serves many jobs of the same qubit count, one CTA each. The
// op records and their order are those of the job's own program, so the
// results equal a per-job run of the same program.
template <class P>
__global__ void __launch_bounds__(512, 1) k_tile_jobs(int n, const TileJobRec* __restrict__ jobs, int njobs,
                                                      const KOp* __restrict__ kops,
                                                      const int32_t* __restrict__ pass_nops) {
  constexpr int E = P::kElem;
  extern __shared__ __align__(128) unsigned char smem[];
  TileGeo g;
  g.k = n;
  g.K = 1 << n;
  g.klow = n;
  g.T = blockDim.x;
  unsigned char* tile = smem;
  KOp* sops = reinterpret_cast<KOp*>(smem + (size_t)g.K * E);
  uint64_t* hioff = reinterpret_cast<uint64_t*>(sops + kMaxKOps);
  if (threadIdx.x == 0) hioff[0] = 0;  // every bit is local
  __syncthreads();
  CopyPlan<E> cp;
  cp.init(hioff, g);
  for (int jx = blockIdx.x; jx < njobs; jx += gridDim.x) {
    const TileJobRec jr = jobs[jx];
    unsigned char* state = reinterpret_cast<unsigned char*>(jr.state);
    cp.load(tile, state);
    cp_commit();
    cp_wait<0>();
    __syncthreads();
    if constexpr (P::kInPairs) {  // IEEE doubles -> float pairs, each thread its own slots
      for (int l = threadIdx.x; l < g.K; l += g.T) {
        const int q = swz<E>(l);
        const dfc v = load_dfc(reinterpret_cast<const double2*>(tile)[q]);
        reinterpret_cast<float4*>(tile)[q] = make_float4(v.rh, v.rl, v.ih, v.il);
      }
    }
    int64_t ob = jr.op_begin;
    for (int p = 0; p < jr.npasses; ++p) {
      const int nops = pass_nops[jr.pass_begin + p];
      __syncthreads();  // the previous pass's readers of sops are done
      const uint4* src = reinterpret_cast<const uint4*>(kops + ob);
      uint4* dst = reinterpret_cast<uint4*>(sops);
      const int words = nops * (int)(sizeof(KOp) / 16);
      for (int q = threadIdx.x; q < words; q += g.T) dst[q] = src[q];
      __syncthreads();
      run_ops<P>(tile, sops, nops, nullptr, 0, g);  // ends with a barrier
      ob += nops;
    }
    if constexpr (P::kOutPairs) {  // float pairs -> IEEE doubles
      for (int l = threadIdx.x; l < g.K; l += g.T) {
        const int q = swz<E>(l);
        const float4 v = reinterpret_cast<const float4*>(tile)[q];
        reinterpret_cast<double2*>(tile)[q] = store_dfc(dfc{v.x, v.y, v.z, v.w});
      }
      __syncthreads();
    }
    cp.store(tile, state);
    __syncthreads();  // the tile buffer is reloaded for the next job
  }
}

// The same per-job work as k_tile_jobs, served by a resident loop: each CTA claims the
// next published slot (slots in publication order), runs the job, then marks the slot
// done. The polls of the ring are the loop's only waits; when none finds work for
// idle_ns the CTA returns (and *served counts the jobs it ran), so a loop never spins
// beyond that budget.
__device__ __forceinline__ uint32_t ld_acquire_sys(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_sys(int32_t* p, int32_t v) {
  asm volatile("st.release.sys.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
template <class P>
__global__ void __launch_bounds__(512, 1) k_job_loop(int n, JobLoopSlot* slots, uint32_t cap,
                                                     const uint32_t* tail, uint32_t* head, uint32_t* served,
                                                     uint64_t idle_ns) {
  constexpr int E = P::kElem;
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ long long s_claim;
  __shared__ JobLoopSlot s_slot;
  TileGeo g;
  g.k = n;
  g.K = 1 << n;
  g.klow = n;
  g.T = blockDim.x;
  unsigned char* tile = smem;
  KOp* sops = reinterpret_cast<KOp*>(smem + (size_t)g.K * E);
  uint64_t* hioff = reinterpret_cast<uint64_t*>(sops + kMaxKOps);
  if (threadIdx.x == 0) hioff[0] = 0;  // every bit is local
  __syncthreads();
  CopyPlan<E> cp;
  cp.init(hioff, g);
  uint64_t last = now_ns();
  uint32_t ran = 0;
  for (;;) {
    if (threadIdx.x == 0) {
      long long claim = -1;
      for (;;) {
        const uint32_t t = ld_acquire_sys(tail);
        const uint32_t h = *reinterpret_cast<volatile uint32_t*>(head);
        if (h >= t) break;
        if (atomicCAS(head, h, h + 1) == h) {
          claim = h;
          break;
        }
      }
      if (claim >= 0) {
        // the slot was written before the host raised tail (the acquire above orders these reads)
        const volatile JobLoopSlot* vs = slots + (claim % cap);
        s_slot.rec.state = vs->rec.state;
        s_slot.rec.op_begin = vs->rec.op_begin;
        s_slot.rec.npasses = vs->rec.npasses;
        s_slot.rec.pass_begin = vs->rec.pass_begin;
        s_slot.kops = vs->kops;
        s_slot.pass_nops = vs->pass_nops;
        last = now_ns();
      } else if (now_ns() - last > idle_ns) {
        claim = -2;  // nothing published for idle_ns: leave
      } else {
        __nanosleep(2000);
      }
      s_claim = claim;
    }
    __syncthreads();
    const long long claim = s_claim;
    __syncthreads();
    if (claim == -2) break;
    if (claim < 0) continue;
    const TileJobRec jr = s_slot.rec;
    const KOp* kops = reinterpret_cast<const KOp*>(s_slot.kops);
    const int32_t* pass_nops = s_slot.pass_nops;
    unsigned char* state = reinterpret_cast<unsigned char*>(jr.state);
    cp.load(tile, state);
    cp_commit();
    cp_wait<0>();
    __syncthreads();
    if constexpr (P::kInPairs) {  // IEEE doubles -> float pairs, each thread its own slots
      for (int l = threadIdx.x; l < g.K; l += g.T) {
        const int q = swz<E>(l);
        const dfc v = load_dfc(reinterpret_cast<const double2*>(tile)[q]);
        reinterpret_cast<float4*>(tile)[q] = make_float4(v.rh, v.rl, v.ih, v.il);
      }
    }
    int64_t ob = jr.op_begin;
    for (int p = 0; p < jr.npasses; ++p) {
      const int nops = pass_nops[jr.pass_begin + p];
      __syncthreads();  // the previous pass's readers of sops are done
      const uint4* src = reinterpret_cast<const uint4*>(kops + ob);
      uint4* dst = reinterpret_cast<uint4*>(sops);
      const int words = nops * (int)(sizeof(KOp) / 16);
      for (int q = threadIdx.x; q < words; q += g.T) dst[q] = src[q];
      __syncthreads();
      run_ops<P>(tile, sops, nops, nullptr, 0, g);  // ends with a barrier
      ob += nops;
    }
    if constexpr (P::kOutPairs) {  // float pairs -> IEEE doubles
      for (int l = threadIdx.x; l < g.K; l += g.T) {
        const int q = swz<E>(l);
        const float4 v = reinterpret_cast<const float4*>(tile)[q];
        reinterpret_cast<double2*>(tile)[q] = store_dfc(dfc{v.x, v.y, v.z, v.w});
      }
      __syncthreads();
    }
    cp.store(tile, state);
    __syncthreads();  // every thread's stores are issued; the tile buffer is free
    if (threadIdx.x == 0) {
      __threadfence_system();  // the state's stores are visible before the flag
      st_release_sys(&slots[claim % cap].done, 1);
      ++ran;
    }
  }
  if (threadIdx.x == 0 && ran) atomicAdd(served, ran);
}

// Host: translate TOps into the compact records of policy P.
template <class P>
void build_kops(KOp* out, const TOp* ops, int64_t nops) {
  std::memset(out, 0, sizeof(KOp) * (size_t)nops);
  for (int64_t o = 0; o < nops; ++o) {
    const TOp& t = ops[o];
    KOp& k = out[o];
    if (t.kind == OK_LAYOUT) {
      k.code = KC_LAYOUT;
      k.tmask = t.dbits[0];
      k.tval = t.dbits[1];
      k.rmr = t.dbits[2];
      for (int j = 0; j < 8; ++j) std::memcpy(&k.c[j], &t.lj[j], 4);
      continue;
    }
    if (t.kind == OK_DENSE) {
      k.code = KC_DENSE;
      k.tmask = t.dk;
      k.tval = (uint32_t)t.doff;
      for (int j = 0; j < t.dk; ++j) k.rmr |= (uint32_t)t.dbits[j] << (4 * j);
      continue;
    }
    if (std::is_same<P, PolD>::value) {
      std::memcpy(k.c, t.m, sizeof(double) * 8);
    } else {
      std::memcpy(k.c, t.mf, sizeof(float) * 16);
    }
    k.tmask = t.tmask;
    k.tval = t.tval;
    k.rmr = t.rmask | (t.rval << 8);
    bool cond = t.tmask != 0 || t.rmask != 0;
    switch (t.kind) {
      case OK_U2:
        k.code = KC_U2 + t.cls * 4 + t.t2;
        k.gmask = k.gval = t.gcmask;
        cond = cond || t.gcmask != 0;
        break;
      case OK_PHASE:  // register bits are part of the code; tmask / gmask make it conditional
        k.code = KC_PHASE + t.cls * 8 + (int)(t.rmask & 7u);
        k.gmask = k.gval = t.gmask;
        cond = t.tmask != 0 || t.gmask != 0;
        break;
      case OK_SWAP: {
        const int a = t.dbits[0], b = t.dbits[1];
        const int pr = (a == 0 && b == 1) ? 0 : (a == 0 ? 1 : 2);
        k.code = KC_SWAP + pr + 3 * (t.flags & 1);
        k.gmask = k.gval = t.gcmask;
        cond = true;
      } break;
      case OK_BLOCKADE:
        k.code = KC_BLOCKADE;
        k.gmask = t.gmask;
        cond = true;
        break;
      case OK_PARITY:
        k.code = KC_PARITY;
        k.gmask = t.gmask;
        cond = true;
        break;
      default:  // OK_COLLAPSE
        k.code = KC_COLLAPSE;
        k.gmask = t.gmask;
        k.gval = t.gval;
        cond = true;
        break;
    }
    if (cond) k.code |= KF_COND;
  }
}

template <class P>
cudaError_t launch_t(int n, const PassDesc& pd, const BatchArgs& ba, const double* d_dense, cudaStream_t st) {
  constexpr int E = P::kElem;
  const int K = 1 << pd.k;
  const int threads = K / kRegs;
  const int nops = (int)(pd.op_end - pd.op_begin);
  if (threads < 1 || threads > 512 || (K * E) % 16 != 0 || K * E < 16 * threads || nops > kMaxKOps ||
      ba.nstates < 1)
    return cudaErrorInvalidValue;
  // complex64 interprets tile pairs when four buffers fit where two 64 KiB ones do
  const int pairs = (P::kTwoTiles && 4 * (size_t)K * E <= 2 * (size_t(64) << 10)) ? 1 : 0;
  const size_t smem = (pairs ? 4 : 2) * (size_t)K * E + sizeof(KOp) * (size_t)nops +
                      sizeof(uint64_t) * (1u << (pd.k - pd.klow));
  const uint64_t ntiles = 1ULL << (n - pd.k);
  const uint64_t work = ntiles * (uint64_t)ba.nstates;
  int per_sm = (int)((220 * 1024) / smem);
  if (per_sm > 2048 / threads) per_sm = 2048 / threads;
  if (per_sm < 1) per_sm = 1;
  uint64_t grid = (uint64_t)kSMs * per_sm;
  if (grid > work) grid = work;
  // One fixed limit for every launch: worker threads launch passes of different
  // sizes concurrently, and a per-launch value could undercut another thread's launch.
  // two 64 KiB tile buffers, the largest op list, the chunk-offset table (2^(12-3) entries)
  constexpr size_t kSmemLimit = 2 * (size_t(64) << 10) + sizeof(KOp) * kMaxKOps + 8 * 512;
  static_assert(kSmemLimit <= 227 * 1024, "shared memory");
  if (smem > kSmemLimit) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k_tile2<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemLimit);
  if (e != cudaSuccess) return e;
  k_tile2<P><<<(unsigned)grid, threads, smem, st>>>(pd, ba, nops, d_dense, ntiles, pairs);
  count_launch(1);
  return cudaGetLastError();
}

}  // namespace

int tile_pass_io(const Program& prog, size_t step) {
  if (prog.arith != QG_ARITH_DOUBLE_FLOAT) return 0;
  auto tiled = [&](size_t j) { return j < prog.steps.size() && prog.steps[j].kind == Step::TILE_PASS; };
  if (!tiled(step)) return 0;
  int io = 0;
  if (step > 0 && tiled(step - 1)) io |= kTileInPairs;
  if (tiled(step + 1)) io |= kTileOutPairs;
  return io;
}

int max_ops_per_tile_pass() { return kMaxKOps; }
size_t kop_record_bytes() { return sizeof(KOp); }

void encode_kops(int precision, int arithmetic, const TOp* tops, int64_t count, void* out) {
  KOp* k = reinterpret_cast<KOp*>(out);
  if (precision == QG_C64) build_kops<PolF>(k, tops, count);
  else if (arithmetic == QG_ARITH_DOUBLE_FLOAT) build_kops<PolDFT<0>>(k, tops, count);
  else build_kops<PolD>(k, tops, count);
}

template <class P>
cudaError_t launch_jobs_t(int n, const TileJobRec* d_jobs, int njobs, const KOp* d_kops, const int32_t* d_pass_nops,
                          cudaStream_t st) {
  constexpr int E = P::kElem;
  const int K = 1 << n;
  const int threads = K / kRegs;
  if (n < 5 || n > kMaxSmallJobQubits || njobs < 1) return cudaErrorInvalidValue;
  const size_t smem = (size_t)K * E + sizeof(KOp) * kMaxKOps + 16;
  cudaError_t e = cudaFuncSetAttribute(k_tile_jobs<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)((size_t(64) << 10) + sizeof(KOp) * kMaxKOps + 16));
  if (e != cudaSuccess) return e;
  k_tile_jobs<P><<<(unsigned)njobs, threads, smem, st>>>(n, d_jobs, njobs, d_kops, d_pass_nops);
  count_launch(1);
  return cudaGetLastError();
}

template <class P>
cudaError_t launch_loop_t(int n, JobLoopSlot* d_slots, uint32_t cap, const uint32_t* d_tail, uint32_t* d_head,
                          uint32_t* d_served, uint64_t idle_ns, cudaStream_t st) {
  constexpr int E = P::kElem;
  const int K = 1 << n;
  const int threads = K / kRegs;
  if (n < 5 || n > kMaxSmallJobQubits || cap < 1) return cudaErrorInvalidValue;
  const size_t smem = (size_t)K * E + sizeof(KOp) * kMaxKOps + 16;
  cudaError_t e = cudaFuncSetAttribute(k_job_loop<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)((size_t(64) << 10) + sizeof(KOp) * kMaxKOps + 16));
  if (e != cudaSuccess) return e;
  k_job_loop<P><<<kJobLoopCtas, threads, smem, st>>>(n, d_slots, cap, d_tail, d_head, d_served, idle_ns);
  count_launch(1);
  return cudaGetLastError();
}

cudaError_t launch_job_loop(int precision, int arithmetic, int n, JobLoopSlot* d_slots, uint32_t cap,
                            const uint32_t* d_tail, uint32_t* d_head, uint32_t* d_served, uint64_t idle_ns,
                            cudaStream_t st) {
  if (precision == QG_C64) return launch_loop_t<PolF>(n, d_slots, cap, d_tail, d_head, d_served, idle_ns, st);
  if (arithmetic == QG_ARITH_DOUBLE_FLOAT)
    return launch_loop_t<PolDFT<3>>(n, d_slots, cap, d_tail, d_head, d_served, idle_ns, st);
  return launch_loop_t<PolD>(n, d_slots, cap, d_tail, d_head, d_served, idle_ns, st);
}

cudaError_t launch_tile_jobs(int precision, int arithmetic, int n, const TileJobRec* d_jobs, int njobs,
                             const void* d_kops, const int32_t* d_pass_nops, cudaStream_t st) {
  const KOp* k = reinterpret_cast<const KOp*>(d_kops);
  if (precision == QG_C64) return launch_jobs_t<PolF>(n, d_jobs, njobs, k, d_pass_nops, st);
  if (arithmetic == QG_ARITH_DOUBLE_FLOAT) return launch_jobs_t<PolDFT<3>>(n, d_jobs, njobs, k, d_pass_nops, st);
  return launch_jobs_t<PolD>(n, d_jobs, njobs, k, d_pass_nops, st);
}

cudaError_t launch_tile_pass(int precision, int arithmetic, int io, int n, const PassDesc& pd,
                             void* const* d_states, int nstates, const void* d_kops, int64_t ops_stride,
                             const double* d_dense, cudaStream_t st) {
  if (pd.k < 3 || pd.k > kMaxTileBits) return cudaErrorInvalidValue;
  BatchArgs ba;
  ba.states = reinterpret_cast<unsigned char* const*>(d_states);
  ba.kops = reinterpret_cast<const KOp*>(d_kops) + pd.op_begin;
  ba.ops_stride = ops_stride;
  ba.nstates = nstates;
  if (precision == QG_C64) return launch_t<PolF>(n, pd, ba, d_dense, st);
  if (arithmetic == QG_ARITH_DOUBLE_FLOAT) {
    switch (io & 3) {
      case 0: return d_dense ? launch_t<PolDFT<0, true>>(n, pd, ba, d_dense, st) : launch_t<PolDFT<0>>(n, pd, ba, d_dense, st);
      case 1: return d_dense ? launch_t<PolDFT<1, true>>(n, pd, ba, d_dense, st) : launch_t<PolDFT<1>>(n, pd, ba, d_dense, st);
      case 2: return d_dense ? launch_t<PolDFT<2, true>>(n, pd, ba, d_dense, st) : launch_t<PolDFT<2>>(n, pd, ba, d_dense, st);
      default: return d_dense ? launch_t<PolDFT<3, true>>(n, pd, ba, d_dense, st) : launch_t<PolDFT<3>>(n, pd, ba, d_dense, st);
    }
  }
  return launch_t<PolD>(n, pd, ba, d_dense, st);
}

}  // namespace qg
