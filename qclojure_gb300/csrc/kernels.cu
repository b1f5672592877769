// sm_103a kernels of libqgpu.so.
//
// State layout in HBM: 2^n interleaved complex amplitudes (double2 for c128,
// float2 for c64), basis index i, qubit q <-> bit (n-1-q) of i.
//
// Arithmetic: every 2x2 class, phase and collapse multiplies with the same
// rounded products and sums the reference's complex multiply and dense row sum
// form (src/org/soulspace/qclojure/domain/gate.clj:384-395,
// src/org/soulspace/qclojure/domain/math/fastmath/complex_linear_algebra.clj:408-431),
// written with explicit __dmul_rn/__dadd_rn so nothing is contracted into an FMA.
// The complex128 path therefore reproduces the CPU restatement bit for bit, and
// the plain (one pass per gate) and tiled (many gates per pass) executors give
// identical amplitudes. Dense fused blocks use FMA and are checked to tolerance.
#include <atomic>
#include <cstdio>

#include "qgpu_internal.h"
#include "quant.cuh"

namespace qg {

namespace {

constexpr int kSMs = 152;

std::atomic<unsigned long long> g_launches{0};
inline void counted(int k = 1) { g_launches.fetch_add((unsigned long long)k, std::memory_order_relaxed); }

template <typename R> struct C2;
template <> struct C2<double> { using T = double2; };
template <> struct C2<float> { using T = float2; };

__device__ __forceinline__ double mul_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float mul_(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add_(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub_(float a, float b) { return __fsub_rn(a, b); }

// reference complex multiply g*x: (g.re x.re - g.im x.im, g.re x.im + g.im x.re)
template <typename V, typename R>
__device__ __forceinline__ V cmul(R gr, R gi, V x) {
  V r;
  r.x = sub_(mul_(gr, x.x), mul_(gi, x.y));
  r.y = add_(mul_(gr, x.y), mul_(gi, x.x));
  return r;
}
template <typename V>
__device__ __forceinline__ V cadd(V a, V b) {
  V r;
  r.x = add_(a.x, b.x);
  r.y = add_(a.y, b.y);
  return r;
}

template <typename R>
struct Mat {
  R m[8];
};

template <typename R>
Mat<R> to_mat(const double* m) {
  Mat<R> r;
  for (int k = 0; k < 8; ++k) r.m[k] = (R)m[k];
  return r;
}

// 2x2 application per class; y0,y1 from x0,x1.
template <int CLS, typename V, typename R>
__device__ __forceinline__ void u2_apply(const R* m, V x0, V x1, V& y0, V& y1) {
  if (CLS == U2_GENERAL) {
    y0 = cadd(cmul(m[0], m[1], x0), cmul(m[2], m[3], x1));
    y1 = cadd(cmul(m[4], m[5], x0), cmul(m[6], m[7], x1));
  } else if (CLS == U2_REAL) {
    y0.x = add_(mul_(m[0], x0.x), mul_(m[2], x1.x));
    y0.y = add_(mul_(m[0], x0.y), mul_(m[2], x1.y));
    y1.x = add_(mul_(m[4], x0.x), mul_(m[6], x1.x));
    y1.y = add_(mul_(m[4], x0.y), mul_(m[6], x1.y));
  } else if (CLS == U2_RXLIKE) {
    // m0=(a,0) m1=(0,b) m2=(0,c) m3=(d,0)
    y0.x = sub_(mul_(m[0], x0.x), mul_(m[3], x1.y));
    y0.y = add_(mul_(m[0], x0.y), mul_(m[3], x1.x));
    y1.x = sub_(mul_(m[6], x1.x), mul_(m[5], x0.y));
    y1.y = add_(mul_(m[5], x0.x), mul_(m[6], x1.y));
  } else if (CLS == U2_DIAG) {
    y0 = cmul(m[0], m[1], x0);
    y1 = cmul(m[6], m[7], x1);
  } else if (CLS == U2_ANTIDIAG) {
    y0 = cmul(m[2], m[3], x1);
    y1 = cmul(m[4], m[5], x0);
  } else if (CLS == U2_X) {
    y0 = x1;
    y1 = x0;
  } else {  // U2_IMAG_ANTI: m1=(0,s1), m2=(0,s2), s=+-1: (0,s)*x = (-s x.im, s x.re)
    if (m[3] > 0) { y0.x = -x1.y; y0.y = x1.x; } else { y0.x = x1.y; y0.y = -x1.x; }
    if (m[5] > 0) { y1.x = -x0.y; y1.y = x0.x; } else { y1.x = x0.y; y1.y = -x0.x; }
  }
}

template <int CLS, typename V, typename R>
__device__ __forceinline__ V phase_apply(const R* m, V x) {
  if (CLS == PH_GENERAL) return cmul(m[0], m[1], x);
  V r;
  if (CLS == PH_NEG) { r.x = -x.x; r.y = -x.y; }
  else if (CLS == PH_I) { r.x = -x.y; r.y = x.x; }
  else { r.x = x.y; r.y = -x.x; }
  return r;
}

// Insert bits: positions ascending; bits in setmask become 1, the others 0.
struct Fixed {
  int n;
  int pos[8];
  uint64_t setmask;
};
__device__ __forceinline__ uint64_t expand(uint64_t j, const Fixed& f) {
#pragma unroll 1
  for (int i = 0; i < f.n; ++i) {
    int b = f.pos[i];
    uint64_t lo = j & ((1ULL << b) - 1);
    j = ((j >> b) << (b + 1)) | lo;
  }
  return j | f.setmask;
}

Fixed make_fixed(uint64_t zero_bits, uint64_t one_bits) {
  Fixed f;
  f.n = 0;
  f.setmask = one_bits;
  uint64_t all = zero_bits | one_bits;
  for (int b = 0; b < 64 && f.n < 8; ++b)
    if (all & (1ULL << b)) f.pos[f.n++] = b;
  return f;
}

inline int grid_for(uint64_t work, int threads) {
  uint64_t g = (work + threads - 1) / threads;
  uint64_t cap = (uint64_t)kSMs * 8;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

// ---------------------------------------------------------------------------
// Plain kernels: one gate, one HBM pass, grid-stride.
// ---------------------------------------------------------------------------
template <int CLS, typename R>
__global__ void __launch_bounds__(256) k_u2(typename C2<R>::T* __restrict__ s, uint64_t work, int t, Fixed f,
                                            Mat<R> m) {
  using V = typename C2<R>::T;
  const uint64_t tb = 1ULL << t;
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < work; j += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t i0 = expand(j, f);
    V x0 = s[i0], x1 = s[i0 | tb], y0, y1;
    u2_apply<CLS, V, R>(m.m, x0, x1, y0, y1);
    s[i0] = y0;
    s[i0 | tb] = y1;
  }
}

template <int CLS, typename R>
__global__ void __launch_bounds__(256) k_phase(typename C2<R>::T* __restrict__ s, uint64_t work, Fixed f, Mat<R> m) {
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < work; j += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t i = expand(j, f);
    s[i] = phase_apply<CLS>(m.m, s[i]);
  }
}

template <typename R>
__global__ void __launch_bounds__(256) k_swap(typename C2<R>::T* __restrict__ s, uint64_t work, uint64_t flip, Fixed f,
                                              int iswap) {
  using V = typename C2<R>::T;
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < work; j += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t i = expand(j, f), p = i ^ flip;
    V a = s[i], b = s[p];
    if (iswap) {
      V ra, rb;
      ra.x = -b.y; ra.y = b.x;   // i * b
      rb.x = -a.y; rb.y = a.x;   // i * a
      a = ra;
      b = rb;
      s[i] = a;
      s[p] = b;
    } else {
      s[i] = b;
      s[p] = a;
    }
  }
}

// kind: 0 blockade (popcount==1 -> ph), 1 parity (ph0/ph1), 2 collapse (match -> scale, else 0)
template <int KIND, typename R>
__global__ void __launch_bounds__(256) k_diag_all(typename C2<R>::T* __restrict__ s, uint64_t N, uint64_t mask,
                                                  uint64_t val, Mat<R> m) {
  using V = typename C2<R>::T;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x) {
    V x = s[i];
    if (KIND == 0) {
      if (__popcll(i & mask) == 1) s[i] = cmul(m.m[0], m.m[1], x);
    } else if (KIND == 1) {
      if (__popcll(i & mask) & 1) s[i] = cmul(m.m[2], m.m[3], x);
      else s[i] = cmul(m.m[0], m.m[1], x);
    } else {
      V r;
      if ((i & mask) == val) { r.x = mul_(x.x, m.m[0]); r.y = mul_(x.y, m.m[0]); }
      else { r.x = 0; r.y = 0; }
      s[i] = r;
    }
  }
}

template <typename R>
cudaError_t plain_op_t(void* sv, int n, const GOp& op, cudaStream_t st) {
  using V = typename C2<R>::T;
  V* s = (V*)sv;
  const int T = 256;
  const uint64_t N = 1ULL << n;
  switch (op.kind) {
    case OK_U2: {
      Fixed f = make_fixed(1ULL << op.t, op.cmask);
      uint64_t work = N >> f.n;
      Mat<R> m = to_mat<R>(op.m);
      int g = grid_for(work, T);
      switch (op.cls) {
        case U2_GENERAL: k_u2<U2_GENERAL, R><<<g, T, 0, st>>>(s, work, op.t, f, m); break;
        case U2_REAL: k_u2<U2_REAL, R><<<g, T, 0, st>>>(s, work, op.t, f, m); break;
        case U2_RXLIKE: k_u2<U2_RXLIKE, R><<<g, T, 0, st>>>(s, work, op.t, f, m); break;
        case U2_DIAG: k_u2<U2_DIAG, R><<<g, T, 0, st>>>(s, work, op.t, f, m); break;
        case U2_ANTIDIAG: k_u2<U2_ANTIDIAG, R><<<g, T, 0, st>>>(s, work, op.t, f, m); break;
        case U2_X: k_u2<U2_X, R><<<g, T, 0, st>>>(s, work, op.t, f, m); break;
        default: k_u2<U2_IMAG_ANTI, R><<<g, T, 0, st>>>(s, work, op.t, f, m); break;
      }
    } break;
    case OK_PHASE: {
      Fixed f = make_fixed(0, op.mask);
      uint64_t work = N >> f.n;
      Mat<R> m = to_mat<R>(op.m);
      int g = grid_for(work, T);
      switch (op.cls) {
        case PH_GENERAL: k_phase<PH_GENERAL, R><<<g, T, 0, st>>>(s, work, f, m); break;
        case PH_NEG: k_phase<PH_NEG, R><<<g, T, 0, st>>>(s, work, f, m); break;
        case PH_I: k_phase<PH_I, R><<<g, T, 0, st>>>(s, work, f, m); break;
        default: k_phase<PH_MINUS_I, R><<<g, T, 0, st>>>(s, work, f, m); break;
      }
    } break;
    case OK_SWAP: {
      Fixed f = make_fixed(1ULL << op.t2, (1ULL << op.t) | op.cmask);
      uint64_t work = N >> f.n;
      k_swap<R><<<grid_for(work, T), T, 0, st>>>(s, work, (1ULL << op.t) | (1ULL << op.t2), f, op.flags & 1);
    } break;
    case OK_BLOCKADE:
      k_diag_all<0, R><<<grid_for(N, T), T, 0, st>>>(s, N, op.mask, 0, to_mat<R>(op.m));
      break;
    case OK_PARITY:
      k_diag_all<1, R><<<grid_for(N, T), T, 0, st>>>(s, N, op.mask, 0, to_mat<R>(op.m));
      break;
    case OK_COLLAPSE:
      k_diag_all<2, R><<<grid_for(N, T), T, 0, st>>>(s, N, op.mask, op.val, to_mat<R>(op.m));
      break;
    default:
      return cudaErrorInvalidValue;
  }
  counted();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Reductions. Per-thread TwoSum accumulation, warp/block combination of
// (sum, compensation) pairs, one pair per block written to d_part.
// ---------------------------------------------------------------------------
struct DD {
  double s, c;
};
__device__ __forceinline__ void two_sum_acc(DD& a, double x) {
  double t = __dadd_rn(a.s, x);
  double bp = __dsub_rn(t, a.s);
  double e = __dadd_rn(__dsub_rn(a.s, __dsub_rn(t, bp)), __dsub_rn(x, bp));
  a.s = t;
  a.c = __dadd_rn(a.c, e);
}
__device__ __forceinline__ DD dd_add(DD a, DD b) {
  DD r = a;
  two_sum_acc(r, b.s);
  r.c = __dadd_rn(r.c, b.c);
  return r;
}
template <int NT>
__device__ __forceinline__ void block_reduce_store(DD v, double* d_part, int slot) {
  __shared__ DD red[NT / 32];
  for (int o = 16; o > 0; o >>= 1) {
    DD w;
    w.s = __shfl_down_sync(0xffffffffu, v.s, o);
    w.c = __shfl_down_sync(0xffffffffu, v.c, o);
    v = dd_add(v, w);
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    DD a = red[0];
    for (int w = 1; w < NT / 32; ++w) a = dd_add(a, red[w]);
    d_part[2 * slot] = a.s;
    d_part[2 * slot + 1] = a.c;
  }
}

template <typename R>
__device__ __forceinline__ double p_of(typename C2<R>::T a) {
  if constexpr (sizeof(R) == 4) {
    // the squares of floats are exact doubles, built on the integer pipes (quant.cuh):
    // only the rounded sum is an FP64 instruction
    return __dadd_rn(qg_sq_float(a.x), qg_sq_float(a.y));
  } else {
    const double re = a.x, im = a.y;
    return __dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im));
  }
}

template <typename R>
__global__ void __launch_bounds__(256) k_probs(const typename C2<R>::T* __restrict__ s, uint64_t N,
                                               double* __restrict__ p) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x)
    p[i] = p_of<R>(s[i]);
}

template <typename R>
__global__ void __launch_bounds__(256) k_norm2(const typename C2<R>::T* __restrict__ s, uint64_t N, double* d_part) {
  DD a{0, 0};
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x)
    two_sum_acc(a, p_of<R>(s[i]));
  block_reduce_store<256>(a, d_part, blockIdx.x);
}

// Re(w * conj(a) b), w in {1, -i, -1, i} indexed by wk (0..3): conj(a)b = R + iI
__device__ __forceinline__ double re_wab(int wk, double ar, double ai, double br, double bi) {
  double R = ar * br + ai * bi, I = ar * bi - ai * br;
  switch (wk & 3) {
    case 0: return R;
    case 1: return I;   // -i*(R+iI) = I - iR
    case 2: return -R;
    default: return -I; //  i*(R+iI) = -I + iR
  }
}

// <psi|P|psi>, (P psi)_i = (-i)^ny (-1)^popc(i&z) psi_{i^x}
template <typename R>
__global__ void __launch_bounds__(256) k_pauli(const typename C2<R>::T* __restrict__ s, uint64_t N, uint64_t xm,
                                               uint64_t zm, int ny, double* d_part) {
  DD acc{0, 0};
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  if (xm == 0) {
    // diagonal: (-1)^popc(i & z) p_i   (ny = 0 when x = 0)
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
      double p = p_of<R>(s[i]);
      two_sum_acc(acc, (__popcll(i & zm) & 1) ? -p : p);
    }
  } else {
    const int hb = 63 - __clzll(xm);
    const uint64_t half = N >> 1;
    for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < half; q += stride) {
      uint64_t i = ((q >> hb) << (hb + 1)) | (q & ((1ULL << hb) - 1));
      uint64_t j = i ^ xm;
      auto a = s[i];
      auto b = s[j];
      // term i: Re(conj(a_i) w_i a_j), term j: Re(conj(a_j) w_j a_i)
      int wi = ny + ((__popcll(i & zm) & 1) ? 2 : 0);
      int wj = ny + ((__popcll(j & zm) & 1) ? 2 : 0);
      double v = re_wab(wi, a.x, a.y, b.x, b.y) + re_wab(wj, b.x, b.y, a.x, a.y);
      two_sum_acc(acc, v);
    }
  }
  block_reduce_store<256>(acc, d_part, blockIdx.x);
}

template <typename R>
__global__ void __launch_bounds__(256) k_expect1q(const typename C2<R>::T* __restrict__ s, uint64_t N, int bit,
                                                  Mat<double> o, double* d_part) {
  DD acc{0, 0};
  const uint64_t half = N >> 1, tb = 1ULL << bit;
  for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < half; q += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t i0 = ((q >> bit) << (bit + 1)) | (q & (tb - 1));
    auto a = s[i0];
    auto b = s[i0 | tb];
    double x0r = a.x, x0i = a.y, x1r = b.x, x1i = b.y;
    double y0r = o.m[0] * x0r - o.m[1] * x0i + o.m[2] * x1r - o.m[3] * x1i;
    double y0i = o.m[0] * x0i + o.m[1] * x0r + o.m[2] * x1i + o.m[3] * x1r;
    double y1r = o.m[4] * x0r - o.m[5] * x0i + o.m[6] * x1r - o.m[7] * x1i;
    double y1i = o.m[4] * x0i + o.m[5] * x0r + o.m[6] * x1i + o.m[7] * x1r;
    two_sum_acc(acc, x0r * y0r + x0i * y0i + x1r * y1r + x1i * y1i);
  }
  block_reduce_store<256>(acc, d_part, blockIdx.x);
}

template <typename R>
__global__ void __launch_bounds__(256) k_inner(const typename C2<R>::T* __restrict__ a,
                                               const typename C2<R>::T* __restrict__ b, uint64_t N, double* d_part) {
  DD re{0, 0}, im{0, 0};
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x) {
    auto x = a[i];
    auto y = b[i];
    two_sum_acc(re, (double)x.x * y.x + (double)x.y * y.y);
    two_sum_acc(im, (double)x.x * y.y - (double)x.y * y.x);
  }
  block_reduce_store<256>(re, d_part, blockIdx.x);
  __syncthreads();
  block_reduce_store<256>(im, d_part, gridDim.x + blockIdx.x);
}

// Distance of a state a (complex64 or complex128) from a complex128 state b, d_i = a_i - b_i.
// Per block, as double-double partials: |d|^2, <b|d> (real, imaginary), |a|^2, |b|^2 and
// sum_i | |a_i|^2 - |b_i|^2 |, the last as |Re(d_i conj(a_i + b_i))| so that it does not
// cancel; and max_i |d_i|^2. 1 - F follows without cancellation from the identity
// <a|a><b|b> - |<b|a>|^2 = <b|b><d|d> - |<b|d>|^2.
template <typename R>
__global__ void __launch_bounds__(256) k_compare(const typename C2<R>::T* __restrict__ a,
                                                 const double2* __restrict__ b, uint64_t N, double* d_part,
                                                 double* d_max) {
  DD dd{0, 0}, re{0, 0}, im{0, 0}, na{0, 0}, nb{0, 0}, tv{0, 0};
  double mx = 0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (uint64_t)gridDim.x * blockDim.x) {
    auto x = a[i];
    double2 y = b[i];
    double ar = (double)x.x, ai = (double)x.y;
    double dr = ar - y.x, di = ai - y.y;
    double d2 = dr * dr + di * di;
    two_sum_acc(dd, d2);
    two_sum_acc(re, y.x * dr + y.y * di);
    two_sum_acc(im, y.x * di - y.y * dr);
    two_sum_acc(na, ar * ar + ai * ai);
    two_sum_acc(nb, y.x * y.x + y.y * y.y);
    two_sum_acc(tv, fabs(dr * (ar + y.x) + di * (ai + y.y)));
    mx = fmax(mx, d2);
  }
  const DD acc[6] = {dd, re, im, na, nb, tv};
  for (int k = 0; k < 6; ++k) {
    block_reduce_store<256>(acc[k], d_part, k * gridDim.x + blockIdx.x);
    __syncthreads();
  }
  __shared__ double mred[8];
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) mred[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = mred[0];
    for (int w = 1; w < 8; ++w) m = fmax(m, mred[w]);
    d_max[blockIdx.x] = m;
  }
}

// Marginal over fixed-bit outcomes: blockIdx.y = outcome over the unique measured bits.
template <typename R>
__global__ void __launch_bounds__(256) k_marginal(const typename C2<R>::T* __restrict__ s, uint64_t work, Fixed f0,
                                                  int m, const int* __restrict__ bits, double* d_pm,
                                                  unsigned long long* d_qm) {
  const int o = blockIdx.y;
  Fixed f = f0;
  uint64_t set = 0;
  for (int k = 0; k < m; ++k)
    if ((o >> k) & 1) set |= 1ULL << bits[k];
  f.setmask = set;
  DD acc{0, 0};
  unsigned long long qs = 0;
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < work; j += (uint64_t)gridDim.x * blockDim.x) {
    double p = p_of<R>(s[expand(j, f)]);
    two_sum_acc(acc, p);
    double v = p * 4611686018427387904.0;
    qs += (v > 0) ? (unsigned long long)v : 0ULL;
  }
  const int slot = o * gridDim.x + blockIdx.x;
  block_reduce_store<256>(acc, d_pm, slot);
  __shared__ unsigned long long qred[8];
  for (int off = 16; off > 0; off >>= 1) qs += __shfl_down_sync(0xffffffffu, qs, off);
  if ((threadIdx.x & 31) == 0) qred[threadIdx.x >> 5] = qs;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < 8; ++w) t += qred[w];
    d_qm[slot] = t;
  }
}

template <typename R>
__global__ void k_gather(const typename C2<R>::T* __restrict__ s, const uint64_t* __restrict__ idx, int64_t count,
                         double* __restrict__ out) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < count; j += (int64_t)gridDim.x * blockDim.x) {
    auto a = s[idx[j]];
    out[2 * j] = a.x;
    out[2 * j + 1] = a.y;
  }
}

template <typename R>
__global__ void k_density(const typename C2<R>::T* __restrict__ s, uint64_t N, double* __restrict__ rho) {
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N * N; e += (uint64_t)gridDim.x * blockDim.x) {
    uint64_t i = e / N, j = e % N;
    auto a = s[i];
    auto b = s[j];
    // a_i conj(a_j)
    rho[2 * e] = (double)a.x * b.x + (double)a.y * b.y;
    rho[2 * e + 1] = (double)a.y * b.x - (double)a.x * b.y;
  }
}

__global__ void k_set_one(void* s, int prec, uint64_t idx) {
  if (prec == QG_C64) reinterpret_cast<float2*>(s)[idx] = make_float2(1.f, 0.f);
  else reinterpret_cast<double2*>(s)[idx] = make_double2(1.0, 0.0);
}

__global__ void k_c128_to_c64(const double2* __restrict__ a, float2* __restrict__ b, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    double2 v = a[i];
    b[i] = make_float2((float)v.x, (float)v.y);
  }
}
__global__ void k_c64_to_c128(const float2* __restrict__ a, double2* __restrict__ b, uint64_t n) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    float2 v = a[i];
    b[i] = make_double2(v.x, v.y);
  }
}

// ---------------------------------------------------------------------------
// Hierarchical sampler. Probabilities are quantised q_i = floor(p_i 2^62);
// chunk (32 amplitudes) and block (256 chunks) sums are exact integers, so the
// cumulative distribution does not depend on launch shape. A shot draws
// u = floor(r64 * T / 2^64) from Philox and takes the first i whose cumulative
// sum exceeds u: block by binary search of the block prefix, chunk by a warp
// scan of the block's chunk sums, amplitude by a warp scan inside the chunk.
// ---------------------------------------------------------------------------
struct SampleGeom {
  uint64_t N;
  int ch;       // amplitudes per chunk (<= 32)
  int cpb;      // chunks per block (<= 256)
  uint64_t nb;  // blocks
  uint64_t nchunks;
};
SampleGeom sample_geom(int n) {
  SampleGeom g;
  g.N = 1ULL << n;
  g.ch = (int)(g.N < 32 ? g.N : 32);
  uint64_t nch = g.N / g.ch;
  g.cpb = (int)(nch < 256 ? nch : 256);
  g.nchunks = nch;
  g.nb = nch / g.cpb;
  return g;
}

// floor(p 2^62) on the integer pipes (quant.cuh): the FP64 product and conversion's value
__device__ __forceinline__ unsigned long long quant(double p) { return qg_quant62(p); }

// one CTA (256 threads = 8 warps) per sample block. Only integer sums are formed here:
// the FP64 total of the normalisation check is derived from them (k_samp_scan). A
// compensated FP64 reduction per chunk ran on the FP64 pipe (about 1/58 of the FP32
// rate on this part) and bound the whole sampler by it.
// Full blocks (256 chunks of 32 amplitudes: states of 13 qubits and more, 16-byte aligned,
// as every state the runtime allocates): warp w takes the block's chunks 32w .. 32w + 31
// and reads them with 16-byte loads, eight per lane in flight (one amplitude per lane and
// load for complex128, two for complex64). Integer sums are associative: every chunk sum
// equals the lane-per-amplitude form's. The quantised probabilities come from the
// fixed-point fast path (qg_quant62_sq_fast, no FP64 instruction) wherever its guard
// allows, and from the FP64 expression (one vote per group of eight loads) where it
// fails; both give the same integers. Parts of 2^-10 or more fail it, and since the
// probabilities sum to one, at most 2^20 amplitudes of a state have them. complex128
// votes on the group's largest part first and sends such groups to the FP64 expression
// whole; for complex64 that check cost more than it saved (28 qubits: 530 against
// 585 us per launch, even for a GHZ state). Three CTAs per SM: 80 registers (ptxas
// otherwise picks 64 for complex128 and spills).
template <typename R>
__global__ void __launch_bounds__(256, 3) k_samp_sums(const typename C2<R>::T* __restrict__ s, SampleGeom g,
                                                   unsigned long long* __restrict__ csum,
                                                   unsigned long long* __restrict__ bsum) {
  using T = typename C2<R>::T;
  constexpr int A = 16 / (int)sizeof(T);  // amplitudes per 16-byte load
  constexpr int CL = 32 / A;              // lanes per chunk
  constexpr int LOADS = 32 / A;           // loads per lane for the warp's 32 chunks
  constexpr int U = 8;                    // loads in flight per lane
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __shared__ unsigned long long wq[8];
  for (uint64_t b = blockIdx.x; b < g.nb; b += gridDim.x) {
    unsigned long long bq = 0;
    if (g.ch == 32 && g.cpb == 256 && (reinterpret_cast<uintptr_t>(s) & 15u) == 0) {
      const uint64_t c0 = b * 256 + (uint64_t)warp * 32;  // the warp's first chunk
      const uint4* src = reinterpret_cast<const uint4*>(s + c0 * 32);
      if constexpr (A == 2) {
        // complex64: load u gives lane L amplitudes 64u + 2L, +1 (chunk 2u + L / 16), so
        // each half-warp holds one partial per chunk of its parity; recursive halving
        // (each step a lane sends the half of its partials it does not keep) leaves lane
        // l of half h the sum of chunk 2l + h after 15 exchanges for all 32 chunks
        unsigned long long w[LOADS];
#pragma unroll
        for (int i0 = 0; i0 < LOADS; i0 += U) {
          uint4 v[U];
#pragma unroll
          for (int u = 0; u < U; ++u) v[u] = __ldg(src + (i0 + u) * 32 + lane);
          unsigned slow = 0;
#pragma unroll
          for (int u = 0; u < U; ++u) {
            uint64_t q0, q1;
            const bool f0 = qg_quant62_sq_fast(__uint_as_float(v[u].x), __uint_as_float(v[u].y), &q0);
            const bool f1 = qg_quant62_sq_fast(__uint_as_float(v[u].z), __uint_as_float(v[u].w), &q1);
            w[i0 + u] = q0 + q1;
            slow |= (unsigned)!(f0 && f1) << u;
          }
          if (__any_sync(0xffffffffu, slow)) {  // the FP64 expression
#pragma unroll
            for (int u = 0; u < U; ++u)
              if (slow & (1u << u)) {
                const float2 x0 = make_float2(__uint_as_float(v[u].x), __uint_as_float(v[u].y));
                const float2 x1 = make_float2(__uint_as_float(v[u].z), __uint_as_float(v[u].w));
                w[i0 + u] = quant(p_of<R>(x0)) + quant(p_of<R>(x1));
              }
          }
        }
#pragma unroll
        for (int o = 8, K = LOADS; o >= 1; o >>= 1, K >>= 1) {
          const bool up = (lane & o) != 0;
#pragma unroll
          for (int i = 0; i < K / 2; ++i) {
            const unsigned long long send = up ? w[i] : w[i + K / 2];
            const unsigned long long keep = up ? w[i + K / 2] : w[i];
            w[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
          }
        }
        csum[c0 + 2 * (uint64_t)(lane & 15) + (uint64_t)(lane >> 4)] = w[0];
        bq = w[0];
      } else {
#pragma unroll
        for (int i0 = 0; i0 < LOADS; i0 += U) {
          uint4 v[U];
#pragma unroll
          for (int u = 0; u < U; ++u) v[u] = __ldg(src + (i0 + u) * 32 + lane);
          uint64_t qs[U];
          bool big = false;
#pragma unroll
          for (int u = 0; u < U; ++u)  // high words: sign, exponent, top of the significand
            big |= max(v[u].y & 0x7FFFFFFFu, v[u].w & 0x7FFFFFFFu) >= (1013u << 20);
          unsigned slow = (1u << U) - 1;
          if (!__any_sync(0xffffffffu, big)) {
            slow = 0;
#pragma unroll
            for (int u = 0; u < U; ++u) {
              const bool f = qg_quant62_sq_fast(__hiloint2double((int)v[u].y, (int)v[u].x),
                                                __hiloint2double((int)v[u].w, (int)v[u].z), &qs[u]);
              slow |= (unsigned)!f << u;
            }
          }
          if (__any_sync(0xffffffffu, slow)) {  // the FP64 expression
#pragma unroll
            for (int u = 0; u < U; ++u)
              if (slow & (1u << u)) {
                const double2 x = make_double2(__hiloint2double((int)v[u].y, (int)v[u].x),
                                               __hiloint2double((int)v[u].w, (int)v[u].z));
                qs[u] = quant(p_of<R>(x));
              }
          }
          // load u holds chunk i0 + u across the warp: recursive halving over lane bits 4,
          // 3, 2 (7 exchanges) leaves lane l a partial of chunk i0 + ((l >> 2) & 7), and two
          // butterfly steps over bits 1, 0 complete it (5 exchanges per chunk before)
#pragma unroll
          for (int o = 16, K = U; o >= 4; o >>= 1, K >>= 1) {
            const bool up = (lane & o) != 0;
#pragma unroll
            for (int i = 0; i < K / 2; ++i) {
              const uint64_t send = up ? qs[i] : qs[i + K / 2];
              const uint64_t keep = up ? qs[i + K / 2] : qs[i];
              qs[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
            }
          }
          unsigned long long q = qs[0];
          q += __shfl_xor_sync(0xffffffffu, q, 2);
          q += __shfl_xor_sync(0xffffffffu, q, 1);
          if ((lane & 3) == 0) {
            csum[c0 + (uint64_t)(i0 + ((lane >> 2) & 7))] = q;
            bq += q;
          }
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) bq += __shfl_xor_sync(0xffffffffu, bq, o);
    } else {
      for (int c = warp; c < g.cpb; c += 8) {
        uint64_t chunk = b * g.cpb + c;
        unsigned long long q = 0;
        if (lane < g.ch) q = quant(p_of<R>(s[chunk * g.ch + lane]));
        for (int o = 16; o > 0; o >>= 1) q += __shfl_down_sync(0xffffffffu, q, o);
        if (lane == 0) {
          csum[chunk] = q;
          bq += q;
        }
      }
    }
    if (lane == 0) wq[warp] = bq;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long t = 0;
      for (int w = 0; w < 8; ++w) t += wq[w];
      bsum[b] = t;
    }
    __syncthreads();
  }
}

// single CTA: exclusive prefix of block sums (bpre[nb] = T) and the FP64 total
// T 2^-62 + N 2^-63: every quantised probability lost less than one unit of
// 2^-62 to the floor, so the estimate is within N 2^-63 of sum p (2e-9 at 34
// qubits, well inside the 1e-8 normalisation tolerance).
__global__ void __launch_bounds__(1024) k_samp_scan(const unsigned long long* __restrict__ bsum, uint64_t nb,
                                                    uint64_t n_amps, unsigned long long* __restrict__ bpre,
                                                    double* __restrict__ total) {
  __shared__ unsigned long long sh[1024];
  __shared__ unsigned long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (uint64_t base = 0; base < nb; base += 1024) {
    uint64_t i = base + threadIdx.x;
    unsigned long long v = i < nb ? bsum[i] : 0ULL;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {  // Hillis-Steele inclusive scan
      unsigned long long add = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0ULL;
      __syncthreads();
      sh[threadIdx.x] += add;
      __syncthreads();
    }
    if (i < nb) bpre[i] = carry + sh[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += sh[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    total[0] = (double)carry * 0x1p-62 + (double)n_amps * 0x1p-63;
    bpre[nb] = carry;
  }
}

// one warp per shot
template <typename R>
__global__ void __launch_bounds__(256) k_samp_resolve(const typename C2<R>::T* __restrict__ s, SampleGeom g,
                                                      const unsigned long long* __restrict__ csum,
                                                      const unsigned long long* __restrict__ bpre, uint64_t shots,
                                                      uint64_t seed, uint64_t* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  const unsigned long long T = bpre[g.nb];
  for (uint64_t shot = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; shot < shots; shot += warps) {
    if (T == 0) {
      if (lane == 0) out[shot] = 0;
      continue;
    }
    unsigned long long u = __umul64hi(draw64(seed, shot, 0u), T);
    // block: first b with bpre[b+1] > u
    uint64_t lo = 0, hi = g.nb - 1;
    while (lo < hi) {
      uint64_t mid = (lo + hi) >> 1;
      if (bpre[mid + 1] > u) hi = mid; else lo = mid + 1;
    }
    const uint64_t b = lo;
    unsigned long long r = u - bpre[b];
    // chunk within block: cpb <= 256 chunk sums, 8 per lane
    const int per = (g.cpb + 31) / 32;
    unsigned long long loc[8];
    unsigned long long mine = 0;
    for (int k = 0; k < per; ++k) {
      int c = lane * per + k;
      loc[k] = c < g.cpb ? csum[b * g.cpb + c] : 0ULL;
      mine += loc[k];
    }
    unsigned long long incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    unsigned long long excl = incl - mine;
    unsigned ballot = __ballot_sync(0xffffffffu, incl > r);
    int owner = ballot ? __ffs(ballot) - 1 : 31;
    int chunk_in_block = 0;
    unsigned long long before = 0;
    if (lane == owner) {
      unsigned long long c = excl;
      int kk = 0;
      for (; kk < per; ++kk) {
        if (c + loc[kk] > r) break;
        c += loc[kk];
      }
      if (kk >= per) kk = per - 1;
      chunk_in_block = lane * per + kk;
      before = c;
      if (chunk_in_block >= g.cpb) chunk_in_block = g.cpb - 1;
    }
    chunk_in_block = __shfl_sync(0xffffffffu, chunk_in_block, owner);
    before = __shfl_sync(0xffffffffu, before, owner);
    unsigned long long r2 = r - before;
    const uint64_t chunk = b * g.cpb + chunk_in_block;
    unsigned long long q = lane < g.ch ? quant(p_of<R>(s[chunk * g.ch + lane])) : 0ULL;
    unsigned long long qi = q;
    for (int o = 1; o < 32; o <<= 1) {
      unsigned long long v = __shfl_up_sync(0xffffffffu, qi, o);
      if (lane >= o) qi += v;
    }
    unsigned bl = __ballot_sync(0xffffffffu, (lane < g.ch) && qi > r2);
    int pick = bl ? __ffs(bl) - 1 : g.ch - 1;
    if (lane == 0) out[shot] = chunk * g.ch + pick;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
unsigned long long kernel_launch_count() { return g_launches.load(); }
void count_launch(int k) { counted(k); }

int reduce_blocks_for(int n) {
  uint64_t N = 1ULL << n;
  uint64_t b = (N + 255) / 256;
  if (b > (uint64_t)kSMs * 4) b = (uint64_t)kSMs * 4;
  return (int)(b < 1 ? 1 : b);
}

cudaError_t launch_set_basis(void* s, int precision, int n, uint64_t idx, cudaStream_t st) {
  size_t bytes = (precision == QG_C64 ? 8ULL : 16ULL) << n;
  cudaError_t e = cudaMemsetAsync(s, 0, bytes, st);
  if (e != cudaSuccess) return e;
  k_set_one<<<1, 1, 0, st>>>(s, precision, idx);
  counted();
  return cudaGetLastError();
}

cudaError_t launch_plain_op(void* s, int precision, int n, const GOp& op, cudaStream_t st) {
  return precision == QG_C64 ? plain_op_t<float>(s, n, op, st) : plain_op_t<double>(s, n, op, st);
}

cudaError_t launch_c128_to_c64(const double* src, float* dst, uint64_t count, cudaStream_t st) {
  k_c128_to_c64<<<grid_for(count, 256), 256, 0, st>>>((const double2*)src, (float2*)dst, count);
  counted();
  return cudaGetLastError();
}
cudaError_t launch_c64_to_c128(const float* src, double* dst, uint64_t count, cudaStream_t st) {
  k_c64_to_c128<<<grid_for(count, 256), 256, 0, st>>>((const float2*)src, (double2*)dst, count);
  counted();
  return cudaGetLastError();
}

cudaError_t launch_probabilities(const void* s, int precision, int n, double* d_p, cudaStream_t st) {
  uint64_t N = 1ULL << n;
  if (precision == QG_C64) k_probs<float><<<grid_for(N, 256), 256, 0, st>>>((const float2*)s, N, d_p);
  else k_probs<double><<<grid_for(N, 256), 256, 0, st>>>((const double2*)s, N, d_p);
  counted();
  return cudaGetLastError();
}

cudaError_t launch_norm2(const void* s, int precision, int n, double* d_part, int nblocks, cudaStream_t st) {
  uint64_t N = 1ULL << n;
  if (precision == QG_C64) k_norm2<float><<<nblocks, 256, 0, st>>>((const float2*)s, N, d_part);
  else k_norm2<double><<<nblocks, 256, 0, st>>>((const double2*)s, N, d_part);
  counted();
  return cudaGetLastError();
}

cudaError_t launch_pauli_expect(const void* s, int precision, int n, uint64_t xmask, uint64_t zmask, int ny,
                                double* d_part, int nblocks, cudaStream_t st) {
  uint64_t N = 1ULL << n;
  if (precision == QG_C64) k_pauli<float><<<nblocks, 256, 0, st>>>((const float2*)s, N, xmask, zmask, ny, d_part);
  else k_pauli<double><<<nblocks, 256, 0, st>>>((const double2*)s, N, xmask, zmask, ny, d_part);
  counted();
  return cudaGetLastError();
}

cudaError_t launch_expect_1q(const void* s, int precision, int n, int bit, const double* o8, double* d_part,
                             int nblocks, cudaStream_t st) {
  uint64_t N = 1ULL << n;
  Mat<double> o = to_mat<double>(o8);
  if (precision == QG_C64) k_expect1q<float><<<nblocks, 256, 0, st>>>((const float2*)s, N, bit, o, d_part);
  else k_expect1q<double><<<nblocks, 256, 0, st>>>((const double2*)s, N, bit, o, d_part);
  counted();
  return cudaGetLastError();
}

cudaError_t launch_inner(const void* a, const void* b, int precision, int n, double* d_part, int nblocks,
                         cudaStream_t st) {
  uint64_t N = 1ULL << n;
  if (precision == QG_C64) k_inner<float><<<nblocks, 256, 0, st>>>((const float2*)a, (const float2*)b, N, d_part);
  else k_inner<double><<<nblocks, 256, 0, st>>>((const double2*)a, (const double2*)b, N, d_part);
  counted();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Noisy trajectories: end of a shot. The Kraus operators were applied without
// renormalisation, so each distinct trajectory state is first scaled by 1 / ||a||
// (state.clj:524-551: every amplitude times (/ 1.0 norm)), one CTA per state. Then
// every shot draws one outcome from its state the way the shot sampler draws:
// quantised probabilities q_i = floor(p_i 2^62), their integer total T,
// u = floor(r64 T / 2^64) and the first i whose inclusive prefix sum exceeds u, one
// CTA per shot. Each thread owns a contiguous chunk of the state; the chunk sums are
// scanned in shared memory and the chunk that holds u is walked by its thread.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(256) k_traj_normalise(void* const* __restrict__ states, int n,
                                                        double* __restrict__ norm2) {
  using T = typename C2<R>::T;
  T* s = reinterpret_cast<T*>(states[blockIdx.x]);
  const uint64_t N = 1ULL << n;
  const uint64_t chunk = (N + blockDim.x - 1) / blockDim.x;
  const uint64_t lo = min(N, (uint64_t)threadIdx.x * chunk), hi = min(N, lo + chunk);
  __shared__ DD red[8];
  __shared__ double scale_sh;
  DD acc{0, 0};
  for (uint64_t i = lo; i < hi; ++i) two_sum_acc(acc, p_of<R>(s[i]));
  for (int o = 16; o > 0; o >>= 1) {
    DD w;
    w.s = __shfl_down_sync(0xffffffffu, acc.s, o);
    w.c = __shfl_down_sync(0xffffffffu, acc.c, o);
    acc = dd_add(acc, w);
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    DD t = red[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) t = dd_add(t, red[w]);
    const double nn = t.s + t.c;
    norm2[blockIdx.x] = nn;
    scale_sh = nn > 0 ? 1.0 / sqrt(nn) : 0.0;
  }
  __syncthreads();
  const double sc = scale_sh;
  for (uint64_t i = lo; i < hi; ++i) {
    T a = s[i];
    a.x = (R)((double)a.x * sc);
    a.y = (R)((double)a.y * sc);
    s[i] = a;
  }
}

template <typename R>
__global__ void __launch_bounds__(256) k_traj_sample(void* const* __restrict__ states,
                                                     const int32_t* __restrict__ state_of, int n, int shift,
                                                     uint64_t seed, uint64_t traj0, uint32_t stream,
                                                     uint64_t* __restrict__ out) {
  using T = typename C2<R>::T;
  const T* s = reinterpret_cast<const T*>(states[state_of[blockIdx.x]]);
  const uint64_t N = 1ULL << n;
  const uint64_t chunk = (N + blockDim.x - 1) / blockDim.x;
  const uint64_t lo = min(N, (uint64_t)threadIdx.x * chunk), hi = min(N, lo + chunk);
  __shared__ unsigned long long pre[256];
  unsigned long long q = 0;
  for (uint64_t i = lo; i < hi; ++i) q += quant(p_of<R>(s[i]));
  pre[threadIdx.x] = q;
  __syncthreads();
  for (unsigned o = 1; o < blockDim.x; o <<= 1) {  // inclusive scan of the chunk sums
    const unsigned long long add = threadIdx.x >= o ? pre[threadIdx.x - o] : 0ULL;
    __syncthreads();
    pre[threadIdx.x] += add;
    __syncthreads();
  }
  const unsigned long long total = pre[blockDim.x - 1];
  if (total == 0) {
    if (threadIdx.x == 0) out[blockIdx.x] = 0;
    return;
  }
  const unsigned long long u = __umul64hi(draw64(seed, traj0 + blockIdx.x, stream), total);
  const unsigned long long before = pre[threadIdx.x] - q;
  if (u >= before && u < pre[threadIdx.x]) {
    unsigned long long c = before;
    for (uint64_t i = lo; i < hi; ++i) {
      c += quant(p_of<R>(s[i]));
      if (c > u) {
        out[blockIdx.x] = i >> shift;
        break;
      }
    }
  }
}

cudaError_t launch_traj_normalise(int precision, void* const* d_states, int nstates, int n, double* d_norm2,
                                  cudaStream_t st) {
  if (nstates < 1) return cudaSuccess;
  if (precision == QG_C64) k_traj_normalise<float><<<nstates, 256, 0, st>>>(d_states, n, d_norm2);
  else k_traj_normalise<double><<<nstates, 256, 0, st>>>(d_states, n, d_norm2);
  counted();
  return cudaGetLastError();
}

cudaError_t launch_traj_sample(int precision, void* const* d_states, const int32_t* d_state_of, int nshots, int n,
                               int shift, uint64_t seed, uint64_t traj0, uint32_t stream, uint64_t* d_out,
                               cudaStream_t st) {
  if (nshots < 1) return cudaSuccess;
  if (precision == QG_C64)
    k_traj_sample<float><<<nshots, 256, 0, st>>>(d_states, d_state_of, n, shift, seed, traj0, stream, d_out);
  else
    k_traj_sample<double><<<nshots, 256, 0, st>>>(d_states, d_state_of, n, shift, seed, traj0, stream, d_out);
  counted();
  return cudaGetLastError();
}

cudaError_t launch_compare(const void* a, int precision, const void* b, int n, double* d_part, double* d_max,
                           int nblocks, cudaStream_t st) {
  uint64_t N = 1ULL << n;
  if (precision == QG_C64)
    k_compare<float><<<nblocks, 256, 0, st>>>((const float2*)a, (const double2*)b, N, d_part, d_max);
  else
    k_compare<double><<<nblocks, 256, 0, st>>>((const double2*)a, (const double2*)b, N, d_part, d_max);
  counted();
  return cudaGetLastError();
}

cudaError_t launch_marginal_host(const void* s, int precision, int n, const int* h_bits, const int* d_bits, int m,
                                 int nbx, double* d_pm, unsigned long long* d_qm, cudaStream_t st) {
  uint64_t zero = 0;
  for (int k = 0; k < m; ++k) zero |= 1ULL << h_bits[k];
  Fixed f = make_fixed(zero, 0);
  uint64_t work = (1ULL << n) >> m;
  dim3 grid(nbx, 1u << m);
  if (precision == QG_C64)
    k_marginal<float><<<grid, 256, 0, st>>>((const float2*)s, work, f, m, d_bits, d_pm, d_qm);
  else
    k_marginal<double><<<grid, 256, 0, st>>>((const double2*)s, work, f, m, d_bits, d_pm, d_qm);
  counted();
  return cudaGetLastError();
}

cudaError_t launch_gather(const void* s, int precision, const uint64_t* d_idx, int64_t count, double* d_out,
                          cudaStream_t st) {
  int g = grid_for((uint64_t)count, 256);
  if (precision == QG_C64) k_gather<float><<<g, 256, 0, st>>>((const float2*)s, d_idx, count, d_out);
  else k_gather<double><<<g, 256, 0, st>>>((const double2*)s, d_idx, count, d_out);
  counted();
  return cudaGetLastError();
}

cudaError_t launch_density(const void* s, int precision, int n, double* d_rho, cudaStream_t st) {
  uint64_t N = 1ULL << n;
  int g = grid_for(N * N, 256);
  if (precision == QG_C64) k_density<float><<<g, 256, 0, st>>>((const float2*)s, N, d_rho);
  else k_density<double><<<g, 256, 0, st>>>((const double2*)s, N, d_rho);
  counted();
  return cudaGetLastError();
}

size_t sampler_scratch_bytes(int n, uint64_t shots) {
  (void)shots;
  return sampler_scratch_bytes_at(n);  // the layout of sample_geom(n) below
}

cudaError_t launch_sample(const void* s, int precision, int n, uint64_t shots, uint64_t seed, void* d_scratch,
                          uint64_t* d_outcomes, double* d_total, cudaStream_t st) {
  SampleGeom g = sample_geom(n);
  unsigned long long* csum = (unsigned long long*)d_scratch;
  unsigned long long* bsum = csum + g.nchunks;
  unsigned long long* bpre = bsum + g.nb;
  int grid = (int)(g.nb < (uint64_t)kSMs * 8 ? g.nb : (uint64_t)kSMs * 8);
  if (precision == QG_C64)
    k_samp_sums<float><<<grid, 256, 0, st>>>((const float2*)s, g, csum, bsum);
  else
    k_samp_sums<double><<<grid, 256, 0, st>>>((const double2*)s, g, csum, bsum);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_samp_scan<<<1, 1024, 0, st>>>(bsum, g.nb, g.N, bpre, d_total);
  e = cudaGetLastError();
  counted(2);
  if (e != cudaSuccess || shots == 0) return e;
  uint64_t warps_needed = shots;
  uint64_t blocks = (warps_needed * 32 + 255) / 256;
  if (blocks > (uint64_t)kSMs * 16) blocks = (uint64_t)kSMs * 16;
  if (precision == QG_C64)
    k_samp_resolve<float><<<(unsigned)blocks, 256, 0, st>>>((const float2*)s, g, csum, bpre, shots, seed, d_outcomes);
  else
    k_samp_resolve<double><<<(unsigned)blocks, 256, 0, st>>>((const double2*)s, g, csum, bpre, shots, seed,
                                                             d_outcomes);
  counted();
  return cudaGetLastError();
}

}  // namespace qg
