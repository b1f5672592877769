// Specialised pass kernels: one sm_103a kernel per tiled pass of a program.
//
// The tiled executor (tile.cu) interprets a pass's op records per tile: every
// op costs a dispatch, a load of its coefficients and, because the op switch
// joins all gate classes, copies of the amplitude registers at the join. For
// large states the same pass runs over 2^(n-12) tiles, so this file turns each
// pass into straight-line code instead: the generator below writes one CUDA
// kernel per pass (matrix entries as exact hex-float literals, register slots,
// layouts and conditions resolved), NVRTC compiles the kernels of a program for
// sm_103a in a few parallel translation units, and the runtime launches them in
// place of the interpreted passes. Compiled programs are cached per device by
// their generated source, so repeated circuits (benchmark steps, served
// duplicates) compile once.
//
// The arithmetic is that of the interpreted path's policies, applied in the same
// gate order: complex64 in FP32 (with FMA contraction), complex128 as
// double-float pairs on the FP32 pipes (pass_prelude.cuh). The exact FP64
// policy and dense fused blocks stay with the interpreter.
//
// NVRTC is loaded with dlopen: without it (or when a compile fails) programs run
// on the interpreted kernels, which are CUDA code on the same device.
#include <dlfcn.h>
#include <nvrtc.h>

#include <algorithm>
#include <chrono>
#include <list>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <sstream>
#include <thread>
#include <unordered_map>

#include "csa.h"
#include "qgpu_internal.h"

namespace qg {

extern const char kEmbedPassPrelude[];
extern const char kEmbedDf64[];

namespace {

struct NvrtcApi {
  decltype(&nvrtcCreateProgram) create = nullptr;
  decltype(&nvrtcCompileProgram) compile = nullptr;
  decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
  decltype(&nvrtcGetProgramLog) log = nullptr;
  decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
  decltype(&nvrtcGetCUBIN) cubin = nullptr;
  decltype(&nvrtcDestroyProgram) destroy = nullptr;
  std::string error;  // empty when every entry point resolved
};

const NvrtcApi& nvrtc_api() {
  static const NvrtcApi api = [] {
    NvrtcApi a;
    const char* names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13"};
    void* h = nullptr;
    for (const char* nm : names)
      if (!h) h = dlopen(nm, RTLD_NOW | RTLD_LOCAL);
    if (!h) {
      a.error = "NVRTC (libnvrtc.so.13) is not available";
      return a;
    }
    a.create = reinterpret_cast<decltype(a.create)>(dlsym(h, "nvrtcCreateProgram"));
    a.compile = reinterpret_cast<decltype(a.compile)>(dlsym(h, "nvrtcCompileProgram"));
    a.log_size = reinterpret_cast<decltype(a.log_size)>(dlsym(h, "nvrtcGetProgramLogSize"));
    a.log = reinterpret_cast<decltype(a.log)>(dlsym(h, "nvrtcGetProgramLog"));
    a.cubin_size = reinterpret_cast<decltype(a.cubin_size)>(dlsym(h, "nvrtcGetCUBINSize"));
    a.cubin = reinterpret_cast<decltype(a.cubin)>(dlsym(h, "nvrtcGetCUBIN"));
    a.destroy = reinterpret_cast<decltype(a.destroy)>(dlsym(h, "nvrtcDestroyProgram"));
    if (!a.create || !a.compile || !a.log_size || !a.log || !a.cubin_size || !a.cubin || !a.destroy)
      a.error = "NVRTC lacks an entry point";
    return a;
  }();
  return api;
}

// exact float literal (C++17 hexadecimal floating literal)
std::string flit(float f) {
  char b[64];
  std::snprintf(b, sizeof(b), "%af", (double)f);
  return b;
}
std::string hex64(uint64_t v) {
  char b[40];
  std::snprintf(b, sizeof(b), "0x%llxull", (unsigned long long)v);
  return b;
}
std::string hex32(uint32_t v) {
  char b[24];
  std::snprintf(b, sizeof(b), "0x%xu", v);
  return b;
}

inline bool hi_lo_nonzero(const TOp& t, int q) { return t.mf[8 + q] != 0.0f; }

// ---------------------------------------------------------------------------
// Source generation for one pass
// ---------------------------------------------------------------------------
// Register planning for the generated kernels: every thread holds 2^R amplitudes
// whose local indices differ in R "register bits". Consecutive ops whose
// non-diagonal bits fit in R bits share one layout; the remaining register bits
// go to the local bits the group's conditions use most, so those conditions
// select registers at compile time. (The interpreter plans the same way with
// R = 3 in compile.cpp; here R is a property of the kernel shape.)
// table = true (kernels shared by the states of a sweep group): parity and
// blockade masks are data (they differ between members, for instance between
// QAOA graphs), so the layout must not depend on them: ops keep their order
// (no sinking, no look-ahead) and the free register bits ignore those masks.
std::vector<TOp> plan_layouts(const TOp* ops, int nops, int k, int R, bool table = false, bool pair0 = false) {
  auto required = [](const TOp& t) -> uint32_t {
    if (t.kind == OK_U2) return 1u << t.t;
    if (t.kind == OK_SWAP) return (1u << t.t) | (1u << t.t2);
    return 0u;
  };
  auto data_mask = [&](const TOp& t) { return table && (t.kind == OK_PARITY || t.kind == OK_BLOCKADE); };
  // Phase gates sink to the latest point they can reach: a phase commutes with
  // every gate that does not change one of its bits, so it waits until a gate
  // targets one of them (or the pass ends). Phases then arrive in runs, which the
  // generator applies through shared per-mask factors (phase_run).
  std::vector<TOp> in;
  {
    std::vector<TOp> pending;
    auto flush = [&](uint32_t bits, bool all) {
      std::vector<TOp> keep;
      for (const TOp& p : pending) {
        if (all || (p.lmask & bits)) in.push_back(p);
        else keep.push_back(p);
      }
      pending.swap(keep);
    };
    for (int i = 0; i < nops; ++i) {
      const TOp& t = ops[i];
      if (t.kind == OK_LAYOUT) continue;
      if (t.kind == OK_PHASE && !table) {
        pending.push_back(t);
        continue;
      }
      const bool diagonal_other = t.kind == OK_BLOCKADE || t.kind == OK_PARITY || t.kind == OK_COLLAPSE;
      flush(required(t), diagonal_other || t.kind == OK_DENSE);
      in.push_back(t);
    }
    flush(0, true);
  }
  std::vector<TOp> out;
  auto cond_bits = [&](const TOp& t) -> uint32_t {
    if (data_mask(t)) return 0u;
    return t.kind == OK_U2 || t.kind == OK_SWAP ? t.lcmask : t.lmask;
  };
  // Groups are formed with look-ahead: an op joins the current layout when its
  // non-diagonal bits fit the register bits and it commutes with every op left
  // out before it (no shared bit that either changes; tile bits are only ever
  // diagonal, so local bits decide). Fewer layouts mean fewer trips through
  // shared memory and fewer barriers.
  std::vector<char> taken(in.size(), 0);
  size_t first = 0;
  while (first < in.size()) {
    uint32_t rb = 0, changed = 0, seen = 0;
    std::vector<TOp> grp;
    for (size_t j = first; j < in.size(); ++j) {
      if (taken[j]) continue;
      const uint32_t req = required(in[j]), tb = req | cond_bits(in[j]);
      const bool commutes = (req & seen) == 0 && ((tb & ~req) & changed) == 0;
      if (commutes && __builtin_popcount(rb | req) <= R) {
        rb |= req;
        grp.push_back(in[j]);
        taken[j] = 1;
      } else {
        if (table) break;
        changed |= req;
        seen |= tb;
      }
    }
    while (first < in.size() && taken[first]) ++first;
    int uses[32] = {0};
    for (const TOp& t : grp) {
      const uint32_t cm = cond_bits(t);
      for (int b = 0; b < k; ++b)
        if (cm & (1u << b)) ++uses[b];
    }
    while (__builtin_popcount(rb) < R) {
      int best = -1;
      for (int b = k - 1; b >= 0; --b)
        if (!(rb & (1u << b)) && (best < 0 || uses[b] > uses[best])) best = b;
      // pair0 (complex64): a free register slot that no condition asks for takes tile
      // bit 0, so registers j and j + 1 share one 16-byte slot pair in shared memory and
      // a layout change moves them with one access
      if (pair0 && uses[best] == 0 && !(rb & 1u)) best = 0;
      rb |= 1u << best;
    }
    int pos[5], np = 0;
    for (int b = 0; b < k && np < R; ++b)
      if (rb & (1u << b)) pos[np++] = b;
    TOp lay;
    std::memset(&lay, 0, sizeof(lay));
    lay.kind = OK_LAYOUT;
    for (int q = 0; q < R; ++q) lay.dbits[q] = pos[q];
    out.push_back(lay);
    auto rpos = [&](int b) {
      for (int q = 0; q < R; ++q)
        if (pos[q] == b) return q;
      return -1;
    };
    auto reg_part = [&](uint32_t m) {
      uint32_t r = 0;
      for (int q = 0; q < R; ++q)
        if (m & (1u << pos[q])) r |= 1u << q;
      return r;
    };
    for (const TOp& t0 : grp) {
      TOp t = t0;
      uint32_t m = 0, v = 0;
      if (t.kind == OK_U2) {
        t.t2 = rpos(t.t);
        m = v = t.lcmask;
      } else if (t.kind == OK_SWAP) {
        const int a = rpos(t.t), b = rpos(t.t2);
        t.dbits[0] = a < b ? a : b;
        t.dbits[1] = a < b ? b : a;
        m = v = t.lcmask;
      } else if (t.kind == OK_PHASE) {
        m = v = t.lmask;
      } else if (t.kind == OK_COLLAPSE) {
        m = t.lmask;
        v = t.lval;
      } else {  // BLOCKADE, PARITY: the mask selects the bits to count
        m = t.lmask;
        v = 0;
      }
      t.rmask = reg_part(m);
      t.rval = reg_part(v);
      t.tmask = m & ~rb;
      t.tval = v & ~rb;
      out.push_back(t);
    }
  }
  return out;
}

// A real or RX-shaped 2x2 whose diagonal is (1, +-1) (a rotation with its
// diagonal factored out): 1 = [[1, b], [c, 1]], 2 = [[1, b], [c, -1]], else 0.
int unit_diagonal(const TOp& t) {
  if (t.kind != OK_U2 || t.m[0] != 1.0 || t.m[1] != 0.0 || t.m[7] != 0.0) return 0;
  if (t.cls == U2_RXLIKE && t.m[6] == 1.0) return 1;
  if (t.cls == U2_REAL && !(t.m[2] == 1.0 && t.m[4] == 1.0)) return t.m[6] == 1.0 ? 1 : t.m[6] == -1.0 ? 2 : 0;
  return 0;
}

// Runs of at least two consecutive parity ops (RZZ) with equal phase pairs: their
// combined phase depends only on how many of them see odd parity, m, so each
// register takes one entry of a table of p0^(E-m) p1^m instead of E products.
bool same_parity_phases(const TOp& a, const TOp& b) {
  return a.kind == OK_PARITY && b.kind == OK_PARITY && a.m[0] == b.m[0] && a.m[1] == b.m[1] && a.m[2] == b.m[2] &&
         a.m[3] == b.m[3];
}
// [begin, end) of the parity run starting at ops[i], or end = i + 1 when none
int parity_run_end(const TOp* ops, int nops, int i) {
  int j = i + 1;
  while (j < nops && same_parity_phases(ops[i], ops[j])) ++j;
  return j;
}
// p0^(E-m) p1^m for m = 0..E, in FP64
std::vector<std::complex<double>> parity_table(const TOp& t, int E) {
  const std::complex<double> p0(t.m[0], t.m[1]), p1(t.m[2], t.m[3]);
  std::vector<std::complex<double>> tab(E + 1);
  for (int m = 0; m <= E; ++m) {
    std::complex<double> v(1.0, 0.0);
    for (int q = 0; q < E - m; ++q) v *= p0;
    for (int q = 0; q < m; ++q) v *= p1;
    tab[m] = v;
  }
  return tab;
}

// Kernel shape: register bits per thread, tile buffers, CTAs per SM.
struct Shape {
  int rbits, bufs, ctas;
};
// Measured on the 30-qubit layered + QFT circuit: double-float keeps 8 registers
// per thread, two tile buffers and one CTA per SM (16 registers per thread spill
// at two CTAs and starve latency hiding at one); complex64 holds 16 registers per
// thread with two buffers and two CTAs per SM.
Shape shape_for(int prec) {
  if (prec == QG_C128) return Shape{3, 2, 1};
  return Shape{4, 2, 2};
}
// A program's own shape (set by the autotuner, qg_tuning) or the precision's default.
Shape shape_of(const Program& prog, int prec) {
  if (prog.rbits > 0 && prog.bufs > 0 && prog.ctas > 0) return Shape{prog.rbits, prog.bufs, prog.ctas};
  return shape_for(prec);
}

class PassGen {
 public:
  // table = true: the matrix entries are read from a per-state table in shared
  // memory (cs[16 * op + q], op numbered in the pass's own op order) instead of
  // literals, so one kernel serves every state of a parameter sweep.
  PassGen(std::ostringstream& o, const PassDesc& pd, const TOp* ops, int nops, int prec, int io, bool table,
          Shape sh)
      : out_(o), pd_(pd), df_(prec == QG_C128), io_(io), tab_(table), sh_(sh) {
    std::vector<TOp> tagged(ops, ops + nops);
    for (int i = 0; i < nops; ++i) {
      tagged[i].pad1 = i;  // the op's row in the coefficient table
      if (ops[i].kind == OK_DENSE) unsupported_ = true;
      if (table && (ops[i].kind == OK_BLOCKADE || ops[i].kind == OK_COLLAPSE)) unsupported_ = true;
    }
    if (!unsupported_) plan_ = plan_layouts(tagged.data(), nops, pd.k, sh_.rbits, table, !df_);
    // pairs handed over by the previous pass may carry unnormalised operations
    if (io & kTileInPairs) carry_ = kRenormEvery / 2 - 1;
    ops_ = plan_.data();
    nops_ = (int)plan_.size();
    ns_ = 1 << sh_.rbits;
    if (ns_ > kMaxRegs) unsupported_ = true;  // the generator's per-register tables hold 16
  }

  // false: the pass holds an op the generator does not specialise
  bool supported() const { return !unsupported_; }

  // ns_name: the namespace of the pass's P (default s<id> / p<id>); kernel = false emits
  // only the namespace (the level kernels of a sweep call several passes' bodies)
  void emit(int id, const std::string& ns_name = std::string(), bool kernel = true) {
    const int E = df_ ? 16 : 8;
    uint64_t lm = 0;
    for (int j = 0; j < pd_.k; ++j) lm |= 1ULL << pd_.lbits[j];
    const std::string ns = ns_name.empty() ? (tab_ ? "s" : "p") + std::to_string(id) : ns_name;
    body();  // into o_; tables it needs go to pre_
    out_ << "namespace " << ns << " {\n" << pre_.str() << "struct P {\n";
    out_ << "  static constexpr int E = " << E << ", K_BITS = " << pd_.k << ", KLOW = " << pd_.klow
         << ", R_BITS = " << sh_.rbits << ", BUFS = " << sh_.bufs << ";\n";
    out_ << "  static constexpr qgp::u64 LM = " << hex64(lm) << ";\n";
    // run offsets: bit j - klow of the run index h deposits at lbits[j]
    out_ << "  static __device__ __forceinline__ qgp::u64 hioff(int h) {\n    qgp::u64 o = 0;\n";
    for (int j = pd_.klow; j < pd_.k; ++j)
      out_ << "    o |= (qgp::u64)((h >> " << (j - pd_.klow) << ") & 1) << " << pd_.lbits[j] << ";\n";
    out_ << "    return o;\n  }\n";
    out_ << "  static __device__ __forceinline__ qgp::u64 tile_base(qgp::u64 t) {\n    return 0";
    for (int r = 0; r < pd_.nruns; ++r)
      out_ << " | (((t >> " << pd_.run_src[r] << ") & " << hex64((1ULL << pd_.run_len[r]) - 1) << ") << "
           << pd_.run_dst[r] << ")";
    out_ << ";\n  }\n";
    out_ << "  static __device__ __forceinline__ void body(unsigned char* buf, qgp::u64 base, "
            "const float* __restrict__ cs) {\n";
    out_ << "    using namespace qgp;\n    const unsigned tid = threadIdx.x;\n    (void)base; (void)tid; (void)cs;\n";
    out_ << o_.str();
    out_ << "  }\n};\n}  // namespace " << ns << "\n";
    if (!kernel) return;
    out_ << "extern \"C\" __global__ void __launch_bounds__(" << ((1 << pd_.k) >> sh_.rbits) << ", " << sh_.ctas
         << ") ";
    if (tab_)
      out_ << "qgs_" << id << "(unsigned char* const* __restrict__ states, const float* __restrict__ coefs, int ncoef, "
           << "unsigned long long ntiles, int nstates) {\n  qgp::run_pass_batch<" << ns
           << "::P>(states, coefs, ncoef, ntiles, nstates);\n}\n\n";
    else
      out_ << "qgp_" << id << "(unsigned char* __restrict__ state, unsigned long long ntiles) {\n  qgp::run_pass<" << ns
           << "::P>(state, ntiles);\n}\n\n";
  }

 private:
  std::ostringstream& out_;
  std::ostringstream o_;  // the body, generated first
  const PassDesc& pd_;
  bool df_;
  int io_;
  bool tab_;
  Shape sh_;
  bool unsupported_ = false;
  std::vector<TOp> plan_;
  const TOp* ops_ = nullptr;
  int nops_ = 0;
  int ns_ = 8;  // registers (amplitudes) per thread: at most kMaxRegs
  static constexpr int kMaxRegs = 16;
  // double-float: operations applied to each register since its last renormalisation
  int since_[kMaxRegs] = {0};
  static constexpr int kRenormEvery = 6;

  void touched(int j) {
    if (!df_) return;
    if (++since_[j] >= kRenormEvery) {
      o_ << "    r" << j << " = DF::renorm(r" << j << ");\n";
      since_[j] = 0;
    }
  }
  // Before registers go to shared memory: renormalise those halfway to the
  // limit; the rest keep their count, and after the next layout every register
  // starts from the largest count left (it may hold any of the stored values).
  void renorm_for_store() {
    if (!df_) return;
    for (int j = 0; j < ns_; ++j)
      if (since_[j] >= kRenormEvery / 2) {
        o_ << "    r" << j << " = DF::renorm(r" << j << ");\n";
        since_[j] = 0;
      }
    carry_ = 0;
    for (int j = 0; j < ns_; ++j) carry_ = std::max(carry_, since_[j]);
  }
  int carry_ = 0;

  // Conditional X gates on register bits are not applied to the registers: a runtime
  // mask xm records them (register p holds the amplitude of logical register p ^ xm),
  // and the next store to shared memory puts register p at the slot of p ^ xm, which is
  // its slot XOR swz(deposit of xm at the register bit positions), the swizzle being
  // linear over XOR. pend_: the register bits xm may have set; rpos_: their positions in
  // the tile index under the current layout. An op that depends on a pending bit
  // (targets it, is conditioned on it or selects registers by it) first applies those
  // bits as conditional swaps (materialise).
  uint32_t pend_ = 0;
  int rpos_[4] = {0, 0, 0, 0};

  void materialise(uint32_t bits) {
    bits &= pend_;
    if (!bits) return;
    const std::string T = df_ ? "dfc" : "float2";
    for (int bb = 0; bb < sh_.rbits; ++bb) {
      if (!((bits >> bb) & 1)) continue;
      o_ << "    if (xm & " << (1u << bb) << "u) {  // pending X on register bit " << bb << "\n";
      for (int j = 0; j < ns_; ++j) {
        if ((j >> bb) & 1) continue;
        const int k = j | (1 << bb);
        o_ << "      { const " << T << " y = " << r(j) << "; " << r(j) << " = " << r(k) << "; " << r(k) << " = y; }\n";
        if (df_) since_[j] = since_[k] = std::max(since_[j], since_[k]);
      }
      o_ << "    }\n";
    }
    o_ << "    xm &= " << hex32(~bits & 0xFFu) << ";\n";
    pend_ &= ~bits;
  }
  // register p goes to the slot of logical register p ^ xm
  // complex64 with tile bit 0 as register bit 0: registers j, j + 1 (j even) fill one
  // 16-byte slot pair (the swizzle keeps bit 0)
  bool paired() const { return !df_ && rpos_[0] == 0; }
  void store_regs(const std::string& fn) {
    if (paired() && !(pend_ & 1u)) {  // a pending X of register bit 0 would swap the halves
      std::string xo = "";
      if (pend_) {
        const int E = 8;
        o_ << "    { const int xo = swz<" << E << ">((int)(0u";
        for (int bb = 0; bb < sh_.rbits; ++bb)
          if ((pend_ >> bb) & 1) o_ << " | (((xm >> " << bb << ") & 1u) << " << rpos_[bb] << ")";
        o_ << "));\n";
        xo = " ^ xo";
      }
      for (int j = 0; j < ns_; j += 2)
        o_ << "    F32::st_pair(buf, q" << j << xo << ", r" << j << ", r" << j + 1 << ");\n";
      if (pend_) o_ << "    }\n    xm = 0u;\n";
      pend_ = 0;
      return;
    }
    if (!pend_) {
      for (int j = 0; j < ns_; ++j) o_ << "    " << fn << "(buf, q" << j << ", r" << j << ");\n";
      return;
    }
    const int E = df_ ? 16 : 8;
    o_ << "    { const int xo = swz<" << E << ">((int)(0u";
    for (int bb = 0; bb < sh_.rbits; ++bb)
      if ((pend_ >> bb) & 1) o_ << " | (((xm >> " << bb << ") & 1u) << " << rpos_[bb] << ")";
    o_ << "));\n";
    for (int j = 0; j < ns_; ++j) o_ << "      " << fn << "(buf, q" << j << " ^ xo, r" << j << ");\n";
    o_ << "    }\n    xm = 0u;\n";
    pend_ = 0;
  }

  const char* pol() const { return df_ ? "DF" : "F32"; }
  std::string ld_raw() const { return df_ && !(io_ & kTileInPairs) ? "DF::ld_doubles" : std::string(pol()) + "::ld_work"; }
  std::string st_raw() const { return df_ && !(io_ & kTileOutPairs) ? "DF::st_doubles" : std::string(pol()) + "::st_work"; }

  // coefficient q of a TOp: hi literal, lo literal (double-float) or the float
  // (complex64); with a table, the entries of the current state in shared memory
  std::string h(const TOp& t, int q) const {
    if (tab_) return "cs[" + std::to_string(16 * t.pad1 + q) + "]";
    return flit(df_ ? t.mf[q] : (float)t.m[q]);
  }
  std::string l(const TOp& t, int q) const {
    if (tab_) return "cs[" + std::to_string(16 * t.pad1 + 8 + q) + "]";
    return flit(t.mf[8 + q]);
  }
  bool lo_nz(const TOp& t, int q) const { return tab_ || hi_lo_nonzero(t, q); }
  std::string b(bool v) const { return v ? "true" : "false"; }

  // condition on tile bits (gm, gv) and thread bits (tm, tv); empty when unconditional
  std::string cond(uint64_t gm, uint64_t gv, uint32_t tm, uint32_t tv) const {
    std::string c;
    if (gm) c += "((base & " + hex64(gm) + ") == " + hex64(gv) + ")";
    if (tm) {
      if (!c.empty()) c += " && ";
      c += "((lt & " + hex32(tm) + ") == " + hex32(tv) + ")";
    }
    return c;
  }

  std::string cmul(const TOp& t, int qr, int qi, const std::string& x) const {
    const float rh = t.mf[qr], rl = t.mf[8 + qr], ih = t.mf[qi], il = t.mf[8 + qi];
    const bool same = ih == rh && il == rl, opp = ih == -rh && il == -rl;
    if (df_ && !tab_ && rh != 0.0f && (same || opp)) {
      // (a + i a) or (a - i a): both parts of the constant the same pair up to sign
      const bool neg = !same;
      return "df_cmul_diag<" + b(lo_nz(t, qr)) + ", " + b(neg) + ">(" + h(t, qr) + ", " + l(t, qr) + ", " + x + ")";
    }
    if (df_)
      return "df_cmul<" + b(lo_nz(t, qr)) + ", " + b(lo_nz(t, qi)) + ">(" + h(t, qr) + ", " + l(t, qr) +
             ", " + h(t, qi) + ", " + l(t, qi) + ", " + x + ")";
    return "f_cmul(" + h(t, qr) + ", " + h(t, qi) + ", " + x + ")";
  }

  void u2_pair(const TOp& t, const std::string& a, const std::string& c) {
    const double* m = t.m;
    switch (t.cls) {
      case U2_GENERAL:
        if (df_) {
          o_ << "      { const dfc y0 = df_row(" << h(t, 0) << ", " << l(t, 0) << ", " << h(t, 1) << ", " << l(t, 1) << ", "
             << h(t, 2) << ", " << l(t, 2) << ", " << h(t, 3) << ", " << l(t, 3) << ", " << a << ", " << c << ");\n";
          o_ << "        const dfc y1 = df_row(" << h(t, 4) << ", " << l(t, 4) << ", " << h(t, 5) << ", " << l(t, 5)
             << ", " << h(t, 6) << ", " << l(t, 6) << ", " << h(t, 7) << ", " << l(t, 7) << ", " << a << ", " << c
             << ");\n";
        } else {
          o_ << "      { const float2 y0 = f_row(" << h(t, 0) << ", " << h(t, 1) << ", " << h(t, 2) << ", " << h(t, 3)
             << ", " << a << ", " << c << ");\n";
          o_ << "        const float2 y1 = f_row(" << h(t, 4) << ", " << h(t, 5) << ", " << h(t, 6) << ", " << h(t, 7)
             << ", " << a << ", " << c << ");\n";
        }
        o_ << "        " << a << " = y0; " << c << " = y1; }\n";
        break;
      case U2_REAL:
        if (unit_diagonal(t)) {
          // [[1, b], [c, +-1]]
          const bool neg = m[6] < 0;
          if (df_)
            o_ << "      df_realunit<" << b(lo_nz(t, 2)) << ", " << b(lo_nz(t, 4)) << ", " << b(neg) << ">(" << h(t, 2)
               << ", " << l(t, 2) << ", " << h(t, 4) << ", " << l(t, 4) << ", " << a << ", " << c << ");\n";
          else
            o_ << "      f_realunit<" << b(neg) << ">(" << h(t, 2) << ", " << h(t, 4) << ", " << a << ", " << c << ");\n";
        } else if (m[0] == m[2] && m[0] == m[4] && m[6] == -m[0] && m[0] == 1.0 && !tab_) {  // [[1, 1], [1, -1]]
          o_ << "      " << (df_ ? "df_sumdiff(" : "f_sumdiff(") << a << ", " << c << ");\n";
        } else if (m[0] == m[2] && m[0] == m[4] && m[6] == -m[0]) {  // [[c, c], [c, -c]]
          if (df_)
            o_ << "      df_hadamard<" << b(lo_nz(t, 0)) << ">(" << h(t, 0) << ", " << l(t, 0) << ", " << a
               << ", " << c << ");\n";
          else
            o_ << "      f_hadamard(" << h(t, 0) << ", " << a << ", " << c << ");\n";
        } else if (df_) {
          o_ << "      df_real<" << b(lo_nz(t, 0)) << ", " << b(lo_nz(t, 2)) << ", "
             << b(lo_nz(t, 4)) << ", " << b(lo_nz(t, 6)) << ">(" << h(t, 0) << ", " << l(t, 0) << ", "
             << h(t, 2) << ", " << l(t, 2) << ", " << h(t, 4) << ", " << l(t, 4) << ", " << h(t, 6) << ", " << l(t, 6)
             << ", " << a << ", " << c << ");\n";
        } else {
          o_ << "      f_real(" << h(t, 0) << ", " << h(t, 2) << ", " << h(t, 4) << ", " << h(t, 6) << ", " << a << ", "
             << c << ");\n";
        }
        break;
      case U2_RXLIKE:  // m0 = (a, 0), m1 = (0, b), m2 = (0, c), m3 = (d, 0)
        if (unit_diagonal(t)) {  // [[1, i b], [i c, 1]]
          if (df_)
            o_ << "      df_rxunit<" << b(lo_nz(t, 3)) << ", " << b(lo_nz(t, 5)) << ">(" << h(t, 3) << ", " << l(t, 3)
               << ", " << h(t, 5) << ", " << l(t, 5) << ", " << a << ", " << c << ");\n";
          else
            o_ << "      f_rxunit(" << h(t, 3) << ", " << h(t, 5) << ", " << a << ", " << c << ");\n";
        } else if (df_)
          o_ << "      df_rxlike<" << b(lo_nz(t, 0)) << ", " << b(lo_nz(t, 3)) << ", "
             << b(lo_nz(t, 5)) << ", " << b(lo_nz(t, 6)) << ">(" << h(t, 0) << ", " << l(t, 0) << ", "
             << h(t, 3) << ", " << l(t, 3) << ", " << h(t, 5) << ", " << l(t, 5) << ", " << h(t, 6) << ", " << l(t, 6)
             << ", " << a << ", " << c << ");\n";
        else
          o_ << "      f_rxlike(" << h(t, 0) << ", " << h(t, 3) << ", " << h(t, 5) << ", " << h(t, 6) << ", " << a
             << ", " << c << ");\n";
        break;
      case U2_DIAG:
        o_ << "      " << a << " = " << cmul(t, 0, 1, a) << ";\n";
        o_ << "      " << c << " = " << cmul(t, 6, 7, c) << ";\n";
        break;
      case U2_ANTIDIAG:
        o_ << "      { const " << (df_ ? "dfc" : "float2") << " y0 = " << cmul(t, 2, 3, c) << ";\n";
        o_ << "        " << c << " = " << cmul(t, 4, 5, a) << "; " << a << " = y0; }\n";
        break;
      case U2_X:
        o_ << "      { const " << (df_ ? "dfc" : "float2") << " y = " << a << "; " << a << " = " << c << "; " << c
           << " = y; }\n";
        break;
      default: {  // U2_IMAG_ANTI: m1 = +-i, m2 = +-i
        const std::string f1 = std::string(pol()) + (m[3] > 0 ? "::mul_i" : "::mul_mi");
        const std::string f2 = std::string(pol()) + (m[5] > 0 ? "::mul_i" : "::mul_mi");
        o_ << "      { const " << (df_ ? "dfc" : "float2") << " y0 = " << f1 << "(" << c << ");\n";
        o_ << "        " << c << " = " << f2 << "(" << a << "); " << a << " = y0; }\n";
      } break;
    }
  }

  static std::string r(int j) { return "r" + std::to_string(j); }

  // A unit rotation ([[1, b], [c, 1]] real, or [[1, i b], [i c, 1]]) on register bit rp
  // while an X of that bit is pending in xm: threads with the X apply b and c exchanged.
  void u2_unit_conj(const TOp& t, int rp, const std::string& c) {
    const bool rx = t.cls == U2_RXLIKE;
    const int qb = rx ? 3 : 2, qc = rx ? 5 : 4;
    const bool same = !tab_ && t.mf[qb] == t.mf[qc] && (!df_ || t.mf[8 + qb] == t.mf[8 + qc]);
    const bool lb = lo_nz(t, qb) || lo_nz(t, qc);
    o_ << "    {  // U2 class " << t.cls << " on register bit " << rp << ", pending X" << (same ? " (symmetric)" : "")
       << "\n";
    std::string Bh = h(t, qb), Ch = h(t, qc), Bl = df_ ? l(t, qb) : "", Cl = df_ ? l(t, qc) : "";
    if (!same) {
      o_ << "      const bool sw = ((xm >> " << rp << ") & 1u) != 0u;\n";
      o_ << "      const float Bh = sw ? " << Ch << " : " << Bh << ", Ch = sw ? " << Bh << " : " << Ch << ";\n";
      if (df_) o_ << "      const float Bl = sw ? " << Cl << " : " << Bl << ", Cl = sw ? " << Bl << " : " << Cl << ";\n";
      Bh = "Bh";
      Ch = "Ch";
      Bl = "Bl";
      Cl = "Cl";
    }
    if (!c.empty()) o_ << "    if (" << c << ") {\n";
    std::vector<int> done;
    for (int q = 0; q < ns_ / 2; ++q) {
      const int j0 = ((q >> rp) << (rp + 1)) | (q & ((1 << rp) - 1));
      const int j1 = j0 | (1 << rp);
      if (df_) {
        if (rx)
          o_ << "      df_rxunit<" << b(lb) << ", " << b(lb) << ">(" << Bh << ", " << Bl << ", " << Ch << ", " << Cl
             << ", " << r(j0) << ", " << r(j1) << ");\n";
        else
          o_ << "      df_realunit<" << b(lb) << ", " << b(lb) << ", false>(" << Bh << ", " << Bl << ", " << Ch << ", "
             << Cl << ", " << r(j0) << ", " << r(j1) << ");\n";
      } else {
        if (rx) o_ << "      f_rxunit(" << Bh << ", " << Ch << ", " << r(j0) << ", " << r(j1) << ");\n";
        else o_ << "      f_realunit<false>(" << Bh << ", " << Ch << ", " << r(j0) << ", " << r(j1) << ");\n";
      }
      done.push_back(j0);
      done.push_back(j1);
    }
    if (!c.empty()) o_ << "    }\n";
    o_ << "    }\n";
    for (int j : done) touched(j);
  }

  void op(const TOp& t) {
    const uint32_t cr = t.rmask & (uint32_t)(ns_ - 1);
    switch (t.kind) {
      case OK_U2: {
        const int rp = t.t2;
        const std::string c = cond(t.gcmask, t.gcmask, t.tmask, t.tval);
        if (t.cls == U2_X && cr == 0 && !c.empty()) {  // a conditional X on every pair: into xm
          o_ << "    xm ^= (unsigned)(" << c << ") << " << rp << ";  // X on register bit " << rp << "\n";
          pend_ |= 1u << rp;
          break;
        }
        materialise(cr);
        // On a pending X of its own bit: a swap is the same on either order of its pair;
        // the unit rotations [[1, b], [c, 1]] and [[1, i b], [i c, 1]] become the same
        // form with b and c exchanged (X U X), chosen per thread from xm; other classes
        // apply the X first.
        const bool unit_rot = unit_diagonal(t) && (t.cls == U2_RXLIKE || (t.cls == U2_REAL && t.m[6] > 0));
        const bool conj = ((pend_ >> rp) & 1) && unit_rot;
        if (t.cls != U2_X && !conj) materialise(1u << rp);
        if (conj) {
          u2_unit_conj(t, rp, c);
          break;
        }
        o_ << "    {  // U2 class " << t.cls << " on register bit " << rp << "\n";
        if (!c.empty()) o_ << "    if (" << c << ") {\n";
        std::vector<int> done;
        for (int q = 0; q < ns_ / 2; ++q) {
          const int j0 = ((q >> rp) << (rp + 1)) | (q & ((1 << rp) - 1));
          const int j1 = j0 | (1 << rp);
          if ((j0 & cr) != cr) continue;
          u2_pair(t, r(j0), r(j1));
          if (t.cls != U2_X && t.cls != U2_IMAG_ANTI) {
            done.push_back(j0);
            done.push_back(j1);
          }
        }
        if (!c.empty()) o_ << "    }\n";
        o_ << "    }\n";
        for (int j : done) touched(j);
      } break;
      case OK_PHASE: {
        materialise(cr);
        const std::string c = cond(t.gmask, t.gmask, t.tmask, t.tval);
        o_ << "    {  // phase class " << t.cls << "\n";
        if (!c.empty()) o_ << "    if (" << c << ") {\n";
        for (int j = 0; j < ns_; ++j) {
          if ((j & cr) != cr) continue;
          std::string v;
          int ex = 0;
          const bool pow2 = !tab_ && t.cls == PH_GENERAL && t.m[1] == 0.0 && t.m[0] != 0.0 &&
                            std::frexp(std::fabs(t.m[0]), &ex) == 0.5;
          if (pow2) v = std::string(df_ ? "df_pow2(" : "f_pow2(") + flit((float)t.m[0]) + ", " + r(j) + ")";
          else if (t.cls == PH_GENERAL) v = cmul(t, 0, 1, r(j));
          else if (t.cls == PH_NEG) v = std::string(pol()) + "::neg(" + r(j) + ")";
          else if (t.cls == PH_I) v = std::string(pol()) + "::mul_i(" + r(j) + ")";
          else v = std::string(pol()) + "::mul_mi(" + r(j) + ")";
          o_ << "      " << r(j) << " = " << v << ";\n";
        }
        if (!c.empty()) o_ << "    }\n";
        o_ << "    }\n";
        if (t.cls == PH_GENERAL)
          for (int j = 0; j < ns_; ++j)
            if ((j & cr) == cr) touched(j);
      } break;
      case OK_SWAP: {
        const int A = t.dbits[0], B = t.dbits[1];
        materialise(cr | (1u << A) | (1u << B));
        const bool isw = (t.flags & 1) != 0;
        const std::string c = cond(t.gcmask, t.gcmask, t.tmask, t.tval);
        o_ << "    {  // swap of register bits " << A << ", " << B << (isw ? " (iSWAP)" : "") << "\n";
        if (!c.empty()) o_ << "    if (" << c << ") {\n";
        for (int j = 0; j < ns_; ++j) {
          if (!((j >> A) & 1) || ((j >> B) & 1) || (j & cr) != cr) continue;
          const int p = j ^ (1 << A) ^ (1 << B);
          const std::string T = df_ ? "dfc" : "float2";
          if (df_) since_[j] = since_[p] = std::max(since_[j], since_[p]);  // conditional: either may move
          if (isw)
            o_ << "      { const " << T << " y = " << r(j) << "; " << r(j) << " = " << pol() << "::mul_i(" << r(p)
               << "); " << r(p) << " = " << pol() << "::mul_i(y); }\n";
          else
            o_ << "      { const " << T << " y = " << r(j) << "; " << r(j) << " = " << r(p) << "; " << r(p)
               << " = y; }\n";
        }
        if (!c.empty()) o_ << "    }\n";
        o_ << "    }\n";
      } break;
      case OK_BLOCKADE: {
        materialise(cr);
        o_ << "    {  // blockade phase\n      const int cnt = __popcll(base & " << hex64(t.gmask) << ") + __popc(lt & "
           << hex32(t.tmask) << ");\n";
        for (int j = 0; j < ns_; ++j) {
          const int need = 1 - __builtin_popcount((unsigned)j & cr);
          if (need < 0) continue;
          o_ << "      if (cnt == " << need << ") " << r(j) << " = " << cmul(t, 0, 1, r(j)) << ";\n";
        }
        o_ << "    }\n";
        for (int j = 0; j < ns_; ++j)
          if (1 - __builtin_popcount((unsigned)j & cr) >= 0) touched(j);
      } break;
      case OK_PARITY: {
        materialise(cr);
        o_ << "    {  // parity phase\n      const bool par = ((__popcll(base & " << hex64(t.gmask) << ") + __popc(lt & "
           << hex32(t.tmask) << ")) & 1) != 0;\n";
        // even register parity takes (par ? p1 : p0), odd (par ? p0 : p1)
        const int nq = df_ ? 4 : 2;
        for (int side = 0; side < 2; ++side) {
          for (int q = 0; q < nq; ++q) {
            // DF: q = 0 re.h, 1 re.l, 2 im.h, 3 im.l ; F32: q = 0 re, 1 im
            auto lit = [&](int entry) {
              const int idx = 2 * entry + (df_ ? q / 2 : q);
              return df_ ? ((q & 1) ? l(t, idx) : h(t, idx)) : h(t, idx);
            };
            const std::string e0 = lit(0), e1 = lit(1);
            o_ << "      const float c" << side << "_" << q << " = par ? " << (side == 0 ? e1 : e0) << " : "
               << (side == 0 ? e0 : e1) << ";\n";
          }
        }
        for (int j = 0; j < ns_; ++j) {
          const int side = __builtin_popcount((unsigned)j & cr) & 1;
          const std::string s = "c" + std::to_string(side) + "_";
          if (df_)
            o_ << "      " << r(j) << " = df_cmul<true, true>(" << s << "0, " << s << "1, " << s << "2, " << s << "3, "
               << r(j) << ");\n";
          else
            o_ << "      " << r(j) << " = f_cmul(" << s << "0, " << s << "1, " << r(j) << ");\n";
        }
        o_ << "    }\n";
        for (int j = 0; j < ns_; ++j) touched(j);
      } break;
      case OK_COLLAPSE: {
        materialise(cr);
        const std::string c = cond(t.gmask, t.gval, t.tmask, t.tval);
        const uint32_t rv = t.rval & (uint32_t)(ns_ - 1);
        o_ << "    {  // collapse\n      const bool tc = " << (c.empty() ? "true" : c) << ";\n";
        for (int j = 0; j < ns_; ++j) {
          if ((j & cr) == rv) {
            const std::string sc = df_ ? "df_scale<" + b(lo_nz(t, 0)) + ">(" + h(t, 0) + ", " + l(t, 0) + ", " +
                                             r(j) + ")"
                                       : "f_scale(" + h(t, 0) + ", " + r(j) + ")";
            o_ << "      " << r(j) << " = tc ? " << sc << " : " << pol() << "::zero();\n";
          } else {
            o_ << "      " << r(j) << " = " << pol() << "::zero();\n";
          }
          touched(j);
        }
        o_ << "    }\n";
      } break;
      default: break;
    }
  }

  // A run of phase ops (diagonal, commuting with each other) multiplies each
  // register by the product of the phases whose conditions it meets. The run
  // collects those products per register-condition mask cr first (one complex
  // product per op, whatever the number of registers it touches); exact unit
  // phases (-1, +-i) without a runtime condition are only counted (a power of i
  // per mask). Register j then needs H[j] = product of the factors of every mask
  // contained in j: a subset-product transform builds all H[j] with at most
  // R 2^(R-1) products. The run is emitted this way when that costs fewer complex
  // products than applying each op to its registers.
  static constexpr int kPhaseRunMin = 3;
  bool unit_phase(const TOp& t) const { return t.cls != PH_GENERAL; }
  int unit_power(const TOp& t) const { return t.cls == PH_NEG ? 2 : t.cls == PH_I ? 1 : 3; }

  // complex products of the run form; *ok = false when it would not pay
  // exponent j (phase = w^j, w = exp(2 pi i / 2^30)) of an exact root phase op, or -1
  static long long root_exponent(const TOp& t) {
    if (t.cls == PH_I) return 1LL << 28;
    if (t.cls == PH_NEG) return 1LL << 29;
    if (t.cls == PH_MINUS_I) return 3LL << 28;
    const double two_pi = 6.283185307179586476925286766559;
    double phi = std::atan2(t.m[1], t.m[0]);
    if (phi < 0) phi += two_pi;
    const long long j = std::llround(phi / two_pi * 1073741824.0) & ((1LL << 30) - 1);
    const double a = two_pi * (double)j / 1073741824.0;
    if (std::fabs(std::cos(a) - t.m[0]) > 4e-16 || std::fabs(std::sin(a) - t.m[1]) > 4e-16) return -1;
    return j;
  }

  // A run whose phases are all powers of w: integer exponents per register mask,
  // added under their conditions, then one table product per register.
  // budget: complex products of the cheapest other form; the root form costs,
  // per register it touches, one product per table chunk plus the lookups
  // (about 0.2 of a product in double-float, 2 in complex64, where a product is
  // four instructions and a lookup a dependent load), and a fraction of a product
  // per conditional exponent add
  bool root_run(int begin, int end, double budget) {
    if (tab_) return false;
    std::vector<long long> ex(end - begin);
    unsigned long long any = 0;
    int conds = 0;
    for (int i = begin; i < end; ++i) {
      ex[i - begin] = root_exponent(ops_[i]);
      if (ex[i - begin] < 0) return false;
      any |= (unsigned long long)ex[i - begin];
      if (ops_[i].gmask || ops_[i].tmask) ++conds;
    }
    const bool A = (any >> 20) & 1023, B = (any >> 10) & 1023, C = any & 1023;
    const int chunks = (A ? 1 : 0) + (B ? 1 : 0) + (C ? 1 : 0);
    const double cost = ns_ * chunks * (1.0 + (df_ ? 0.2 : 2.0)) + conds * (df_ ? 0.1 : 0.5);
    if (cost >= budget) return false;
    bool used[kMaxRegs] = {false};
    unsigned long long konst[kMaxRegs] = {0};
    o_ << "    {  // run of " << (end - begin) << " phase ops, exponents of exp(2 pi i / 2^30)\n";
    for (int i = begin; i < end; ++i) {
      const TOp& t = ops_[i];
      const int cr = (int)(t.rmask & (uint32_t)(ns_ - 1));
      const std::string c = cond(t.gmask, t.gmask, t.tmask, t.tval);
      if (c.empty()) {
        konst[cr] += (unsigned long long)ex[i - begin];
        continue;
      }
      if (!used[cr]) {
        used[cr] = true;
        o_ << "      unsigned E" << cr << " = 0u;\n";
      }
      o_ << "      if (" << c << ") E" << cr << " += " << hex32((uint32_t)ex[i - begin]) << ";\n";
    }
    for (int j = 0; j < ns_; ++j) {
      std::string sum;
      unsigned long long k = 0;
      bool any_j = false;
      for (int cr = 0; cr < ns_; ++cr) {
        if ((j & cr) != cr) continue;
        k += konst[cr];
        if (konst[cr]) any_j = true;
        if (used[cr]) {
          sum += (sum.empty() ? "E" : " + E") + std::to_string(cr);
          any_j = true;
        }
      }
      if (!any_j) continue;
      k &= (1ULL << 30) - 1;
      if (sum.empty() && k == 0) continue;
      const std::string T = "((" + (sum.empty() ? std::string("0u") : sum) + " + " + hex32((uint32_t)k) + ") & 0x3fffffffu)";
      o_ << "      r" << j << " = " << (df_ ? "df_root_mul_impl<" : "f_root_mul_impl<") << b(A) << ", " << b(B) << ", "
         << b(C) << ">(" << T << ", r" << j << ");\n";
      touched(j);
    }
    o_ << "    }\n";
    return true;
  }

  void phase_run(int begin, int end) {
    const int R = sh_.rbits;
    {  // the run selects registers by its ops' register masks
      uint32_t m = 0;
      for (int i = begin; i < end; ++i) m |= ops_[i].rmask & (uint32_t)(ns_ - 1);
      materialise(m);
    }
    // cost of the op-by-op form: complex products
    int cost_ops = 0;
    for (int i = begin; i < end; ++i) {
      const TOp& t = ops_[i];
      if (unit_phase(t)) continue;
      const int cr = (int)(t.rmask & (uint32_t)(ns_ - 1));
      cost_ops += 1 << (R - __builtin_popcount((unsigned)cr));
    }
    // the run form: factor updates, subset products, applications
    bool gen[kMaxRegs] = {false};
    int unit[kMaxRegs] = {0};
    int cost_run = 0;
    for (int i = begin; i < end; ++i) {
      const TOp& t = ops_[i];
      const int cr = (int)(t.rmask & (uint32_t)(ns_ - 1));
      const bool runtime = t.gmask != 0 || t.tmask != 0;
      if (unit_phase(t) && !runtime) continue;
      if (gen[cr] && !unit_phase(t)) ++cost_run;
      gen[cr] = true;
    }
    bool def[kMaxRegs];
    for (int j = 0; j < ns_; ++j) def[j] = gen[j];
    for (int b = 0; b < R; ++b)
      for (int j = 0; j < ns_; ++j)
        if ((j >> b) & 1) {
          if (def[j] && def[j ^ (1 << b)]) ++cost_run;
          def[j] = def[j] || def[j ^ (1 << b)];
        }
    for (int j = 0; j < ns_; ++j) cost_run += def[j] ? 1 : 0;
    if (root_run(begin, end, std::min(cost_run, cost_ops))) return;
    if (cost_run >= cost_ops) {
      for (int i = begin; i < end; ++i) op(ops_[i]);
      return;
    }
    const std::string V = df_ ? "dfc" : "float2";
    auto mul = [&](const std::string& f, const std::string& g) {  // f * g, both variables
      return df_ ? "df_cmul<true, true>(" + f + ".rh, " + f + ".rl, " + f + ".ih, " + f + ".il, " + g + ")"
                 : "f_cmul(" + f + ".x, " + f + ".y, " + g + ")";
    };
    auto rot = [&](int pw, const std::string& x) {  // x * i^pw
      pw &= 3;
      if (pw == 0) return x;
      return std::string(pol()) + (pw == 1 ? "::mul_i(" : pw == 2 ? "::neg(" : "::mul_mi(") + x + ")";
    };
    bool made[kMaxRegs] = {false};
    int prods[kMaxRegs] = {0};
    o_ << "    {  // run of " << (end - begin) << " phase ops\n";
    const std::string one = df_ ? "dfc{1.0f, 0.0f, 0.0f, 0.0f}" : "make_float2(1.0f, 0.0f)";
    for (int i = begin; i < end; ++i) {
      const TOp& t = ops_[i];
      const int cr = (int)(t.rmask & (uint32_t)(ns_ - 1));
      const std::string c = cond(t.gmask, t.gmask, t.tmask, t.tval);
      if (unit_phase(t) && c.empty()) {
        unit[cr] += unit_power(t);
        continue;
      }
      const std::string F = "F" + std::to_string(cr);
      std::string lit;  // the phase as a value of the register type
      if (t.cls == PH_GENERAL)
        lit = df_ ? "dfc{" + h(t, 0) + ", " + l(t, 0) + ", " + h(t, 1) + ", " + l(t, 1) + "}"
                  : "make_float2(" + h(t, 0) + ", " + h(t, 1) + ")";
      else
        lit = rot(unit_power(t), one);
      if (!made[cr]) {
        made[cr] = true;
        o_ << "      " << V << " " << F << " = " << (c.empty() ? lit : "(" + c + ") ? " + lit + " : " + one) << ";\n";
        continue;
      }
      const std::string upd = t.cls == PH_GENERAL ? cmul(t, 0, 1, F) : rot(unit_power(t), F);
      o_ << "      " << (c.empty() ? "" : "if (" + c + ") ") << F << " = " << upd << ";\n";
      if (df_ && t.cls == PH_GENERAL && ++prods[cr] >= kRenormEvery) {
        o_ << "      " << F << " = DF::renorm(" << F << ");\n";
        prods[cr] = 0;
      }
    }
    // subset products H[j] = prod over masks cr contained in j of F[cr]
    for (int j = 0; j < ns_; ++j)
      if (made[j]) o_ << "      " << V << " H" << j << " = F" << j << ";\n";
    bool have[kMaxRegs];
    for (int j = 0; j < ns_; ++j) have[j] = made[j];
    for (int b = 0; b < R; ++b)
      for (int j = ns_ - 1; j >= 0; --j)
        if (((j >> b) & 1) && have[j ^ (1 << b)]) {
          const std::string lo = "H" + std::to_string(j ^ (1 << b));
          if (have[j]) o_ << "      H" << j << " = " << mul(lo, "H" + std::to_string(j)) << ";\n";
          else o_ << "      " << V << " H" << j << " = " << lo << ";\n";
          have[j] = true;
        }
    for (int j = 0; j < ns_; ++j) {
      int pw = 0;
      for (int cr = 0; cr < ns_; ++cr)
        if ((j & cr) == cr) pw += unit[cr];
      if (!have[j] && (pw & 3) == 0) continue;
      std::string v = "r" + std::to_string(j);
      if (have[j]) v = mul("H" + std::to_string(j), v);
      o_ << "      r" << j << " = " << rot(pw, v) << ";\n";
      if (have[j]) touched(j);
    }
    o_ << "    }\n";
  }

  // A run of E parity ops with one phase pair (p0 on even, p1 on odd parity):
  // register j counts the ops that see odd parity, m_j, and is multiplied by
  // p0^(E-m_j) p1^m_j from a table. With literal masks the register parities are
  // resolved at generation time; with a coefficient table (sweep groups) the
  // masks come from the op's row (tile bits in floats 12-13, thread bits in 14, and in
  // 15 the register-parity mask: bit j = parity of register j's bits under the op's
  // register mask, as raw bits) and the table's entries from the run's rows (entry
  // m < E in floats 0-3 of row first + m, entry E in floats 4-7 of row first). There
  // the counts are kept bit-sliced: per op, the set of registers that see odd parity is
  // one XOR of that mask, added into bit planes c_p (bit j of c_p: bit p of m_j) with
  // two logic operations per plane, and each m_j is read out of the planes once.
  std::ostringstream pre_;  // namespace-scope declarations (literal phase tables)
  int ntables_ = 0;
  void parity_run(int begin, int end) {
    const int E = end - begin;
    {  // register parities: the ops' register masks (from the table: any register bit)
      uint32_t m = tab_ ? (uint32_t)(ns_ - 1) : 0u;
      for (int i = begin; i < end; ++i) m |= ops_[i].rmask & (uint32_t)(ns_ - 1);
      materialise(m);
    }
    o_ << "    {  // parity run of " << E << " ops\n";
    if (tab_) {
      int planes = 0;
      while ((1 << planes) <= E) ++planes;  // counts 0..E
      // op e's word (bit j: its parity for register j) into a carry-save counter (csa.h)
      const CsaPlan plan = csa_plan(E, planes);
      for (const CsaOp& c : plan.ops) {
        if (c.kind == CsaOp::IN) {
          const int row = 16 * ops_[begin + c.a].pad1;
          o_ << "      unsigned k" << c.s << ";\n";
          o_ << "      { const qgp::u64 G = (qgp::u64)__float_as_uint(cs[" << row + 12
             << "]) | ((qgp::u64)__float_as_uint(cs[" << row + 13 << "]) << 32);\n";
          o_ << "        const unsigned T = __float_as_uint(cs[" << row + 14 << "]), P = __float_as_uint(cs["
             << row + 15 << "]);\n";
          o_ << "        k" << c.s << " = P ^ (0u - (unsigned)((__popcll(base & G) + __popc(lt & T)) & 1)); }\n";
        } else if (c.kind == CsaOp::FULL) {
          o_ << "      const unsigned k" << c.s << " = k" << c.a << " ^ k" << c.b << " ^ k" << c.c << ";\n";
          if (c.cy >= 0)
            o_ << "      const unsigned k" << c.cy << " = (k" << c.a << " & k" << c.b << ") | (k" << c.c << " & (k"
               << c.a << " ^ k" << c.b << "));\n";
        } else {
          o_ << "      const unsigned k" << c.s << " = k" << c.a << " ^ k" << c.b << ";\n";
          if (c.cy >= 0) o_ << "      const unsigned k" << c.cy << " = k" << c.a << " & k" << c.b << ";\n";
        }
      }
      for (int p = 0; p < planes; ++p)
        o_ << "      const unsigned c" << p << " = "
           << (plan.planes[p] >= 0 ? "k" + std::to_string(plan.planes[p]) : std::string("0u")) << ";\n";
      if (planes <= 8) {
        // counts as bytes: nibble k of plane p spread to bit p of four bytes with one
        // multiply (bit i times 2^(7i + p) lands on bit 8i + p; the four terms never
        // overlap), then each register's byte taken out
        const int words = ns_ / 4;
        for (int k = 0; k < words; ++k) {
          o_ << "      const unsigned b" << k << " = ";
          for (int p = 0; p < planes; ++p)
            o_ << (p ? "\n        | " : "") << "((((c" << p << " >> " << 4 * k << ") & 0xFu) * " << hex32(0x00204081u << p)
               << ") & " << hex32(0x01010101u << p) << ")";
          o_ << ";\n";
        }
        for (int j = 0; j < ns_; ++j)
          o_ << "      const int m" << j << " = (int)__byte_perm(b" << j / 4 << ", 0u, " << hex32(0x4440u | (unsigned)(j % 4))
             << ");\n";
      } else {
        for (int j = 0; j < ns_; ++j) {
          o_ << "      const int m" << j << " = (int)(";
          for (int p = 0; p < planes; ++p)
            o_ << (p ? " | " : "") << "(((c" << p << " >> " << j << ") & 1u) << " << p << ")";
          o_ << ");\n";
        }
      }
    } else {
      o_ << "      int";
      for (int j = 0; j < ns_; ++j) o_ << (j ? ", m" : " m") << j << " = 0";
      o_ << ";\n";
    }
    for (int e = begin; e < end && !tab_; ++e) {
      const TOp& t = ops_[e];
      std::string oe;
      if (t.gmask) oe += "__popcll(base & " + hex64(t.gmask) + ")";
      if (t.tmask) oe += std::string(oe.empty() ? "" : " + ") + "__popc(lt & " + hex32(t.tmask) + ")";
      const uint32_t R = t.rmask & (uint32_t)(ns_ - 1);
      if (oe.empty()) {
        for (int j = 0; j < ns_; ++j)
          if (__builtin_popcount((unsigned)j & R) & 1) o_ << "      m" << j << " += 1;\n";
        continue;
      }
      o_ << "      { const int o = (" << oe << ") & 1;\n";
      for (int j = 0; j < ns_; ++j)
        o_ << "        m" << j << " += " << ((__builtin_popcount((unsigned)j & R) & 1) ? "1 - o" : "o") << ";\n";
      o_ << "      }\n";
    }
    std::string tab;
    if (!tab_) {
      tab = "PT" + std::to_string(ntables_++);
      const auto ent = parity_table(ops_[begin], E);
      pre_ << "static __device__ const " << (df_ ? "float4 " : "float2 ") << tab << "[" << (E + 1) << "] = {";
      for (int m = 0; m <= E; ++m) {
        const double re = ent[m].real(), im = ent[m].imag();
        const float rh = (float)re, ih = (float)im;
        if (df_)
          pre_ << (m ? ", " : "") << "{" << flit(rh) << ", " << flit((float)(re - (double)rh)) << ", " << flit(ih)
               << ", " << flit((float)(im - (double)ih)) << "}";
        else
          pre_ << (m ? ", " : "") << "{" << flit(rh) << ", " << flit(ih) << "}";
      }
      pre_ << "};\n";
    }
    const int first = 16 * ops_[begin].pad1;
    for (int j = 0; j < ns_; ++j) {
      if (tab_) {
        o_ << "      { const int a = (m" << j << " < " << E << ") ? " << first << " + 16 * m" << j << " : " << first + 4
           << ";\n";
        if (df_) o_ << "        r" << j << " = df_cmul<true, true>(cs[a], cs[a + 1], cs[a + 2], cs[a + 3], r" << j << "); }\n";
        else o_ << "        r" << j << " = f_cmul(cs[a], cs[a + 1], r" << j << "); }\n";
      } else {
        if (df_)
          o_ << "      { const float4 v = " << tab << "[m" << j << "]; r" << j << " = df_cmul<true, true>(v.x, v.y, v.z, v.w, r"
             << j << "); }\n";
        else
          o_ << "      { const float2 v = " << tab << "[m" << j << "]; r" << j << " = f_cmul(v.x, v.y, r" << j << "); }\n";
      }
      touched(j);
    }
    o_ << "    }\n";
  }

  void body() {
    const std::string V = df_ ? "dfc" : "float2";
    const int E = df_ ? 16 : 8;
    o_ << "    " << V;
    for (int j = 0; j < ns_; ++j) o_ << (j ? ", r" : " r") << j;
    o_ << ";\n    int";
    for (int j = 0; j < ns_; ++j) o_ << (j ? ", q" : " q") << j;
    o_ << ";\n    unsigned lt = 0, xm = 0u;\n";
    o_ << "    (void)lt; (void)xm;\n";
    pend_ = 0;
    bool in_regs = false, raw = true;
    for (int i = 0; i < nops_; ++i) {
      const TOp& t = ops_[i];
      if (t.kind == OK_LAYOUT) {
        if (in_regs) {
          renorm_for_store();
          store_regs(std::string(pol()) + "::st_work");
          o_ << "    __syncthreads();\n";
          raw = false;
        }
        for (int q = 0; q < sh_.rbits; ++q) rpos_[q] = t.dbits[q];
        // thread bits: zeros inserted at the register positions (ascending)
        o_ << "    lt = tid;\n";
        for (int q = 0; q < sh_.rbits; ++q) {
          const int b = t.dbits[q];
          o_ << "    lt = ((lt >> " << b << ") << " << (b + 1) << ") | (lt & " << hex32((1u << b) - 1) << ");\n";
        }
        for (int j = 0; j < ns_; ++j) {
          uint32_t lj = 0;
          for (int q = 0; q < sh_.rbits; ++q)
            if ((j >> q) & 1) lj |= 1u << t.dbits[q];
          o_ << "    q" << j << " = swz<" << E << ">((int)(lt | " << hex32(lj) << "));\n";
        }
        const std::string ld = raw ? ld_raw() : std::string(pol()) + "::ld_work";
        if (paired()) {  // complex64: raw and working forms are the same
          for (int j = 0; j < ns_; j += 2)
            o_ << "    F32::ld_pair(buf, q" << j << ", r" << j << ", r" << j + 1 << ");\n";
        } else {
          for (int j = 0; j < ns_; ++j) o_ << "    r" << j << " = " << ld << "(buf, q" << j << ");\n";
        }
        for (int j = 0; j < ns_; ++j) since_[j] = carry_;
        in_regs = true;
        continue;
      }
      if (t.kind == OK_PARITY) {
        const int j = parity_run_end(ops_, nops_, i);
        if (tab_ || j - i >= 2) {
          parity_run(i, j);
          i = j - 1;
          continue;
        }
      }
      if (t.kind == OK_PHASE) {
        int j = i;
        while (j < nops_ && ops_[j].kind == OK_PHASE) ++j;
        if (j - i >= kPhaseRunMin) {
          phase_run(i, j);
          i = j - 1;
          continue;
        }
      }
      op(t);
    }
    if (in_regs) {
      if (io_ & kTileOutPairs) renorm_for_store();  // st_doubles normalises on its own
      store_regs(st_raw());
    } else if (df_ && ((io_ & kTileInPairs) != 0) != ((io_ & kTileOutPairs) != 0)) {
      // no op loaded the tile: convert its storage form in place, each thread its own slots
      o_ << "    for (int l = (int)tid; l < (1 << K_BITS); l += (1 << K_BITS) >> R_BITS) {\n"
         << "      const int q = swz<16>(l);\n      " << st_raw() << "(buf, q, " << ld_raw() << "(buf, q));\n    }\n";
    }
    o_ << "    __syncthreads();\n";
  }
};

// ---------------------------------------------------------------------------
// Compilation and the per-device cache
// ---------------------------------------------------------------------------
struct Unit {
  std::string src;
  std::vector<int> steps;  // program steps of the kernels in this unit (kernel qgp_<step>)
  std::vector<char> cubin;
  std::string err;
};

void compile_unit(Unit* u) {
  const NvrtcApi& api = nvrtc_api();
  nvrtcProgram p = nullptr;
  const char* hdr_src[2] = {kEmbedPassPrelude, kEmbedDf64};
  const char* hdr_names[2] = {"pass_prelude.cuh", "df64.cuh"};
  if (api.create(&p, u->src.c_str(), "passes.cu", 2, hdr_src, hdr_names) != NVRTC_SUCCESS) {
    u->err = "nvrtcCreateProgram failed";
    return;
  }
  const char* opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "--fmad=false", "-default-device"};
  const nvrtcResult rc = api.compile(p, 4, opts);
  if (rc != NVRTC_SUCCESS) {
    size_t n = 0;
    api.log_size(p, &n);
    std::string log(n, '\0');
    if (n) api.log(p, &log[0]);
    u->err = "pass kernel compile failed: " + log.substr(0, 2000);
    api.destroy(&p);
    return;
  }
  size_t n = 0;
  api.cubin_size(p, &n);
  u->cubin.resize(n);
  api.cubin(p, u->cubin.data());
  api.destroy(&p);
}

// w^(a 2^20), w^(b 2^10), w^c (w = exp(2 pi i / 2^30)) as double-float entries,
// copied into a loaded module's qgp_roots table.
cudaError_t fill_root_table(cudaLibrary_t lib) {
  static const std::vector<float> host = [] {
    std::vector<float> t(3072 * 4);
    const double two_pi = 6.283185307179586476925286766559;
    for (int part = 0; part < 3; ++part)
      for (int i = 0; i < 1024; ++i) {
        const double j = (double)i * (part == 0 ? 1048576.0 : part == 1 ? 1024.0 : 1.0);
        const double a = two_pi * j / 1073741824.0, re = std::cos(a), im = std::sin(a);
        float* e = &t[4 * (1024 * part + i)];
        e[0] = (float)re;
        e[1] = (float)(re - (double)e[0]);
        e[2] = (float)im;
        e[3] = (float)(im - (double)e[2]);
      }
    return t;
  }();
  void* d = nullptr;
  size_t bytes = 0;
  cudaError_t e = cudaLibraryGetGlobal(&d, &bytes, lib, "qgp_roots");
  if (e != cudaSuccess) return e;
  if (bytes != sizeof(float) * host.size()) return cudaErrorInvalidValue;
  return cudaMemcpy(d, host.data(), bytes, cudaMemcpyHostToDevice);
}

struct Compiled : PassKernels {
  Shape sh{0, 0, 0};                 // the kernels' launch shape
  std::vector<cudaLibrary_t> libs;
  std::vector<cudaKernel_t> kernel;  // per program step (nullptr: interpreted)
  std::vector<int> smem;             // dynamic shared memory per step
  double compile_ms = 0;
  ~Compiled() {
    for (cudaLibrary_t l : libs) cudaLibraryUnload(l);
  }
};

// Compiled programs per device, least recently used first out beyond
// kMaxCachedPrograms (a serving process meets ever new circuits). An evicted
// program's modules unload when its last user lets go: a run holds its program
// until its passes have finished, a sweep for its lifetime.
constexpr size_t kMaxCachedPrograms = 64;
struct CacheEntry {
  std::shared_ptr<Compiled> prog;  // nullptr: the compile failed
  std::list<std::string>::iterator pos;
};
struct DeviceCache {
  std::unordered_map<std::string, CacheEntry> map;
  std::list<std::string> lru;  // most recent first
  std::shared_ptr<Compiled>* find(const std::string& key) {
    auto it = map.find(key);
    if (it == map.end()) return nullptr;
    lru.splice(lru.begin(), lru, it->second.pos);
    return &it->second.prog;
  }
  std::shared_ptr<Compiled> insert(const std::string& key, std::shared_ptr<Compiled> p) {
    auto it = map.find(key);
    if (it != map.end()) {  // another thread compiled it meanwhile
      if (!it->second.prog) it->second.prog = p;
      return it->second.prog;
    }
    lru.push_front(key);
    map.emplace(key, CacheEntry{p, lru.begin()});
    while (map.size() > kMaxCachedPrograms) {
      map.erase(lru.back());
      lru.pop_back();
    }
    return p;
  }
};
std::mutex g_mu;
DeviceCache g_cache[64];
size_t g_cache_hits = 0, g_cache_misses = 0;

}  // namespace

const char* pass_kernels_unavailable() {
  const NvrtcApi& api = nvrtc_api();
  return api.error.empty() ? nullptr : api.error.c_str();
}

namespace {

// Generate the program's supported passes and group them into translation units.
bool generate_units(const Program& prog, int prec, std::vector<Unit>* units, std::string* key, std::string* why,
                    bool table = false) {
  if (prec == QG_C128 && prog.arith != QG_ARITH_DOUBLE_FLOAT) {
    *why = "complex128 exact arithmetic runs interpreted";
    return false;
  }
  std::vector<std::pair<int, std::string>> pieces;
  size_t total = 0;
  for (size_t i = 0; i < prog.steps.size(); ++i) {
    const Step& st = prog.steps[i];
    const Shape sh = shape_of(prog, prec);
    // a tile of at least 2^10 amplitudes, a warp or more of threads
    if (st.kind != Step::TILE_PASS || st.pass.k < 10 || st.pass.k - sh.rbits < 5) continue;
    const TOp* ops = prog.tops.data() + st.pass.op_begin;
    const int nops = (int)(st.pass.op_end - st.pass.op_begin);
    std::ostringstream o;
    PassGen g(o, st.pass, ops, nops, prec, tile_pass_io(prog, i), table, sh);
    if (!g.supported()) continue;
    g.emit((int)i);
    pieces.emplace_back((int)i, o.str());
    total += pieces.back().second.size();
  }
  if (pieces.empty()) {
    *why = "no pass to specialise";
    return false;
  }
  *key = std::to_string(prec) + ":";
  key->reserve(total + 64);
  for (auto& p : pieces) *key += p.second;
  // one unit per host thread; passes dealt largest first to the smallest unit (the
  // compile time of a pass grows faster than its source, so big passes go alone)
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nunits = std::min<size_t>(pieces.size(), std::min(hw, 32u));
  units->assign(nunits, Unit());
  std::vector<size_t> load(nunits, 0), order(pieces.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::sort(order.begin(), order.end(),
            [&](size_t a, size_t b) { return pieces[a].second.size() > pieces[b].second.size(); });
  for (size_t u = 0; u < nunits; ++u) (*units)[u].src = "#include \"pass_prelude.cuh\"\n\n";
  for (size_t i : order) {
    const size_t u = std::min_element(load.begin(), load.end()) - load.begin();
    (*units)[u].src += pieces[i].second;
    (*units)[u].steps.push_back(pieces[i].first);
    load[u] += pieces[i].second.size() * (1 + pieces[i].second.size() / 16384);
  }
  return true;
}

// Compile every unit (in parallel threads); false with the first error.
bool compile_units(std::vector<Unit>& units, std::string* why) {
  if (const char* e = pass_kernels_unavailable()) {
    *why = e;
    return false;
  }
  std::vector<std::thread> th;
  for (size_t u = 1; u < units.size(); ++u) th.emplace_back(compile_unit, &units[u]);
  compile_unit(&units[0]);
  for (auto& t : th) t.join();
  for (Unit& u : units)
    if (!u.err.empty()) {
      *why = u.err;
      return false;
    }
  return true;
}

}  // namespace

int pass_kernels_build_only(const Program& prog, int prec, int* kernels, double* compile_ms, std::string* why,
                            bool table) {
  std::vector<Unit> units;
  std::string key;
  *kernels = 0;
  *compile_ms = 0;
  if (!generate_units(prog, prec, &units, &key, why, table)) return 0;
  const auto t0 = std::chrono::steady_clock::now();
  if (!compile_units(units, why)) return -1;
  *compile_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  for (Unit& u : units) *kernels += (int)u.steps.size();
  return 1;
}

std::string pass_kernels_source(const Program& prog, int prec) {
  std::vector<Unit> units;
  std::string key, why;
  if (!generate_units(prog, prec, &units, &key, &why)) return std::string();
  std::string s;
  for (Unit& u : units) s += u.src;
  return s;
}

std::string pass_structure_key(const Program& prog, bool table) {
  // the program's passes as bytes (descriptors, hand-over form, op records), which
  // determine the generated source; with a coefficient table the entries' values
  // are left out and only the value-dependent code choices are kept (the
  // Hadamard shape of a real 2x2, the signs of an imaginary antidiagonal)
  std::string key = std::to_string(prog.arith) + (table ? ":table:" : ":lit:");
  for (size_t i = 0; i < prog.steps.size(); ++i) {
    const Step& st = prog.steps[i];
    key += (char)st.kind;
    if (st.kind != Step::TILE_PASS) continue;
    const int io = tile_pass_io(prog, i);
    key.append(reinterpret_cast<const char*>(&io), sizeof(io));
    key.append(reinterpret_cast<const char*>(&st.pass), sizeof(PassDesc));
    const TOp* prev = nullptr;
    for (int64_t o = st.pass.op_begin; o < st.pass.op_end; ++o) {
      TOp t = prog.tops[o];
      if (table) {
        // the generator re-plans layouts, so the interpreter's layout records and
        // layout-relative fields do not matter; parity masks are data
        if (t.kind == OK_LAYOUT) continue;
        const double* m = t.m;
        const char shape[5] = {(char)(t.cls == U2_REAL && m[0] == m[2] && m[0] == m[4] && m[6] == -m[0]),
                               (char)(m[3] > 0), (char)(m[5] > 0),
                               (char)(prev && same_parity_phases(*prev, prog.tops[o])),
                               (char)(unit_diagonal(t))};
        prev = &prog.tops[o];
        std::memset(t.m, 0, sizeof(t.m));
        std::memset(t.mf, 0, sizeof(t.mf));
        t.t2 = t.kind == OK_U2 ? 0 : t.t2;
        t.rmask = t.rval = t.tmask = t.tval = 0;
        std::memset(t.dbits, 0, sizeof(t.dbits));
        std::memset(t.lj, 0, sizeof(t.lj));
        if (t.kind == OK_PARITY) t.lmask = t.lval = 0, t.gmask = t.gval = 0;
        key.append(shape, 5);
      }
      key.append(reinterpret_cast<const char*>(&t), sizeof(TOp));
    }
  }
  return key;
}

std::shared_ptr<const PassKernels> pass_kernels_for(const Program& prog, int prec, int device, std::string* why,
                                                    bool table) {
  NvtxRange nvtx("qg pass kernels");
  if (device < 0 || device >= 64) {
    *why = "device ordinal out of range";
    return nullptr;
  }
  // generating the source for every run of a cached program would cost more than a lookup
  const Shape shape = shape_of(prog, prec);
  const std::string key = std::to_string(prec) + ":" + std::to_string(shape.rbits) + "/" +
                          std::to_string(shape.bufs) + "/" + std::to_string(shape.ctas) + ":" +
                          pass_structure_key(prog, table);
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (std::shared_ptr<Compiled>* hit = g_cache[device].find(key)) {
      ++g_cache_hits;
      if (!*hit) *why = "this program's pass kernels failed to compile before";
      return *hit;
    }
  }
  auto remember_failure = [&]() {
    std::lock_guard<std::mutex> lk(g_mu);
    g_cache[device].insert(key, nullptr);
    return nullptr;
  };
  std::vector<Unit> units;
  std::string src_key;
  if (!generate_units(prog, prec, &units, &src_key, why, table)) return nullptr;
  const auto t0 = std::chrono::steady_clock::now();
  if (!compile_units(units, why)) return remember_failure();
  auto c = std::make_shared<Compiled>();
  c->sh = shape;
  c->kernel.assign(prog.steps.size(), nullptr);
  c->smem.assign(prog.steps.size(), 0);
  const int E = prec == QG_C128 ? 16 : 8;
  for (Unit& u : units) {
    cudaLibrary_t lib = nullptr;
    cudaError_t e = cudaLibraryLoadData(&lib, u.cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) {
      *why = std::string("loading pass kernels: ") + cudaGetErrorString(e);
      return nullptr;
    }
    c->libs.push_back(lib);
    e = fill_root_table(lib);
    if (e != cudaSuccess) {
      *why = std::string("pass kernel tables: ") + cudaGetErrorString(e);
      return nullptr;
    }
    for (int s : u.steps) {
      cudaKernel_t k = nullptr;
      const std::string name = (table ? "qgs_" : "qgp_") + std::to_string(s);
      e = cudaLibraryGetKernel(&k, lib, name.c_str());
      if (e != cudaSuccess) {
        *why = "pass kernel " + name + " missing";
        return nullptr;
      }
      const Shape sh = shape;
      const PassDesc& pd = prog.steps[s].pass;
      const int smem = sh.bufs * (1 << pd.k) * E + (table ? 16 * 4 * (int)(pd.op_end - pd.op_begin) : 0);
      e = cudaKernelSetAttributeForDevice(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem, device);
      if (e != cudaSuccess) {
        *why = std::string("pass kernel attribute: ") + cudaGetErrorString(e);
        return nullptr;
      }
      c->kernel[s] = k;
      c->smem[s] = smem;
    }
  }
  c->compile_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  std::lock_guard<std::mutex> lk(g_mu);
  ++g_cache_misses;
  return g_cache[device].insert(key, c);
}

// ---------------------------------------------------------------------------
// Sweep level kernels: for a sweep of several sizes, level l runs the l-th pass of
// every group (qubit count) that has one, in one launch over all the groups' items
// (qgl_<l>, a GroupLevel descriptor per group). The bodies are the table-form pass
// bodies of each group; groups must share the tile size and the kernel shape.
// ---------------------------------------------------------------------------
struct LevelKernels : PassKernels {
  Shape sh{0, 0, 0};
  int threads = 0;                            // threads per CTA (tile / registers per thread)
  std::vector<cudaLibrary_t> libs;
  std::vector<cudaKernel_t> kernel;           // per level
  std::vector<int> smem;                      // per level
  std::vector<std::vector<int>> groups;       // per level: the groups it runs, in descriptor order
  double compile_ms = 0;
  ~LevelKernels() {
    for (cudaLibrary_t l : libs) cudaLibraryUnload(l);
  }
};

std::shared_ptr<const PassKernels> level_kernels_for(const std::vector<const Program*>& progs,
                                                     const std::vector<std::vector<int>>& pass_steps, int prec,
                                                     int device, std::string* why) {
  NvtxRange nvtx("qg level kernels");
  if (progs.empty() || progs.size() != pass_steps.size()) {
    *why = "no groups";
    return nullptr;
  }
  const Shape sh = shape_of(*progs[0], prec);
  const int E = prec == QG_C128 ? 16 : 8;
  int K = -1;
  size_t levels = 0;
  for (size_t g = 0; g < progs.size(); ++g) {
    if (prec == QG_C128 && progs[g]->arith != QG_ARITH_DOUBLE_FLOAT) {
      *why = "complex128 exact arithmetic runs interpreted";
      return nullptr;
    }
    for (int st : pass_steps[g]) {
      const int k = progs[g]->steps[st].pass.k;
      if (K < 0) K = k;
      if (k != K) {
        *why = "groups with different tile sizes";
        return nullptr;
      }
    }
    levels = std::max(levels, pass_steps[g].size());
  }
  if (K < 10 || K - sh.rbits < 5 || levels == 0) {
    *why = "no pass to specialise";
    return nullptr;
  }
  auto lk = std::make_shared<LevelKernels>();
  lk->sh = sh;
  lk->threads = (1 << K) >> sh.rbits;
  lk->groups.resize(levels);
  lk->smem.assign(levels, 0);
  // generate: one piece per level holding its groups' bodies and the level kernel
  std::vector<std::pair<int, std::string>> pieces;
  for (size_t l = 0; l < levels; ++l) {
    std::ostringstream o;
    std::vector<std::string> names;
    for (size_t g = 0; g < progs.size(); ++g) {
      if (l >= pass_steps[g].size()) continue;
      const Program& pr = *progs[g];
      const int st = pass_steps[g][l];
      const PassDesc& pd = pr.steps[st].pass;
      const TOp* ops = pr.tops.data() + pd.op_begin;
      const int nops = (int)(pd.op_end - pd.op_begin);
      const std::string ns = "g" + std::to_string(g) + "l" + std::to_string(l);
      PassGen gen(o, pd, ops, nops, prec, tile_pass_io(pr, (size_t)st), true, sh);
      if (!gen.supported()) {
        *why = "a sweep pass the generator does not specialise";
        return nullptr;
      }
      gen.emit(st, ns, false);
      names.push_back(ns);
      lk->groups[l].push_back((int)g);
      lk->smem[l] = std::max(lk->smem[l], sh.bufs * (1 << K) * E + 16 * 4 * nops);
    }
    o << "extern \"C\" __global__ void __launch_bounds__(" << ((1 << K) >> sh.rbits) << ", " << sh.ctas << ") qgl_"
      << l << "(const qgp::GroupLevel* __restrict__ gl, unsigned long long total) {\n  (void)total;\n";
    for (size_t q = 0; q < names.size(); ++q)
      o << "  qgp::run_group_share<" << names[q] << "::P>(gl[" << q << "]);\n";
    o << "}\n\n";
    pieces.emplace_back((int)l, o.str());
  }
  // units: levels dealt largest first, one unit per host thread
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nunits = std::min<size_t>(pieces.size(), std::min(hw, 32u));
  std::vector<Unit> units(nunits);
  std::vector<size_t> load(nunits, 0), order(pieces.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::sort(order.begin(), order.end(),
            [&](size_t a, size_t b) { return pieces[a].second.size() > pieces[b].second.size(); });
  for (Unit& u : units) u.src = "#include \"pass_prelude.cuh\"\n\n";
  for (size_t i : order) {
    const size_t u = std::min_element(load.begin(), load.end()) - load.begin();
    units[u].src += pieces[i].second;
    units[u].steps.push_back(pieces[i].first);
    load[u] += pieces[i].second.size() * (1 + pieces[i].second.size() / 16384);
  }
  const auto t0 = std::chrono::steady_clock::now();
  if (!compile_units(units, why)) return nullptr;
  lk->kernel.assign(levels, nullptr);
  for (Unit& u : units) {
    cudaLibrary_t lib = nullptr;
    cudaError_t e = cudaLibraryLoadData(&lib, u.cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) {
      *why = std::string("loading level kernels: ") + cudaGetErrorString(e);
      return nullptr;
    }
    lk->libs.push_back(lib);
    e = fill_root_table(lib);
    if (e != cudaSuccess) {
      *why = std::string("level kernel tables: ") + cudaGetErrorString(e);
      return nullptr;
    }
    for (int l : u.steps) {
      cudaKernel_t k = nullptr;
      const std::string name = "qgl_" + std::to_string(l);
      e = cudaLibraryGetKernel(&k, lib, name.c_str());
      if (e == cudaSuccess)
        e = cudaKernelSetAttributeForDevice(k, cudaFuncAttributeMaxDynamicSharedMemorySize, lk->smem[l], device);
      if (e != cudaSuccess) {
        *why = "level kernel " + name + ": " + cudaGetErrorString(e);
        return nullptr;
      }
      lk->kernel[l] = k;
    }
  }
  lk->compile_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return lk;
}

int level_count(const PassKernels& lk) { return (int)static_cast<const LevelKernels&>(lk).kernel.size(); }
const std::vector<int>& level_groups(const PassKernels& lk, int level) {
  return static_cast<const LevelKernels&>(lk).groups[(size_t)level];
}
double level_kernels_compile_ms(const PassKernels& lk) { return static_cast<const LevelKernels&>(lk).compile_ms; }

cudaError_t launch_level_kernel(const PassKernels& lkb, int level, const GroupLevelDesc* d_desc, uint64_t total,
                                cudaStream_t st) {
  const LevelKernels& lk = static_cast<const LevelKernels&>(lkb);
  if (level < 0 || level >= (int)lk.kernel.size() || !lk.kernel[(size_t)level] || total == 0)
    return cudaErrorInvalidValue;
  uint64_t grid = (uint64_t)kSMCount * lk.sh.ctas;
  if (grid > total) grid = total;
  const GroupLevelDesc* dp = d_desc;
  unsigned long long tt = total;
  void* args[2] = {&dp, &tt};
  cudaError_t e = cudaLaunchKernel((const void*)lk.kernel[(size_t)level], dim3((unsigned)grid),
                                   dim3((unsigned)lk.threads), args, (size_t)lk.smem[(size_t)level], st);
  count_launch(1);
  return e;
}

std::shared_ptr<const PassKernels> pass_kernels_cached(const Program& prog, int prec, int device) {
  if (device < 0 || device >= 64 || prog.tops.empty()) return nullptr;
  const Shape shape = shape_of(prog, prec);
  const std::string key = std::to_string(prec) + ":" + std::to_string(shape.rbits) + "/" +
                          std::to_string(shape.bufs) + "/" + std::to_string(shape.ctas) + ":" +
                          pass_structure_key(prog, false);
  std::lock_guard<std::mutex> lk(g_mu);
  std::shared_ptr<Compiled>* hit = g_cache[device].find(key);
  if (!hit || !*hit) return nullptr;
  ++g_cache_hits;
  return *hit;
}

bool pass_kernel_ready(const PassKernels& pk, size_t step) {
  const Compiled& c = static_cast<const Compiled&>(pk);
  return step < c.kernel.size() && c.kernel[step] != nullptr;
}

double pass_kernels_compile_ms(const PassKernels& pk) { return static_cast<const Compiled&>(pk).compile_ms; }

cudaError_t launch_pass_kernel(const PassKernels& pk, size_t step, int n, const PassDesc& pd, void* state, int prec,
                               cudaStream_t st) {
  const Compiled& c = static_cast<const Compiled&>(pk);
  if (step >= c.kernel.size() || !c.kernel[step]) return cudaErrorInvalidValue;
  const uint64_t ntiles = 1ULL << (n - pd.k);
  const Shape sh = c.sh;
  (void)prec;
  uint64_t grid = (uint64_t)kSMCount * sh.ctas;
  if (grid > ntiles) grid = ntiles;
  unsigned long long nt = ntiles;
  unsigned char* sp = static_cast<unsigned char*>(state);
  void* args[2] = {&sp, &nt};
  cudaError_t e = cudaLaunchKernel((const void*)c.kernel[step], dim3((unsigned)grid),
                                   dim3((unsigned)((1 << pd.k) >> sh.rbits)), args, (size_t)c.smem[step], st);
  count_launch(1);
  return e;
}

cudaError_t launch_pass_kernel_batch(const PassKernels& pk, size_t step, int n, const PassDesc& pd,
                                     void* const* d_states, int nstates, const float* d_coefs, int prec,
                                     cudaStream_t st) {
  const Compiled& c = static_cast<const Compiled&>(pk);
  if (step >= c.kernel.size() || !c.kernel[step] || nstates < 1) return cudaErrorInvalidValue;
  const uint64_t ntiles = 1ULL << (n - pd.k);
  const Shape sh = c.sh;
  (void)prec;
  uint64_t grid = (uint64_t)kSMCount * sh.ctas;
  if (grid > ntiles * (uint64_t)nstates) grid = ntiles * (uint64_t)nstates;
  unsigned long long nt = ntiles;
  int ns = nstates;
  int ncoef = 16 * (int)(pd.op_end - pd.op_begin);
  void* states = const_cast<void**>(d_states);
  const float* coefs = d_coefs;
  void* args[5] = {&states, &coefs, &ncoef, &nt, &ns};
  cudaError_t e = cudaLaunchKernel((const void*)c.kernel[step], dim3((unsigned)grid),
                                   dim3((unsigned)((1 << pd.k) >> sh.rbits)), args, (size_t)c.smem[step], st);
  count_launch(1);
  return e;
}

// Coefficient rows of one pass for the table form: 16 floats per op, in the
// pass's op order (double-float: hi[8], lo[8]; complex64: the 8 entries as
// floats). Parity ops instead hold their masks under the kernel's layout (tile
// bits in floats 12-13, thread bits in 14, and in 15 the register-parity mask, bit j
// the parity of register j's bits under the op's register mask; as raw bits) and,
// per run, the table of combined phases (entry m < E in floats 0-3 of the run's
// row m, entry E in floats 4-7 of its first row; complex64: 2 floats each).
void pass_coefficients(const Program& prog, size_t step, int prec, float* out) {
  const PassDesc& pd = prog.steps[step].pass;
  const int nops = (int)(pd.op_end - pd.op_begin);
  const TOp* ops = prog.tops.data() + pd.op_begin;
  bool parity = false;
  for (int i = 0; i < nops; ++i) {
    const TOp& t = ops[i];
    float* row = out + 16 * i;
    parity = parity || t.kind == OK_PARITY;
    if (prec == QG_C128) {
      std::memcpy(row, t.mf, sizeof(float) * 16);
    } else {
      for (int q = 0; q < 8; ++q) row[q] = (float)t.m[q];
      for (int q = 8; q < 16; ++q) row[q] = 0.0f;
    }
  }
  if (!parity) return;
  std::vector<TOp> tagged(ops, ops + nops);
  for (int i = 0; i < nops; ++i) tagged[i].pad1 = i;
  const std::vector<TOp> plan =
      plan_layouts(tagged.data(), nops, pd.k, shape_of(prog, prec).rbits, true, prec == QG_C64);
  const int ns = 1 << shape_of(prog, prec).rbits;  // registers per thread
  auto put = [&](float* at, std::complex<double> v) {
    if (prec == QG_C128) {
      const float rh = (float)v.real(), ih = (float)v.imag();
      at[0] = rh;
      at[1] = (float)(v.real() - (double)rh);
      at[2] = ih;
      at[3] = (float)(v.imag() - (double)ih);
    } else {
      at[0] = (float)v.real();
      at[1] = (float)v.imag();
      at[2] = at[3] = 0.0f;
    }
  };
  for (size_t i = 0; i < plan.size(); ++i) {
    if (plan[i].kind != OK_PARITY) continue;
    const int end = parity_run_end(plan.data(), (int)plan.size(), (int)i);
    const int E = end - (int)i;
    const auto tab = parity_table(plan[i], E);
    for (int e = 0; e < E; ++e) {
      const TOp& t = plan[i + e];
      float* row = out + 16 * t.pad1;
      // register-parity mask: bit j = parity of register j's bits under the op's mask
      uint32_t par = 0;
      for (int j = 0; j < ns; ++j) par |= (uint32_t)(__builtin_popcount((unsigned)j & t.rmask) & 1) << j;
      const uint32_t g0 = (uint32_t)t.gmask, g1 = (uint32_t)(t.gmask >> 32), tm = t.tmask;
      std::memcpy(row + 12, &g0, 4);
      std::memcpy(row + 13, &g1, 4);
      std::memcpy(row + 14, &tm, 4);
      std::memcpy(row + 15, &par, 4);
      put(row, tab[e]);
    }
    put(out + 16 * plan[i].pad1 + 4, tab[E]);
    i = (size_t)end - 1;
  }
}

void pass_kernel_cache_stats(size_t* hits, size_t* misses) {
  std::lock_guard<std::mutex> lk(g_mu);
  *hits = g_cache_hits;
  *misses = g_cache_misses;
}

}  // namespace qg
