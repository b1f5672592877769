// Circuit compiler: reference operations -> device gate ops -> HBM passes.
//
// lower_circuit() restates the gate dispatch of
// src/org/soulspace/qclojure/domain/circuit.clj:933-1112 and the gate matrices of
// src/org/soulspace/qclojure/domain/gate.clj:38-283 (angles through libm cos/sin
// with the same argument expressions). Every 2x2 is classified by its exact zero,
// one and unit-imaginary entries, so permutations and sign/i phases run without
// floating-point arithmetic and the remaining classes use only the products the
// reference's complex multiply forms (gate.clj:384-395 via the dense row sum).
//
// schedule() groups gate runs into passes. PLAIN: one HBM pass per gate.
// TILED: consecutive gates whose non-diagonal target bits fit in one tile of
// 2^k amplitudes share a pass (diagonal gates and control bits need no
// locality). DENSE: gate runs on at most fuse_k qubits are multiplied into a
// 2^k x 2^k FP64 block, applied in one pass (the gate fuser hooked where
// src/org/soulspace/qclojure/domain/gate_optimization.clj:776-860 runs).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>

#include "qgpu_internal.h"

namespace qg {

namespace {

using cd = std::complex<double>;

inline int bitof(int n, int q) { return n - 1 - q; }

void set_m(double m[8], double a, double b, double c, double d, double e, double f, double g, double h) {
  m[0] = a; m[1] = b; m[2] = c; m[3] = d; m[4] = e; m[5] = f; m[6] = g; m[7] = h;
}

// gate.clj:38-283 (same libm argument expressions as the oracle)
bool gate_matrix(int opcode, double angle, double m[8]) {
  const double s2 = 1.0 / std::sqrt(2.0);
  switch (opcode) {
    case QG_OP_X: set_m(m, 0, 0, 1, 0, 1, 0, 0, 0); return true;
    case QG_OP_Y: set_m(m, 0, 0, 0, -1, 0, 1, 0, 0); return true;
    case QG_OP_Z: set_m(m, 1, 0, 0, 0, 0, 0, -1, 0); return true;
    case QG_OP_H: set_m(m, s2, 0, s2, 0, s2, 0, -s2, 0); return true;
    case QG_OP_S: set_m(m, 1, 0, 0, 0, 0, 0, 0, 1); return true;
    case QG_OP_SDAG: set_m(m, 1, 0, 0, 0, 0, 0, 0, -1); return true;
    case QG_OP_T: set_m(m, 1, 0, 0, 0, 0, 0, std::cos(M_PI / 4), std::sin(M_PI / 4)); return true;
    case QG_OP_TDAG: set_m(m, 1, 0, 0, 0, 0, 0, std::cos(M_PI / -4), std::sin(M_PI / -4)); return true;
    case QG_OP_PHASE: set_m(m, 1, 0, 0, 0, 0, 0, std::cos(angle), std::sin(angle)); return true;
    case QG_OP_RX: {
      double c = std::cos(angle / 2), s = std::sin(angle / 2);
      set_m(m, c, 0, 0, -s, 0, -s, c, 0);
      return true;
    }
    case QG_OP_RY: {
      double c = std::cos(angle / 2), s = std::sin(angle / 2);
      set_m(m, c, 0, -s, 0, s, 0, c, 0);
      return true;
    }
    case QG_OP_RZ:
      set_m(m, std::cos(angle / -2), std::sin(angle / -2), 0, 0, 0, 0, std::cos(angle / 2), std::sin(angle / 2));
      return true;
    default: return false;
  }
}

void transpose(double m[8]) {
  std::swap(m[2], m[4]);
  std::swap(m[3], m[5]);
}

inline bool is0(double re, double im) { return re == 0.0 && im == 0.0; }
inline bool is1(double re, double im) { return re == 1.0 && im == 0.0; }

// Build the device op for a 2x2 matrix on bit t under control mask cmask.
GOp classify(const double m[8], int t, uint64_t cmask) {
  GOp g;
  std::memset(&g, 0, sizeof(g));
  g.kind = OK_U2;
  g.t = t;
  g.cmask = cmask;
  std::memcpy(g.m, m, sizeof(double) * 8);
  bool off0 = is0(m[2], m[3]) && is0(m[4], m[5]);
  bool dia0 = is0(m[0], m[1]) && is0(m[6], m[7]);
  if (off0) {
    if (is1(m[0], m[1])) {
      // only the bit=1 half changes: a phase on (idx & (cmask|bit)) == ...
      g.kind = OK_PHASE;
      g.mask = cmask | (1ULL << t);
      g.m[0] = m[6];
      g.m[1] = m[7];
      for (int k = 2; k < 8; ++k) g.m[k] = 0;
      if (m[6] == 1.0 && m[7] == 0.0) {
        g.kind = -1;  // identity
      } else if (m[6] == -1.0 && m[7] == 0.0) {
        g.cls = PH_NEG;
      } else if (m[6] == 0.0 && m[7] == 1.0) {
        g.cls = PH_I;
      } else if (m[6] == 0.0 && m[7] == -1.0) {
        g.cls = PH_MINUS_I;
      } else {
        g.cls = PH_GENERAL;
      }
      return g;
    }
    g.cls = U2_DIAG;
    return g;
  }
  if (dia0) {
    if (is1(m[2], m[3]) && is1(m[4], m[5])) {
      g.cls = U2_X;
    } else if (m[2] == 0.0 && (m[3] == 1.0 || m[3] == -1.0) && m[4] == 0.0 && (m[5] == 1.0 || m[5] == -1.0)) {
      g.cls = U2_IMAG_ANTI;
    } else {
      g.cls = U2_ANTIDIAG;
    }
    return g;
  }
  if (m[1] == 0.0 && m[3] == 0.0 && m[5] == 0.0 && m[7] == 0.0) {
    g.cls = U2_REAL;
  } else if (m[1] == 0.0 && m[7] == 0.0 && m[2] == 0.0 && m[4] == 0.0) {
    g.cls = U2_RXLIKE;
  } else {
    g.cls = U2_GENERAL;
  }
  return g;
}

GOp make_phase(uint64_t mask, double re, double im) {
  GOp g;
  std::memset(&g, 0, sizeof(g));
  g.kind = OK_PHASE;
  g.mask = mask;
  g.m[0] = re;
  g.m[1] = im;
  g.cls = PH_GENERAL;
  if (re == -1.0 && im == 0.0) g.cls = PH_NEG;
  else if (re == 0.0 && im == 1.0) g.cls = PH_I;
  else if (re == 0.0 && im == -1.0) g.cls = PH_MINUS_I;
  else if (re == 1.0 && im == 0.0) g.kind = -1;
  return g;
}

bool push(std::vector<GOp>* out, const GOp& g) {
  if (g.kind >= 0) out->push_back(g);
  return true;
}

}  // namespace

int lower_circuit(const qg_circuit* c, std::vector<GOp>* gops, std::vector<std::vector<int>>* measures,
                  std::vector<int>* measure_at, std::string* err) {
  const int n = c->num_qubits;
  if (n < 1 || n > QG_MAX_QUBITS) {
    *err = "num-qubits must be a positive integer within the device limit";
    return QG_ERR_INVALID_ARG;
  }
  if (c->num_ops < 0 || (c->num_ops > 0 && !c->ops)) {
    *err = "operations must be a vector";
    return QG_ERR_INVALID_ARG;
  }
  auto inrange = [n](int q) { return q >= 0 && q < n; };
  int32_t kraus_sites = 0;
  for (int k = 0; k < c->num_ops; ++k) {
    const qg_op& op = c->ops[k];
    const int oc = op.opcode;
    double m[8];
    auto qerr = [&](const char* what) {
      *err = std::string(what) + " (operation " + std::to_string(k) + ")";
      return QG_ERR_QUBIT_RANGE;
    };
    if (op.nq < 0 || op.nq > QG_MAX_OP_QUBITS) {
      *err = "invalid operand count";
      return QG_ERR_INVALID_ARG;
    }
    switch (oc) {
      case QG_OP_X: case QG_OP_Y: case QG_OP_Z: case QG_OP_H: case QG_OP_S: case QG_OP_SDAG:
      case QG_OP_T: case QG_OP_TDAG: case QG_OP_RX: case QG_OP_RY: case QG_OP_RZ: case QG_OP_PHASE:
      case QG_OP_U: {
        int q = op.q[0];
        if (!inrange(q)) return qerr("Assert failed: (< qubit-index (:num-qubits state))");
        if (oc == QG_OP_U) std::memcpy(m, op.m, sizeof(m));
        else gate_matrix(oc, op.angle, m);
        push(gops, classify(m, bitof(n, q), 0));
      } break;
      case QG_OP_KRAUS: {  // general matrix, tagged with its ordinal so the noisy runner can patch it
        int q = op.q[0];
        if (!inrange(q)) return qerr("Assert failed: (< qubit-index (:num-qubits state))");
        GOp g;
        std::memset(&g, 0, sizeof(g));
        g.kind = OK_U2;
        g.cls = U2_GENERAL;
        g.t = bitof(n, q);
        std::memcpy(g.m, op.m, sizeof(g.m));
        g.tag = ++kraus_sites;
        gops->push_back(g);
      } break;
      case QG_OP_CNOT: case QG_OP_CZ: case QG_OP_CY: case QG_OP_CRX: case QG_OP_CRY: case QG_OP_CRZ:
      case QG_OP_RYDBERG_CZ: case QG_OP_CU: {
        int ctl = op.q[0], tgt = op.q[1];
        if (!inrange(ctl) || !inrange(tgt)) return qerr("control and target must be qubits of the state");
        if (ctl == tgt) return qerr("control and target must differ");
        int base = oc == QG_OP_CNOT ? QG_OP_X
                 : (oc == QG_OP_CZ || oc == QG_OP_RYDBERG_CZ) ? QG_OP_Z
                 : oc == QG_OP_CY ? QG_OP_Y
                 : oc == QG_OP_CRX ? QG_OP_RX
                 : oc == QG_OP_CRY ? QG_OP_RY : QG_OP_RZ;
        if (oc == QG_OP_CU) std::memcpy(m, op.m, sizeof(m));
        else gate_matrix(base, op.angle, m);
        transpose(m);  // gate.clj:473-483 applies G^T
        push(gops, classify(m, bitof(n, tgt), 1ULL << bitof(n, ctl)));
      } break;
      case QG_OP_RYDBERG_CPHASE: {
        int ctl = op.q[0], tgt = op.q[1];
        if (!inrange(ctl) || !inrange(tgt)) return qerr("control and target must be qubits of the state");
        push(gops, make_phase((1ULL << bitof(n, ctl)) | (1ULL << bitof(n, tgt)), std::cos(op.angle),
                              std::sin(op.angle)));
      } break;
      case QG_OP_RZZ: {
        int a = op.q[0], b = op.q[1];
        if (!inrange(a) || !inrange(b) || a == b) return qerr("RZZ needs two distinct qubits of the state");
        GOp g;
        std::memset(&g, 0, sizeof(g));
        g.kind = OK_PARITY;
        g.mask = (1ULL << bitof(n, a)) | (1ULL << bitof(n, b));
        g.m[0] = std::cos(op.angle / -2);
        g.m[1] = std::sin(op.angle / -2);
        g.m[2] = std::cos(op.angle / 2);
        g.m[3] = std::sin(op.angle / 2);
        gops->push_back(g);
      } break;
      case QG_OP_SWAP: case QG_OP_ISWAP: {
        int b1 = op.q[0], b2 = op.q[1];  // LSB bit positions (gate.clj:768-778)
        if (!inrange(b1) || !inrange(b2)) return qerr("SWAP qubits must index bits of the state");
        if (b1 == b2) break;             // equal bits: the reference leaves every amplitude in place
        GOp g;
        std::memset(&g, 0, sizeof(g));
        g.kind = OK_SWAP;
        g.t = std::min(b1, b2);
        g.t2 = std::max(b1, b2);
        g.flags = oc == QG_OP_ISWAP ? 1 : 0;
        gops->push_back(g);
      } break;
      case QG_OP_TOFFOLI: {
        int c1 = op.q[0], c2 = op.q[1], t = op.q[2];
        if (!inrange(c1) || !inrange(c2) || !inrange(t)) return qerr("Toffoli operands must be qubits of the state");
        if (c1 == c2 || c1 == t || c2 == t) return qerr("Toffoli operands must be distinct");
        gate_matrix(QG_OP_X, 0, m);
        push(gops, classify(m, bitof(n, t), (1ULL << bitof(n, c1)) | (1ULL << bitof(n, c2))));
      } break;
      case QG_OP_FREDKIN: {
        int ctl = op.q[0], t1 = op.q[1], t2 = op.q[2];
        if (!inrange(ctl) || !inrange(t1) || !inrange(t2)) return qerr("Fredkin operands must be qubits of the state");
        if (ctl == t1 || ctl == t2 || t1 == t2) return qerr("Fredkin operands must be distinct");
        GOp g;
        std::memset(&g, 0, sizeof(g));
        g.kind = OK_SWAP;
        int a = bitof(n, t1), b = bitof(n, t2);
        g.t = std::min(a, b);
        g.t2 = std::max(a, b);
        g.cmask = 1ULL << bitof(n, ctl);
        gops->push_back(g);
      } break;
      case QG_OP_RYDBERG_BLOCKADE: {
        if (op.nq < 1) return qerr("Rydberg blockade requires qubit-indices");
        uint64_t mask = 0;
        for (int j = 0; j < op.nq; ++j) {
          if (!inrange(op.q[j])) return qerr("blockade qubit out of range");
          uint64_t b = 1ULL << bitof(n, op.q[j]);
          if (mask & b) return qerr("blockade qubits must be distinct");
          mask |= b;
        }
        GOp g;
        std::memset(&g, 0, sizeof(g));
        g.kind = OK_BLOCKADE;
        g.mask = mask;
        g.m[0] = std::cos(op.angle);
        g.m[1] = std::sin(op.angle);
        gops->push_back(g);
      } break;
      case QG_OP_GLOBAL_RX: case QG_OP_GLOBAL_RY: case QG_OP_GLOBAL_RZ: case QG_OP_GLOBAL_H:
      case QG_OP_GLOBAL_X: case QG_OP_GLOBAL_Y: case QG_OP_GLOBAL_Z: {
        int base = (oc == QG_OP_GLOBAL_RX || oc == QG_OP_GLOBAL_X) ? QG_OP_RX
                 : (oc == QG_OP_GLOBAL_RY || oc == QG_OP_GLOBAL_Y) ? QG_OP_RY
                 : (oc == QG_OP_GLOBAL_RZ || oc == QG_OP_GLOBAL_Z) ? QG_OP_RZ : QG_OP_H;
        double ang = (oc == QG_OP_GLOBAL_X || oc == QG_OP_GLOBAL_Y || oc == QG_OP_GLOBAL_Z) ? M_PI : op.angle;
        gate_matrix(base, ang, m);
        for (int q = 0; q < n; ++q) push(gops, classify(m, bitof(n, q), 0));
      } break;
      case QG_OP_MEASURE: {
        if (op.nq < 1 || op.nq > 20) return qerr("Measure requires 1..20 measurement-qubits");
        std::vector<int> qs;
        for (int j = 0; j < op.nq; ++j) {
          if (!inrange(op.q[j])) return qerr("measurement qubit out of range");
          qs.push_back(op.q[j]);
        }
        measures->push_back(qs);
        measure_at->push_back((int)gops->size());
      } break;
      default:
        *err = "Unknown gate type (operation " + std::to_string(k) + ")";
        return QG_ERR_UNKNOWN_GATE;
    }
  }
  return QG_OK;
}

// Scalar factoring for the tolerance-held policies (double-float c128, c64):
//   - uncontrolled diagonal gates diag(d0, d1) become a phase d1/d0 on the bit-1
//     half and a global factor d0;
//   - Hadamards [[s, s], [s, -s]] become the sum / difference [[1, 1], [1, -1]]
//     and a factor s = 1/sqrt 2;
//   - rotations with equal diagonal entries (RY-shaped [[c, -s], [s, c]], RX-shaped
//     [[c, ib], [ib, c]]) become a form with unit diagonal, [[1, t], [u, +-1]],
//     and a factor: the diagonal entry when it is the larger in magnitude, else the
//     off-diagonal one, with an X (a register renaming) after the gate. Each output
//     then needs one product and one sum instead of two products and a sum.
// The collected factor is applied as one op on every amplitude before each
// measurement and at the end of the circuit (the state is only scaled in
// between); whenever its magnitude falls below 2^-20 the state is rescaled by
// 2^-20 exactly, so magnitudes stay within the float range. The exact policy
// keeps the reference's products. measure_at (positions of measurements before
// op indices) is rewritten for the new op list. rotations = kFactorNone leaves
// the rotations alone: sweep members of one structure must keep equal op lists,
// and both the form a rotation takes and the number of rescales depend on the
// angles.
void factor_global_phases(std::vector<GOp>* gops, std::vector<int>* measure_at, int rotations) {
  const double s2 = 1.0 / std::sqrt(2.0);
  std::vector<GOp> out;
  out.reserve(gops->size() + 8);
  std::vector<int> newpos(gops->size() + 1, 0);
  cd pending(1.0, 0.0);
  auto emit_scale = [&]() {
    const GOp ph = make_phase(0, pending.real(), pending.imag());
    if (ph.kind >= 0) out.push_back(ph);
    pending = cd(1.0, 0.0);
  };
  auto absorb = [&](cd f) {
    pending *= f;
    while (std::abs(pending) < 0x1p-20) {  // keep the unscaled amplitudes below 2^20 times their norm
      out.push_back(make_phase(0, 0x1p-20, 0.0));
      pending *= 0x1p20;
    }
  };
  auto xgate = [&](int t) {
    double m[8] = {0, 0, 1, 0, 1, 0, 0, 0};
    GOp x = classify(m, t, 0);
    return x;
  };
  std::vector<char> measured_before(gops->size() + 1, 0);
  for (int at : *measure_at)
    if (at >= 0 && at <= (int)gops->size()) measured_before[at] = 1;
  for (size_t i = 0; i < gops->size(); ++i) {
    if (measured_before[i]) emit_scale();
    newpos[i] = (int)out.size();
    GOp g = (*gops)[i];
    const double* m = g.m;
    bool then_x = false;
    cd f(1.0, 0.0);
    if (g.kind == OK_U2 && g.cmask == 0) {
      if (g.cls == U2_DIAG) {
        const cd d0(m[0], m[1]), d1(m[6], m[7]);
        if (d0 != cd(0.0, 0.0)) {
          const cd r = d1 / d0;
          f = d0;
          g = make_phase(1ULL << g.t, r.real(), r.imag());
        }
      } else if (g.cls == U2_REAL && m[0] == s2 && m[2] == s2 && m[4] == s2 && m[6] == -s2) {
        f = cd(s2, 0.0);
        g.m[0] = g.m[2] = g.m[4] = 1.0;
        g.m[6] = -1.0;
      } else if (rotations && g.cls == U2_REAL && m[0] == m[6] && m[2] == -m[4] && m[0] != 0.0 && m[4] != 0.0) {
        double n[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (std::fabs(m[0]) >= std::fabs(m[4])) {  // c [[1, -s/c], [s/c, 1]]
          f = cd(m[0], 0.0);
          n[0] = 1.0, n[2] = m[2] / m[0], n[4] = m[4] / m[0], n[6] = 1.0;
        } else {  // X then s [[1, c/s], [c/s, -1]]: the rows of X.R over s
          f = cd(m[4], 0.0);
          n[0] = 1.0, n[2] = m[6] / m[4], n[4] = m[0] / m[4], n[6] = m[2] / m[4];
          then_x = true;
        }
        g = classify(n, g.t, 0);
      } else if (rotations && g.cls == U2_RXLIKE && m[0] == m[6] && m[3] == m[5] && m[0] != 0.0 && m[3] != 0.0) {
        double n[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (std::fabs(m[0]) >= std::fabs(m[3])) {  // c [[1, i b/c], [i b/c, 1]]
          f = cd(m[0], 0.0);
          n[0] = 1.0, n[3] = m[3] / m[0], n[5] = m[5] / m[0], n[6] = 1.0;
        } else {  // X then (i b) [[1, -i c/b], [-i c/b, 1]]
          f = cd(0.0, m[3]);
          n[0] = 1.0, n[3] = -m[0] / m[3], n[5] = -m[6] / m[3], n[6] = 1.0;
          then_x = true;
        }
        g = classify(n, g.t, 0);
      }
    }
    if (g.kind >= 0) out.push_back(g);
    if (then_x) out.push_back(xgate(g.t));
    if (f != cd(1.0, 0.0)) absorb(f);
  }
  if (measured_before[gops->size()]) emit_scale();
  newpos[gops->size()] = (int)out.size();
  if (!measured_before[gops->size()]) emit_scale();
  for (int& at : *measure_at)
    if (at >= 0 && at <= (int)gops->size()) at = newpos[at];
  gops->swap(out);
}

// ---------------------------------------------------------------------------
// Scheduling
// ---------------------------------------------------------------------------
namespace {

uint64_t required_local(const GOp& g) {
  switch (g.kind) {
    case OK_U2: return 1ULL << g.t;
    case OK_SWAP: return (1ULL << g.t) | (1ULL << g.t2);
    case OK_DENSE: {
      uint64_t r = 0;
      for (int j = 0; j < g.dk; ++j) r |= 1ULL << g.dbits[j];
      return r;
    }
    default: return 0;  // diagonal in the computational basis
  }
}

uint64_t touched(const GOp& g) {
  switch (g.kind) {
    case OK_U2: return (1ULL << g.t) | g.cmask;
    case OK_SWAP: return (1ULL << g.t) | (1ULL << g.t2) | g.cmask;
    case OK_DENSE: return required_local(g);
    default: return g.mask;
  }
}

void fill_pass_desc(int n, uint64_t L, PassDesc* pd) {
  std::memset(pd, 0, sizeof(*pd));
  int k = 0;
  for (int b = 0; b < n; ++b)
    if (L & (1ULL << b)) pd->lbits[k++] = b;
  pd->k = k;
  int klow = 0;
  while (klow < k && pd->lbits[klow] == klow) ++klow;
  pd->klow = klow;
  // runs of non-local bits, in ascending absolute order
  int src = 0, nr = 0, b = 0;
  while (b < n) {
    if (L & (1ULL << b)) { ++b; continue; }
    int start = b;
    while (b < n && !(L & (1ULL << b))) ++b;
    pd->run_src[nr] = src;
    pd->run_dst[nr] = start;
    pd->run_len[nr] = b - start;
    src += b - start;
    ++nr;
  }
  pd->nruns = nr;
}

TOp localize(const GOp& g, const int* lpos /* abs bit -> local or -1 */, int n) {
  TOp t;
  std::memset(&t, 0, sizeof(t));
  t.kind = g.kind;
  t.cls = g.cls;
  t.flags = g.flags;
  t.dk = g.dk;
  t.doff = g.doff;
  t.tag = (uint32_t)g.tag;
  std::memcpy(t.m, g.m, sizeof(t.m));
  auto split = [&](uint64_t mask, uint32_t* lm, uint64_t* gm) {
    *lm = 0;
    *gm = 0;
    for (int b = 0; b < n; ++b) {
      if (!(mask & (1ULL << b))) continue;
      if (lpos[b] >= 0) *lm |= 1u << lpos[b];
      else *gm |= 1ULL << b;
    }
  };
  if (g.kind == OK_U2 || g.kind == OK_SWAP) {
    t.t = lpos[g.t];
    t.t2 = g.kind == OK_SWAP ? lpos[g.t2] : 0;
  }
  split(g.cmask, &t.lcmask, &t.gcmask);
  split(g.mask, &t.lmask, &t.gmask);
  split(g.val, &t.lval, &t.gval);
  for (int j = 0; j < g.dk; ++j) t.dbits[j] = lpos[g.dbits[j]];
  return t;
}

// host FP64 application of a gate op to a small register (bits remapped through pos[])
void host_apply(std::vector<cd>& v, int kb, const int* pos, const GOp& g) {
  const uint64_t N = 1ULL << kb;
  auto remap = [&](uint64_t mask) {
    uint64_t r = 0;
    for (int j = 0; j < kb; ++j)
      if (mask & (1ULL << pos[j])) r |= 1ULL << j;
    return r;
  };
  auto lb = [&](int b) {
    for (int j = 0; j < kb; ++j)
      if (pos[j] == b) return j;
    return -1;
  };
  if (g.kind == OK_U2) {
    int t = lb(g.t);
    uint64_t cm = remap(g.cmask), tb = 1ULL << t;
    cd m0(g.m[0], g.m[1]), m1(g.m[2], g.m[3]), m2(g.m[4], g.m[5]), m3(g.m[6], g.m[7]);
    for (uint64_t i = 0; i < N; ++i) {
      if ((i & tb) || (i & cm) != cm) continue;
      cd x0 = v[i], x1 = v[i | tb];
      v[i] = m0 * x0 + m1 * x1;
      v[i | tb] = m2 * x0 + m3 * x1;
    }
  } else if (g.kind == OK_PHASE) {
    uint64_t mk = remap(g.mask);
    cd ph(g.m[0], g.m[1]);
    if (g.cls == PH_NEG) ph = cd(-1, 0);
    if (g.cls == PH_I) ph = cd(0, 1);
    if (g.cls == PH_MINUS_I) ph = cd(0, -1);
    for (uint64_t i = 0; i < N; ++i)
      if ((i & mk) == mk) v[i] *= ph;
  } else if (g.kind == OK_SWAP) {
    int a = lb(g.t), b = lb(g.t2);
    uint64_t cm = remap(g.cmask);
    for (uint64_t i = 0; i < N; ++i) {
      if ((i & cm) != cm) continue;
      if (((i >> a) & 1) && !((i >> b) & 1)) {
        uint64_t j = i ^ (1ULL << a) ^ (1ULL << b);
        cd x = v[i], y = v[j];
        if (g.flags & 1) {
          v[i] = cd(0, 1) * y;
          v[j] = cd(0, 1) * x;
        } else {
          v[i] = y;
          v[j] = x;
        }
      }
    }
  } else if (g.kind == OK_BLOCKADE) {
    uint64_t mk = remap(g.mask);
    cd ph(g.m[0], g.m[1]);
    for (uint64_t i = 0; i < N; ++i)
      if (__builtin_popcountll(i & mk) == 1) v[i] *= ph;
  } else if (g.kind == OK_PARITY) {
    uint64_t mk = remap(g.mask);
    cd p0(g.m[0], g.m[1]), p1(g.m[2], g.m[3]);
    for (uint64_t i = 0; i < N; ++i) v[i] *= (__builtin_popcountll(i & mk) & 1) ? p1 : p0;
  }
}

}  // namespace

int tile_bits_for(int n, int precision) {
  (void)precision;
  const int kmax = 12;  // 4096 amplitudes: 512 threads x 8 registers
  return n < kmax ? n : kmax;
}

namespace {

// Split the 2x2 coefficients into float pairs for the double-float policy.
void split_coeffs(TOp* t) {
  for (int q = 0; q < 8; ++q) {
    const float hi = (float)t->m[q];
    t->mf[q] = hi;
    t->mf[8 + q] = (float)(t->m[q] - (double)hi);
  }
}

}  // namespace

void set_op_matrix(TOp* t, const double m[8]) {
  std::memcpy(t->m, m, sizeof(t->m));
  split_coeffs(t);
}

namespace {

// Insert OK_LAYOUT ops: consecutive ops whose non-diagonal bits fit in three
// register bits form a group; the register positions are written into the ops.
void plan_register_groups(std::vector<TOp>& ops, int k) {
  std::vector<TOp> out;
  size_t i = 0;
  while (i < ops.size()) {
    if (ops[i].kind == OK_DENSE) {
      out.push_back(ops[i++]);
      continue;
    }
    uint32_t rb = 0;
    size_t j = i;
    while (j < ops.size() && ops[j].kind != OK_DENSE) {
      uint32_t req = 0;
      if (ops[j].kind == OK_U2) req = 1u << ops[j].t;
      else if (ops[j].kind == OK_SWAP) req = (1u << ops[j].t) | (1u << ops[j].t2);
      if (__builtin_popcount(rb | req) > 3) break;
      rb |= req;
      ++j;
    }
    // Pad the register bits with the local bits that the group's conditions use most
    // (phase masks, controls): a condition on register bits selects registers at
    // compile time, one on thread bits costs every register of a divergent warp.
    // Ties go to the highest bit so the thread bits stay low.
    int uses[32] = {0};
    for (size_t q = i; q < j; ++q) {
      const uint32_t cm = ops[q].kind == OK_U2 || ops[q].kind == OK_SWAP ? ops[q].lcmask : ops[q].lmask;
      for (int b = 0; b < k; ++b)
        if (cm & (1u << b)) ++uses[b];
    }
    while (__builtin_popcount(rb) < 3) {
      int best = -1;
      for (int b = k - 1; b >= 0; --b)
        if (!(rb & (1u << b)) && (best < 0 || uses[b] > uses[best])) best = b;
      rb |= 1u << best;
    }
    int pos[3], np = 0;
    for (int b = 0; b < k && np < 3; ++b)
      if (rb & (1u << b)) pos[np++] = b;
    TOp lay;
    std::memset(&lay, 0, sizeof(lay));
    lay.kind = OK_LAYOUT;
    for (int q = 0; q < 3; ++q) lay.dbits[q] = pos[q];
    for (int s = 0; s < 8; ++s)
      lay.lj[s] = ((uint32_t)(s & 1) << pos[0]) | ((uint32_t)((s >> 1) & 1) << pos[1]) |
                  ((uint32_t)((s >> 2) & 1) << pos[2]);
    out.push_back(lay);
    auto rpos = [&](int b) { return b == pos[0] ? 0 : b == pos[1] ? 1 : 2; };
    const uint32_t rbm = (1u << pos[0]) | (1u << pos[1]) | (1u << pos[2]);
    auto reg_part = [&](uint32_t m) {
      uint32_t r = 0;
      for (int q = 0; q < 3; ++q)
        if (m & (1u << pos[q])) r |= 1u << q;
      return r;
    };
    for (size_t q = i; q < j; ++q) {
      TOp t = ops[q];
      uint32_t m = 0, v = 0;
      if (t.kind == OK_U2) {
        t.t2 = rpos(t.t);
        m = v = t.lcmask;
      } else if (t.kind == OK_SWAP) {
        int a = rpos(t.t), b = rpos(t.t2);
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
      t.tmask = m & ~rbm;
      t.tval = v & ~rbm;
      out.push_back(t);
    }
    i = j;
  }
  ops.swap(out);
}

}  // namespace

int schedule(int n, int precision, int fusion, int fuse_k, const std::vector<GOp>& gops,
             const std::vector<std::vector<int>>& measures, const std::vector<int>& measure_at, Program* prog,
             std::string* err, bool reorder, int tile_bits) {
  prog->n = n;
  prog->steps.clear();
  prog->tops.clear();
  prog->dense.clear();
  prog->dense_tc.clear();
  prog->hbm_passes = 0;
  size_t mi = 0;
  auto emit_measures_at = [&](size_t gi) {
    while (mi < measures.size() && (size_t)measure_at[mi] == gi) {
      Step s;
      s.kind = Step::MEASURE;
      s.mqubits = measures[mi];
      prog->steps.push_back(s);
      prog->hbm_passes += 2;  // marginal reduction + collapse
      ++mi;
    }
  };

  if (fusion == QG_FUSE_PLAIN || n < 5) {  // registers need at least 2^5 amplitudes per tile
    for (size_t gi = 0; gi < gops.size(); ++gi) {
      emit_measures_at(gi);
      Step s;
      s.kind = Step::PLAIN_OP;
      s.op = gops[gi];
      prog->steps.push_back(s);
      prog->hbm_passes += 1;
    }
    emit_measures_at(gops.size());
    return QG_OK;
  }

  const int k = (tile_bits >= 5 && tile_bits <= kMaxTileBits && tile_bits <= n) ? tile_bits : tile_bits_for(n, precision);
  // bits 0..klow_min-1 stay local in every pass: contiguous 128-byte runs in HBM
  const int klow_min = std::min(k, precision == QG_C64 ? 4 : 3);
  const uint64_t low_mask = (klow_min >= 64) ? ~0ULL : ((1ULL << klow_min) - 1);

  // Optional dense-block fusion: rewrite gate runs into OK_DENSE ops first.
  std::vector<GOp> ops;
  std::vector<size_t> orig_index;  // first original gate index of each op (for measurement placement)
  if (fusion == QG_FUSE_DENSE) {
    int kb_max = std::max(1, std::min(fuse_k, std::min(5, n)));
    size_t gi = 0;
    while (gi < gops.size()) {
      // stop a block at a measurement boundary
      size_t limit = gops.size();
      for (size_t j = mi; j < measures.size(); ++j)
        if ((size_t)measure_at[j] > gi) { limit = std::min(limit, (size_t)measure_at[j]); break; }
      uint64_t bits = 0;
      size_t gj = gi;
      while (gj < limit) {
        uint64_t tb = touched(gops[gj]);
        if (__builtin_popcountll(bits | tb) > kb_max) break;
        bits |= tb;
        ++gj;
      }
      if (gj == gi) {  // a single gate wider than the block: keep it as is
        ops.push_back(gops[gi]);
        orig_index.push_back(gi);
        ++gi;
        continue;
      }
      int pos[5], kb = 0;
      for (int b = 0; b < n; ++b)
        if (bits & (1ULL << b)) pos[kb++] = b;
      const uint64_t D = 1ULL << kb;
      GOp d;
      std::memset(&d, 0, sizeof(d));
      d.kind = OK_DENSE;
      d.dk = kb;
      for (int j = 0; j < kb; ++j) d.dbits[j] = pos[j];
      d.doff = (int64_t)(prog->dense.size() / 2);
      std::vector<double> mat(2 * D * D);
      for (uint64_t col = 0; col < D; ++col) {
        std::vector<cd> v(D, cd(0, 0));
        v[col] = cd(1, 0);
        for (size_t g = gi; g < gj; ++g) host_apply(v, kb, pos, gops[g]);
        for (uint64_t row = 0; row < D; ++row) {
          mat[2 * (row * D + col)] = v[row].real();
          mat[2 * (row * D + col) + 1] = v[row].imag();
        }
      }
      if (precision == QG_C64 && dense_tc_eligible(n, kb)) {
        // complex64 blocks run on the tensor cores, one HBM pass each
        std::vector<float> w;
        int tb[5];
        const int ke = dense_tc_prepare(n, kb, pos, mat.data(), &w, tb);
        d.dk = ke;
        for (int j = 0; j < ke; ++j) d.dbits[j] = tb[j];
        d.flags = kDenseTcFlag;
        d.doff = (int64_t)prog->dense_tc.size();
        prog->dense_tc.insert(prog->dense_tc.end(), w.begin(), w.end());
      } else if (precision == QG_C128 && prog->arith == QG_ARITH_DOUBLE_FLOAT) {
        // double-float blocks: each entry as (re.hi, re.lo, im.hi, im.lo) floats, 16 bytes
        // like an FP64 entry, so the entry offsets stay the same
        const size_t at = prog->dense.size();
        prog->dense.resize(at + mat.size());
        float* q = reinterpret_cast<float*>(prog->dense.data() + at);
        for (size_t e = 0; e < mat.size(); ++e) {
          const float h = (float)mat[e];
          q[2 * e] = h;
          q[2 * e + 1] = (float)(mat[e] - (double)h);
        }
      } else {
        prog->dense.insert(prog->dense.end(), mat.begin(), mat.end());
      }
      ops.push_back(d);
      orig_index.push_back(gi);
      gi = gj;
    }
    if (precision == QG_C64 && !prog->dense.empty()) {
      // complex64 blocks multiply in FP32: the entries are stored as float pairs, so a
      // block's offset in complex entries indexes a float2 array
      std::vector<float> f(prog->dense.begin(), prog->dense.end());
      std::vector<double> packed(f.size() / 2);
      std::memcpy(packed.data(), f.data(), sizeof(float) * f.size());
      prog->dense.swap(packed);
    }
  } else {
    ops = gops;
    for (size_t g = 0; g < gops.size(); ++g) orig_index.push_back(g);
  }

  // Greedy pass formation with look-ahead (reorder): an op later in the circuit
  // joins the pass when its non-diagonal bits fit the tile and it touches no
  // qubit of an op left out before it (so it commutes past every op it
  // overtakes). Ops stay in circuit order inside a pass and never cross a
  // measurement. Overtaking changes the order of roundings, so the exact policy
  // (bit-identical to the reference's gate order) forms passes strictly in order.
  std::vector<char> done(ops.size(), 0);
  const uint64_t all_bits = n >= 64 ? ~0ULL : ((1ULL << n) - 1);
  size_t oi = 0;
  mi = 0;
  while (oi < ops.size() || mi < measures.size()) {
    while (oi < ops.size() && done[oi]) ++oi;
    // measurements that come before the next op
    size_t next_gate = oi < ops.size() ? orig_index[oi] : gops.size();
    if (mi < measures.size() && (size_t)measure_at[mi] <= next_gate) {
      Step s;
      s.kind = Step::MEASURE;
      s.mqubits = measures[mi];
      prog->steps.push_back(s);
      prog->hbm_passes += 2;
      ++mi;
      continue;
    }
    if (oi >= ops.size()) break;
    if (ops[oi].kind == OK_DENSE && (ops[oi].flags & kDenseTcFlag)) {  // a tensor-core block is its own pass
      Step s;
      s.kind = Step::PLAIN_OP;
      s.op = ops[oi];
      prog->steps.push_back(s);
      prog->hbm_passes += 1;
      done[oi] = 1;
      continue;
    }
    uint64_t L = low_mask;
    size_t begin = oi;
    size_t limit = ops.size();
    if (mi < measures.size()) {
      // ops before the next measurement only
      while (limit > begin && orig_index[limit - 1] >= (size_t)measure_at[mi]) --limit;
    }
    // at most half the kernel-parameter op records: every gate may need a layout op before it
    const size_t max_ops = (size_t)max_ops_per_tile_pass() / 2;
    // Ops left out so far: bits they change (non-diagonal targets) and bits they
    // read or phase. A later op commutes past them when its own non-diagonal
    // bits avoid both sets and its diagonal bits (controls, phase masks) avoid
    // the changed ones: diagonal ops commute with each other.
    std::vector<size_t> members;
    uint64_t changed = 0, seen = 0;
    for (size_t j = begin; j < limit && members.size() < max_ops; ++j) {
      if (done[j]) continue;
      if (ops[j].kind == OK_DENSE && (ops[j].flags & kDenseTcFlag)) break;
      const uint64_t tb = touched(ops[j]), r = required_local(ops[j]);
      const bool commutes = (r & seen) == 0 && ((tb & ~r) & changed) == 0;
      if (commutes && __builtin_popcountll(L | r) <= k) {
        L |= r;
        members.push_back(j);
        done[j] = 1;
      } else {
        if (!reorder) break;
        changed |= r;
        seen |= tb;
        if ((changed & all_bits) == all_bits) break;
      }
    }
    if (members.empty()) {  // cannot happen for k >= 5 (at most 5 bits per op) but keep it safe
      *err = "operation wider than a tile";
      return QG_ERR_UNSUPPORTED;
    }
    // fill the tile with the lowest remaining bits
    for (int b = 0; b < n && __builtin_popcountll(L) < k; ++b) L |= 1ULL << b;
    Step s;
    s.kind = Step::TILE_PASS;
    fill_pass_desc(n, L, &s.pass);
    int lpos[64];
    for (int b = 0; b < 64; ++b) lpos[b] = -1;
    for (int j = 0; j < s.pass.k; ++j) lpos[s.pass.lbits[j]] = j;
    std::vector<TOp> pass_ops;
    for (size_t j : members) pass_ops.push_back(localize(ops[j], lpos, n));
    plan_register_groups(pass_ops, s.pass.k);
    s.pass.op_begin = (int64_t)prog->tops.size();
    for (TOp& t : pass_ops) {
      split_coeffs(&t);
      prog->tops.push_back(t);
    }
    s.pass.op_end = (int64_t)prog->tops.size();
    prog->steps.push_back(s);
    prog->hbm_passes += 1;
  }
  return QG_OK;
}

}  // namespace qg
