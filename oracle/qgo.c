/*
 * qgo.c - CPU oracle: a plain-C FP64 restatement of QClojure's ideal simulator.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py load this library, and only as the
 * checker or as the timed CPU implementation of the reference algorithm. The
 * product (libqgpu.so) never links, loads or calls it.
 *
 * Parity pinning: the reference (Clojure/JVM) cannot run in this container, so
 * this restatement is pinned against the known-answer tests of the reference's
 * own test suite (tests/golden/reference_kat.json, each case citing its
 * test file:line). Multi-layer circuits beyond those tests are pinned by the
 * restatement alone.
 *
 * Semantics followed (all paths relative to the reference project root):
 *  - basis order: qubit q <-> bit (n-1-q) (src/org/soulspace/qclojure/domain/state.clj:114-136)
 *  - 1-qubit gates: dense Kronecker mat-vec (domain/gate.clj:323-395 with
 *    domain/math/fastmath/complex_linear_algebra.clj:408-431). Every row has two
 *    non-zero entries, the other products are exact zeros, so the row sum is
 *    fl(g_r0*x_lo + g_r1*x_hi) with complex mult (ac-bd, ad+bc) and no FMA
 *    (this file is compiled with -ffp-contract=off).
 *  - controlled gates apply the transpose (domain/gate.clj:424-486, :473-483):
 *    new[t0] = x0*g00 + x1*g10, new[t1] = x0*g01 + x1*g11.
 *  - SWAP / iSWAP operands are LSB bit positions (domain/gate.clj:760-834).
 *  - Toffoli / Fredkin big-endian (domain/gate.clj:837-969).
 *  - Rydberg CZ = controlled Z, CPhase multiplies |11> by e^{i phi}, blockade
 *    multiplies states with exactly one excited qubit (domain/gate.clj:977-1096).
 *  - global gates are n sequential 1-qubit gates; global X/Y/Z are RX/RY/RZ(pi)
 *    (domain/gate.clj:1098-1250).
 *  - :i and unknown opcodes fail like circuit.clj:1072 ("Unknown gate type").
 *  - probabilities p = |a|^2 (state.clj:658-682).
 *  - sampling and collapse choose the first outcome whose cumulative probability
 *    exceeds the draw (state.clj:897-911, :976-987); the draw is a Philox4x32-10
 *    uniform (Salmon et al., SC'11) turned into an integer in [0, T) over
 *    probabilities quantised to 2^-62, so CPU and GPU agree on the same seed.
 *  - Pauli expectation Re<psi|P|psi>, char i of the string on qubit i
 *    (domain/observables.clj:216-251, domain/hamiltonian.clj:82-114).
 *  - QG_OP_KRAUS (noisy trajectories): the operator's 2x2 matrix on its qubit
 *    (apply-matrix-to-amplitude, domain/channel.clj:127-146), then normalize-state
 *    (state.clj:524-551): every amplitude times 1/norm when norm > 1e-12
 *    (apply-single-qubit-kraus-operator, domain/channel.clj:148-192).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/qgpu.h"

#define ORC_OK 0
#define ORC_ERR 1

typedef struct { double re, im; } cpx;

static inline cpx cmul(cpx a, cpx b) {
  cpx r;
  r.re = a.re * b.re - a.im * b.im;
  r.im = a.re * b.im + a.im * b.re;
  return r;
}
static inline cpx cadd(cpx a, cpx b) {
  cpx r;
  r.re = a.re + b.re;
  r.im = a.im + b.im;
  return r;
}
static inline cpx ld(const double* s, uint64_t i) { cpx r; r.re = s[2 * i]; r.im = s[2 * i + 1]; return r; }
static inline void st(double* s, uint64_t i, cpx v) { s[2 * i] = v.re; s[2 * i + 1] = v.im; }
static inline cpx mk(double re, double im) { cpx r; r.re = re; r.im = im; return r; }

/* ---- gate matrices (domain/gate.clj:38-283) ------------------------------ */
static void gate_matrix(int opcode, double angle, cpx g[4]) {
  double s2 = 1.0 / sqrt(2.0);
  switch (opcode) {
    case QG_OP_X: g[0] = mk(0, 0); g[1] = mk(1, 0); g[2] = mk(1, 0); g[3] = mk(0, 0); break;
    case QG_OP_Y: g[0] = mk(0, 0); g[1] = mk(0, -1); g[2] = mk(0, 1); g[3] = mk(0, 0); break;
    case QG_OP_Z: g[0] = mk(1, 0); g[1] = mk(0, 0); g[2] = mk(0, 0); g[3] = mk(-1, 0); break;
    case QG_OP_H: g[0] = mk(s2, 0); g[1] = mk(s2, 0); g[2] = mk(s2, 0); g[3] = mk(-s2, 0); break;
    case QG_OP_S: g[0] = mk(1, 0); g[1] = mk(0, 0); g[2] = mk(0, 0); g[3] = mk(0, 1); break;
    case QG_OP_SDAG: g[0] = mk(1, 0); g[1] = mk(0, 0); g[2] = mk(0, 0); g[3] = mk(0, -1); break;
    case QG_OP_T: g[0] = mk(1, 0); g[1] = mk(0, 0); g[2] = mk(0, 0); g[3] = mk(cos(M_PI / 4), sin(M_PI / 4)); break;
    case QG_OP_TDAG: g[0] = mk(1, 0); g[1] = mk(0, 0); g[2] = mk(0, 0); g[3] = mk(cos(M_PI / -4), sin(M_PI / -4)); break;
    case QG_OP_PHASE: g[0] = mk(1, 0); g[1] = mk(0, 0); g[2] = mk(0, 0); g[3] = mk(cos(angle), sin(angle)); break;
    case QG_OP_RX: {
      double c = cos(angle / 2), s = sin(angle / 2);
      g[0] = mk(c, 0); g[1] = mk(0, -s); g[2] = mk(0, -s); g[3] = mk(c, 0);
    } break;
    case QG_OP_RY: {
      double c = cos(angle / 2), s = sin(angle / 2);
      g[0] = mk(c, 0); g[1] = mk(-s, 0); g[2] = mk(s, 0); g[3] = mk(c, 0);
    } break;
    case QG_OP_RZ:
      g[0] = mk(cos(angle / -2), sin(angle / -2)); g[1] = mk(0, 0); g[2] = mk(0, 0);
      g[3] = mk(cos(angle / 2), sin(angle / 2));
      break;
    default: g[0] = mk(1, 0); g[1] = mk(0, 0); g[2] = mk(0, 0); g[3] = mk(1, 0); break;
  }
}

/* The matrix of gate_matrix as 8 doubles (re, im of m00 m01 m10 m11), for the CPU
   state-vector baseline built beside the oracle. */
void or_gate_matrix8(int opcode, double angle, double m[8]) {
  cpx g[4];
  gate_matrix(opcode, angle, g);
  for (int k = 0; k < 4; ++k) {
    m[2 * k] = g[k].re;
    m[2 * k + 1] = g[k].im;
  }
}

/* apply-single-qubit-gate (gate.clj:355-395): y_r = g_r0*x_lo + g_r1*x_hi */
static void apply_1q(double* s, int n, int q, const cpx g[4]) {
  uint64_t N = 1ULL << n, tb = 1ULL << (n - 1 - q);
  for (uint64_t i = 0; i < N; ++i) {
    if (i & tb) continue;
    cpx x0 = ld(s, i), x1 = ld(s, i | tb);
    st(s, i, cadd(cmul(g[0], x0), cmul(g[1], x1)));
    st(s, i | tb, cadd(cmul(g[2], x0), cmul(g[3], x1)));
  }
}

/* apply-controlled-gate (gate.clj:424-486): Gt applied where all control bits are 1 */
static void apply_controlled(double* s, int n, uint64_t cmask, int q, const cpx g[4]) {
  uint64_t N = 1ULL << n, tb = 1ULL << (n - 1 - q);
  for (uint64_t i = 0; i < N; ++i) {
    if ((i & tb) || (i & cmask) != cmask) continue;
    cpx x0 = ld(s, i), x1 = ld(s, i | tb);
    st(s, i, cadd(cmul(x0, g[0]), cmul(x1, g[2])));
    st(s, i | tb, cadd(cmul(x0, g[1]), cmul(x1, g[3])));
  }
}

static void apply_phase_where(double* s, int n, uint64_t mask, cpx ph) {
  uint64_t N = 1ULL << n;
  for (uint64_t i = 0; i < N; ++i)
    if ((i & mask) == mask) st(s, i, cmul(ld(s, i), ph));
}

/* swap-gate / iswap-gate with LSB bit positions (gate.clj:760-834) */
static void apply_swap_lsb(double* s, int n, int b1, int b2, int iswap) {
  uint64_t N = 1ULL << n;
  double* out = (double*)malloc(sizeof(double) * 2 * N);
  for (uint64_t i = 0; i < N; ++i) {
    uint64_t bit1 = (i >> b1) & 1, bit2 = (i >> b2) & 1;
    if (bit1 == bit2) {
      st(out, i, ld(s, i));
    } else {
      uint64_t j = i & ~(1ULL << b1) & ~(1ULL << b2);
      j |= bit2 << b1;
      j |= bit1 << b2;
      cpx v = ld(s, j);
      st(out, i, iswap ? cmul(mk(0, 1), v) : v);
    }
  }
  memcpy(s, out, sizeof(double) * 2 * N);
  free(out);
}

/* fredkin-gate (gate.clj:902-969) */
static void apply_fredkin(double* s, int n, int c, int t1, int t2) {
  uint64_t N = 1ULL << n, cb = 1ULL << (n - 1 - c), b1 = 1ULL << (n - 1 - t1), b2 = 1ULL << (n - 1 - t2);
  for (uint64_t i = 0; i < N; ++i) {
    if (!(i & cb)) continue;
    if ((i & b1) && !(i & b2)) {
      uint64_t j = (i & ~b1) | b2;
      cpx a = ld(s, i), b = ld(s, j);
      st(s, i, b);
      st(s, j, a);
    }
  }
}

/* rydberg-blockade-gate (gate.clj:1050-1096) */
static void apply_blockade(double* s, int n, uint64_t mask, cpx ph) {
  uint64_t N = 1ULL << n;
  for (uint64_t i = 0; i < N; ++i)
    if (__builtin_popcountll(i & mask) == 1) st(s, i, cmul(ld(s, i), ph));
}

/* ---- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) -------------------- */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* 64 random bits for (seed, index, stream) */
uint64_t or_draw64(uint64_t seed, uint64_t index, uint32_t stream) {
  uint32_t ctr[4] = {(uint32_t)index, (uint32_t)(index >> 32), stream, 0u};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  or_philox4x32_10(ctr, key, o);
  return ((uint64_t)o[1] << 32) | o[0];
}

static inline uint64_t mulhi64(uint64_t a, uint64_t b) { return (uint64_t)(((__uint128_t)a * b) >> 64); }

/* p -> floor(p * 2^62) */
uint64_t or_quantize(double p) {
  double v = p * 4611686018427387904.0;
  if (!(v > 0)) return 0;
  return (uint64_t)v;
}

/* The sampler's quantised chunk sums: csum[c] = sum of floor(p_i 2^62) over the chunk's
   min(2^n, 32) amplitudes, p_i = re^2 + im^2 in FP64 as in measure-state
   (state.clj:869-913); returns their total, the T a draw is scaled by. */
uint64_t or_chunk_sums(const double* s, int n, uint64_t* csum) {
  uint64_t N = 1ULL << n, ch = N < 32 ? N : 32, T = 0;
  for (uint64_t c = 0; c < N / ch; ++c) {
    uint64_t q = 0;
    for (uint64_t i = c * ch; i < (c + 1) * ch; ++i) q += or_quantize(s[2 * i] * s[2 * i] + s[2 * i + 1] * s[2 * i + 1]);
    csum[c] = q;
    T += q;
  }
  return T;
}

/* ---- measure-specific-qubits (state.clj:915-1014) ------------------------ */
int or_measure(double* s, int n, const int* qubits, int m, uint64_t seed, uint64_t draw_index,
               uint64_t* outcome_out, double* prob_out) {
  uint64_t N = 1ULL << n, nout = 1ULL << m;
  double* P = (double*)calloc(nout, sizeof(double));
  uint64_t* Q = (uint64_t*)calloc(nout, sizeof(uint64_t));
  for (uint64_t i = 0; i < N; ++i) {
    uint64_t o = 0;
    for (int k = 0; k < m; ++k) o |= ((i >> (n - 1 - qubits[k])) & 1ULL) << k;
    double re = s[2 * i], im = s[2 * i + 1];
    double p = re * re + im * im;
    P[o] += p;
    Q[o] += or_quantize(p);
  }
  uint64_t T = 0;
  for (uint64_t o = 0; o < nout; ++o) T += Q[o];
  uint64_t sel = nout - 1;
  if (T > 0) {
    uint64_t u = mulhi64(or_draw64(seed, draw_index, 1u), T), c = 0;
    for (uint64_t o = 0; o < nout; ++o) {
      c += Q[o];
      if (c > u) { sel = o; break; }
    }
  }
  double ps = P[sel];
  double nf = ps > 0 ? 1.0 / sqrt(ps) : 1.0;
  for (uint64_t i = 0; i < N; ++i) {
    uint64_t o = 0;
    for (int k = 0; k < m; ++k) o |= ((i >> (n - 1 - qubits[k])) & 1ULL) << k;
    if (o == sel) {
      s[2 * i] *= nf;
      s[2 * i + 1] *= nf;
    } else {
      s[2 * i] = 0.0;
      s[2 * i + 1] = 0.0;
    }
  }
  if (outcome_out) *outcome_out = sel;
  if (prob_out) *prob_out = ps;
  free(P);
  free(Q);
  return ORC_OK;
}

static int check_q(int n, int q) { return q >= 0 && q < n; }

/* apply one reference operation (circuit.clj:933-1112); measure_count counts
   mid-circuit measurements so each draws its own Philox stream index. */
int or_apply_op(double* s, int n, const qg_op* op, uint64_t seed, uint64_t* measure_count) {
  cpx g[4];
  int oc = op->opcode;
  switch (oc) {
    case QG_OP_X: case QG_OP_Y: case QG_OP_Z: case QG_OP_H: case QG_OP_S: case QG_OP_SDAG:
    case QG_OP_T: case QG_OP_TDAG: case QG_OP_RX: case QG_OP_RY: case QG_OP_RZ: case QG_OP_PHASE:
      if (!check_q(n, op->q[0])) return ORC_ERR;
      gate_matrix(oc, op->angle, g);
      apply_1q(s, n, op->q[0], g);
      return ORC_OK;
    case QG_OP_U:
      if (!check_q(n, op->q[0])) return ORC_ERR;
      for (int k = 0; k < 4; ++k) g[k] = mk(op->m[2 * k], op->m[2 * k + 1]);
      apply_1q(s, n, op->q[0], g);
      return ORC_OK;
    case QG_OP_KRAUS: {
      if (!check_q(n, op->q[0])) return ORC_ERR;
      for (int k = 0; k < 4; ++k) g[k] = mk(op->m[2 * k], op->m[2 * k + 1]);
      apply_1q(s, n, op->q[0], g);
      uint64_t N = 1ULL << n;
      double acc = 0.0;
      for (uint64_t i = 0; i < N; ++i) acc += s[2 * i] * s[2 * i] + s[2 * i + 1] * s[2 * i + 1];
      double norm = sqrt(acc);
      if (norm > 0 && norm > 1e-12) {
        double inv = 1.0 / norm;
        for (uint64_t i = 0; i < 2 * N; ++i) s[i] *= inv;
      }
      return ORC_OK;
    }
    case QG_OP_CNOT: case QG_OP_CZ: case QG_OP_CY: case QG_OP_CRX: case QG_OP_CRY: case QG_OP_CRZ:
    case QG_OP_RYDBERG_CZ: case QG_OP_CU: {
      int c = op->q[0], t = op->q[1];
      if (!check_q(n, c) || !check_q(n, t) || c == t) return ORC_ERR;
      int base = oc == QG_OP_CNOT ? QG_OP_X : (oc == QG_OP_CZ || oc == QG_OP_RYDBERG_CZ) ? QG_OP_Z
               : oc == QG_OP_CY ? QG_OP_Y : oc == QG_OP_CRX ? QG_OP_RX : oc == QG_OP_CRY ? QG_OP_RY : QG_OP_RZ;
      if (oc == QG_OP_CU) {
        for (int k = 0; k < 4; ++k) g[k] = mk(op->m[2 * k], op->m[2 * k + 1]);
      } else {
        gate_matrix(base, op->angle, g);
      }
      apply_controlled(s, n, 1ULL << (n - 1 - c), t, g);
      return ORC_OK;
    }
    case QG_OP_RYDBERG_CPHASE: {
      int c = op->q[0], t = op->q[1];
      if (!check_q(n, c) || !check_q(n, t)) return ORC_ERR;
      apply_phase_where(s, n, (1ULL << (n - 1 - c)) | (1ULL << (n - 1 - t)), mk(cos(op->angle), sin(op->angle)));
      return ORC_OK;
    }
    case QG_OP_RZZ: {
      int a = op->q[0], b = op->q[1];
      if (!check_q(n, a) || !check_q(n, b) || a == b) return ORC_ERR;
      uint64_t N = 1ULL << n, ba = 1ULL << (n - 1 - a), bb = 1ULL << (n - 1 - b);
      cpx even = mk(cos(op->angle / -2), sin(op->angle / -2)), odd = mk(cos(op->angle / 2), sin(op->angle / 2));
      for (uint64_t i = 0; i < N; ++i) {
        int par = (!!(i & ba)) ^ (!!(i & bb));
        st(s, i, cmul(ld(s, i), par ? odd : even));
      }
      return ORC_OK;
    }
    case QG_OP_SWAP: case QG_OP_ISWAP: {
      int b1 = op->q[0], b2 = op->q[1];
      if (!check_q(n, b1) || !check_q(n, b2)) return ORC_ERR;
      apply_swap_lsb(s, n, b1, b2, oc == QG_OP_ISWAP);
      return ORC_OK;
    }
    case QG_OP_TOFFOLI: {
      int c1 = op->q[0], c2 = op->q[1], t = op->q[2];
      if (!check_q(n, c1) || !check_q(n, c2) || !check_q(n, t) || c1 == c2 || c1 == t || c2 == t) return ORC_ERR;
      gate_matrix(QG_OP_X, 0, g);
      apply_controlled(s, n, (1ULL << (n - 1 - c1)) | (1ULL << (n - 1 - c2)), t, g);
      return ORC_OK;
    }
    case QG_OP_FREDKIN: {
      int c = op->q[0], t1 = op->q[1], t2 = op->q[2];
      if (!check_q(n, c) || !check_q(n, t1) || !check_q(n, t2) || c == t1 || c == t2 || t1 == t2) return ORC_ERR;
      apply_fredkin(s, n, c, t1, t2);
      return ORC_OK;
    }
    case QG_OP_RYDBERG_BLOCKADE: {
      uint64_t mask = 0;
      if (op->nq < 1) return ORC_ERR;
      for (int k = 0; k < op->nq; ++k) {
        if (!check_q(n, op->q[k])) return ORC_ERR;
        uint64_t b = 1ULL << (n - 1 - op->q[k]);
        if (mask & b) return ORC_ERR;
        mask |= b;
      }
      apply_blockade(s, n, mask, mk(cos(op->angle), sin(op->angle)));
      return ORC_OK;
    }
    case QG_OP_GLOBAL_RX: case QG_OP_GLOBAL_RY: case QG_OP_GLOBAL_RZ: case QG_OP_GLOBAL_H:
    case QG_OP_GLOBAL_X: case QG_OP_GLOBAL_Y: case QG_OP_GLOBAL_Z: {
      int base = (oc == QG_OP_GLOBAL_RX || oc == QG_OP_GLOBAL_X) ? QG_OP_RX
               : (oc == QG_OP_GLOBAL_RY || oc == QG_OP_GLOBAL_Y) ? QG_OP_RY
               : (oc == QG_OP_GLOBAL_RZ || oc == QG_OP_GLOBAL_Z) ? QG_OP_RZ : QG_OP_H;
      double ang = (oc == QG_OP_GLOBAL_X || oc == QG_OP_GLOBAL_Y || oc == QG_OP_GLOBAL_Z) ? M_PI : op->angle;
      gate_matrix(base, ang, g);
      for (int q = 0; q < n; ++q) apply_1q(s, n, q, g);
      return ORC_OK;
    }
    case QG_OP_MEASURE: {
      int qs[QG_MAX_OP_QUBITS];
      if (op->nq < 1 || op->nq > 20) return ORC_ERR;
      for (int k = 0; k < op->nq; ++k) {
        if (!check_q(n, op->q[k])) return ORC_ERR;
        qs[k] = op->q[k];
      }
      uint64_t idx = (*measure_count)++;
      return or_measure(s, n, qs, op->nq, seed, idx, NULL, NULL);
    }
    default:
      return ORC_ERR; /* :i and anything unknown: "Unknown gate type" */
  }
}

/* Run a whole circuit in place. Returns the index of the failing op + 1, or 0. */
int or_run_circuit(double* s, int n, const qg_op* ops, int nops, uint64_t seed) {
  uint64_t mc = 0;
  for (int k = 0; k < nops; ++k)
    if (or_apply_op(s, n, &ops[k], seed, &mc) != ORC_OK) return k + 1;
  return 0;
}

void or_zero_state(double* s, int n) {
  memset(s, 0, sizeof(double) * 2 * (1ULL << n));
  s[0] = 1.0;
}

void or_probabilities(const double* s, int n, double* p) {
  uint64_t N = 1ULL << n;
  for (uint64_t i = 0; i < N; ++i) p[i] = s[2 * i] * s[2 * i] + s[2 * i + 1] * s[2 * i + 1];
}

/* measure-state repeated `shots` times (result.clj:224, state.clj:869-913).
   Returns 1 (and samples nothing) when |sum p - 1| > 1e-8, like state.clj:901. */
int or_sample(const double* s, int n, uint64_t shots, uint64_t seed, uint64_t* outcomes) {
  uint64_t N = 1ULL << n;
  uint64_t* C = (uint64_t*)malloc(sizeof(uint64_t) * N);
  double tot = 0.0;
  uint64_t acc = 0;
  for (uint64_t i = 0; i < N; ++i) {
    double p = s[2 * i] * s[2 * i] + s[2 * i + 1] * s[2 * i + 1];
    tot += p;
    acc += or_quantize(p);
    C[i] = acc;
  }
  if (fabs(tot - 1.0) > 1e-8) { free(C); return 1; }
  uint64_t T = acc;
  for (uint64_t j = 0; j < shots; ++j) {
    uint64_t u = mulhi64(or_draw64(seed, j, 0u), T);
    uint64_t lo = 0, hi = N - 1;
    while (lo < hi) { /* first i with C[i] > u */
      uint64_t mid = lo + (hi - lo) / 2;
      if (C[mid] > u) hi = mid; else lo = mid + 1;
    }
    outcomes[j] = lo;
  }
  free(C);
  return 0;
}

/* One outcome of a normalised state for the draw (seed, index, stream): the first i
   whose cumulative quantised probability exceeds floor(r64 T / 2^64) (measure-state,
   state.clj:869-913, with the sampler's integer prefix sums). */
uint64_t or_sample_one(const double* s, int n, uint64_t seed, uint64_t index, uint32_t stream) {
  uint64_t N = 1ULL << n, T = 0;
  for (uint64_t i = 0; i < N; ++i) T += or_quantize(s[2 * i] * s[2 * i] + s[2 * i + 1] * s[2 * i + 1]);
  if (T == 0) return 0;
  uint64_t u = mulhi64(or_draw64(seed, index, stream), T), c = 0;
  for (uint64_t i = 0; i < N; ++i) {
    c += or_quantize(s[2 * i] * s[2 * i] + s[2 * i + 1] * s[2 * i + 1]);
    if (c > u) return i;
  }
  return N - 1;
}

/* Re<psi|P|psi> with the explicit Pauli action (observables.clj:216-251) */
double or_pauli_expectation(const double* s, int n, const char* pauli) {
  uint64_t N = 1ULL << n, xm = 0, zm = 0;
  int ny = 0;
  for (int q = 0; q < n; ++q) {
    uint64_t b = 1ULL << (n - 1 - q);
    char c = pauli[q];
    if (c == 'X') xm |= b;
    else if (c == 'Y') { xm |= b; zm |= b; ny++; }
    else if (c == 'Z') zm |= b;
  }
  /* (P psi)_i = (-i)^ny (-1)^popc(i & zm) psi_{i^xm} */
  cpx yph = mk(1, 0);
  for (int k = 0; k < (ny & 3); ++k) yph = cmul(yph, mk(0, -1));
  double acc = 0.0;
  for (uint64_t i = 0; i < N; ++i) {
    cpx a = ld(s, i), b = ld(s, i ^ xm);
    cpx pb = cmul(yph, b);
    if (__builtin_popcountll(i & zm) & 1) { pb.re = -pb.re; pb.im = -pb.im; }
    acc += a.re * pb.re + a.im * pb.im;
  }
  return acc;
}

/* Re<psi|O_t|psi> for a 2x2 observable on one qubit (result.clj:254-288) */
double or_expectation_1q(const double* s, int n, const double* o8, int t) {
  uint64_t N = 1ULL << n, tb = 1ULL << (n - 1 - t);
  cpx o[4];
  for (int k = 0; k < 4; ++k) o[k] = mk(o8[2 * k], o8[2 * k + 1]);
  double acc = 0.0;
  for (uint64_t i = 0; i < N; ++i) {
    if (i & tb) continue;
    cpx x0 = ld(s, i), x1 = ld(s, i | tb);
    cpx y0 = cadd(cmul(o[0], x0), cmul(o[1], x1));
    cpx y1 = cadd(cmul(o[2], x0), cmul(o[3], x1));
    acc += x0.re * y0.re + x0.im * y0.im + x1.re * y1.re + x1.im * y1.im;
  }
  return acc;
}

/* <a|b> (complex_linear_algebra.clj:318) */
void or_inner(const double* a, const double* b, int n, double* re, double* im) {
  uint64_t N = 1ULL << n;
  double r = 0, m = 0;
  for (uint64_t i = 0; i < N; ++i) {
    cpx x = ld(a, i), y = ld(b, i);
    r += x.re * y.re + x.im * y.im;
    m += x.re * y.im - x.im * y.re;
  }
  *re = r;
  *im = m;
}

/* ---- the reference ALGORITHM, for CPU timing ------------------------------
 * Rows [r0, r0+nr) of (I x .. x G x .. x I) x, visiting every column of each row
 * as the dense Kronecker mat-vec of gate.clj:346-395 does (one complex multiply
 * and add per matrix entry, zeros included). O(2^n) work per output amplitude. */
void or_refalgo_rows(const double* x, int n, const double* g8, int target, uint64_t r0, uint64_t nr, double* y) {
  uint64_t N = 1ULL << n, tb = 1ULL << (n - 1 - target);
  cpx g[4];
  for (int k = 0; k < 4; ++k) g[k] = mk(g8[2 * k], g8[2 * k + 1]);
  for (uint64_t r = r0; r < r0 + nr; ++r) {
    cpx acc = mk(0, 0);
    int rb = (r & tb) ? 1 : 0;
    for (uint64_t c = 0; c < N; ++c) {
      cpx m;
      if ((r ^ c) & ~tb) m = mk(0, 0);
      else m = g[rb * 2 + ((c & tb) ? 1 : 0)];
      acc = cadd(acc, cmul(m, ld(x, c)));
    }
    st(y, r - r0, acc);
  }
}

/* A whole circuit run the way the reference runs it, for CPU timing of config-0 sized
 * jobs: every single-qubit gate as the dense Kronecker mat-vec above (gate.clj:346-395,
 * all 2^n x 2^n entries visited, into a fresh output vector as the reference builds a
 * new one), every other operation with the O(2^n) loops of or_apply_op (gate.clj:424-486
 * and the permutation gates); then `shots` shots, each the reference's measure-state
 * (state.clj:869-913): the full probability vector, its running sums and a scan for the
 * first cumulative sum >= u, with u drawn from Philox (the reference draws `rand`).
 * The final state equals or_run_circuit's bit for bit (the dense row adds exact zeros).
 * Returns 0, 1 + the index of a failing operation, or -1 when the state is not
 * normalised for sampling. */
int or_refalgo_circuit(double* s, int n, const qg_op* ops, int nops, uint64_t shots, uint64_t seed,
                       uint64_t* outcomes) {
  uint64_t N = 1ULL << n, mc = 0;
  double* y = (double*)malloc(sizeof(double) * 2 * N);
  double* cum = (double*)malloc(sizeof(double) * N);
  if (!y || !cum) { free(y); free(cum); return -1; }
  for (int k = 0; k < nops; ++k) {
    const qg_op* op = &ops[k];
    int oc = op->opcode;
    int oneq = oc == QG_OP_X || oc == QG_OP_Y || oc == QG_OP_Z || oc == QG_OP_H || oc == QG_OP_S ||
               oc == QG_OP_SDAG || oc == QG_OP_T || oc == QG_OP_TDAG || oc == QG_OP_RX || oc == QG_OP_RY ||
               oc == QG_OP_RZ || oc == QG_OP_PHASE;
    if (oneq) {
      if (!check_q(n, op->q[0])) { free(y); free(cum); return k + 1; }
      cpx g[4];
      double g8[8];
      gate_matrix(oc, op->angle, g);
      for (int j = 0; j < 4; ++j) { g8[2 * j] = g[j].re; g8[2 * j + 1] = g[j].im; }
      or_refalgo_rows(s, n, g8, op->q[0], 0, N, y);
      memcpy(s, y, sizeof(double) * 2 * N);
    } else if (or_apply_op(s, n, op, seed, &mc) != ORC_OK) {
      free(y);
      free(cum);
      return k + 1;
    }
  }
  for (uint64_t j = 0; j < shots; ++j) {
    double tot = 0.0;
    for (uint64_t i = 0; i < N; ++i) {
      tot += s[2 * i] * s[2 * i] + s[2 * i + 1] * s[2 * i + 1];
      cum[i] = tot;
    }
    if (fabs(tot - 1.0) > 1e-8) { free(y); free(cum); return -1; }
    double u = (double)(or_draw64(seed, j, 0u) >> 11) * 0x1.0p-53 * tot;
    uint64_t c = 0;
    for (uint64_t i = 0; i < N; ++i) c += cum[i] < u;
    outcomes[j] = c < N ? c : N - 1;
  }
  free(y);
  free(cum);
  return 0;
}
