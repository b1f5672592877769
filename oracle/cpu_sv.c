/*
 * cpu_sv.c - an optimised CPU state-vector simulator, for the benchmark's "not the
 * reference" CPU figure only.
 *
 * TEST INFRASTRUCTURE ONLY, like the oracle it is built beside: only the CPU-baseline leg
 * of bench.py and the tests load it; the product library never links it. It is not the
 * reference's algorithm (that is the dense Kronecker mat-vec restated in qgo.c): it applies
 * each gate as one in-place pass over the state on all host cores (OpenMP), with the
 * oracle's gate matrices and operand conventions (controlled gates apply the transpose,
 * SWAP operands are LSB bit positions), so its results agree with the oracle's.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/qgpu.h"

/* from qgo.c, compiled into the same library */
void or_gate_matrix8(int opcode, double angle, double m[8]);

static inline void cmac2(const double* g, double xr0, double xi0, double xr1, double xi1, double* yr, double* yi) {
  /* y = g0 x0 + g1 x1, rounded like the oracle's cadd(cmul(g0, x0), cmul(g1, x1)) (qgo.c apply_1q):
     each complex product first, then the two sums */
  *yr = (g[0] * xr0 - g[1] * xi0) + (g[2] * xr1 - g[3] * xi1);
  *yi = (g[0] * xi0 + g[1] * xr0) + (g[2] * xi1 + g[3] * xr1);
}

/* k with a zero bit inserted at each position of `bits` (ascending, at most 3) */
static inline uint64_t spread(uint64_t k, const int* bits, int nb) {
  for (int j = 0; j < nb; ++j) {
    const uint64_t lo = k & ((1ULL << bits[j]) - 1);
    k = ((k >> bits[j]) << (bits[j] + 1)) | lo;
  }
  return k;
}

/* rows r0 = (m00, m01), r1 = (m10, m11) applied to pairs (i0, i0 | tb) where i0 & cmask == cmask
   (cmask: at most one bit); only the pairs that match are visited */
static void pass_2x2(double* s, int n, int bit, uint64_t cmask, const double r0[4], const double r1[4]) {
  const uint64_t tb = 1ULL << bit;
  int bits[2], nb = 0;
  if (cmask) {
    const int cb = __builtin_ctzll(cmask);
    bits[0] = cb < bit ? cb : bit;
    bits[1] = cb < bit ? bit : cb;
    nb = 2;
  } else {
    bits[0] = bit;
    nb = 1;
  }
  const uint64_t cnt = (1ULL << n) >> nb;
#pragma omp parallel for schedule(static)
  for (uint64_t k = 0; k < cnt; ++k) {
    const uint64_t i0 = spread(k, bits, nb) | cmask;
    const uint64_t i1 = i0 | tb;
    const double xr0 = s[2 * i0], xi0 = s[2 * i0 + 1], xr1 = s[2 * i1], xi1 = s[2 * i1 + 1];
    double yr, yi;
    cmac2(r0, xr0, xi0, xr1, xi1, &yr, &yi);
    s[2 * i0] = yr;
    s[2 * i0 + 1] = yi;
    cmac2(r1, xr0, xi0, xr1, xi1, &yr, &yi);
    s[2 * i1] = yr;
    s[2 * i1 + 1] = yi;
  }
}

/* amp *= (pr + i pi) where all bits of mask (two bits) are set, like the oracle's
   cmul(amp, ph) (qgo.c apply_phase_where) */
static void pass_phase(double* s, int n, uint64_t mask, double pr, double pi) {
  int bits[2];
  bits[0] = __builtin_ctzll(mask);
  bits[1] = 63 - __builtin_clzll(mask);
  const int nb = bits[0] == bits[1] ? 1 : 2;
  const uint64_t cnt = (1ULL << n) >> nb;
#pragma omp parallel for schedule(static)
  for (uint64_t k = 0; k < cnt; ++k) {
    const uint64_t i = spread(k, bits, nb) | mask;
    const double ar = s[2 * i], ai = s[2 * i + 1];
    s[2 * i] = ar * pr - ai * pi;
    s[2 * i + 1] = ar * pi + ai * pr;
  }
}

/* exchange amplitudes whose bits b1, b2 differ (each pair once) */
static void pass_swap(double* s, int n, int b1, int b2) {
  if (b1 == b2) return;
  const uint64_t N = 1ULL << n, m1 = 1ULL << b1, m2 = 1ULL << b2;
#pragma omp parallel for schedule(static)
  for (uint64_t i = 0; i < N; ++i) {
    if ((i & m1) && !(i & m2)) {
      const uint64_t j = (i & ~m1) | m2;
      const double r = s[2 * i], im = s[2 * i + 1];
      s[2 * i] = s[2 * j];
      s[2 * i + 1] = s[2 * j + 1];
      s[2 * j] = r;
      s[2 * j + 1] = im;
    }
  }
}

/* Run the gates of a circuit in place; returns 0, or 1 + the index of the first
   operation this baseline does not implement. */
int sv_run_circuit(double* s, int n, const qg_op* ops, int nops) {
  double m[8];
  for (int k = 0; k < nops; ++k) {
    const qg_op* op = &ops[k];
    const int oc = op->opcode;
    switch (oc) {
      case QG_OP_X: case QG_OP_Y: case QG_OP_Z: case QG_OP_H: case QG_OP_S: case QG_OP_SDAG:
      case QG_OP_T: case QG_OP_TDAG: case QG_OP_RX: case QG_OP_RY: case QG_OP_RZ: case QG_OP_PHASE:
      case QG_OP_U: {
        if (oc == QG_OP_U) memcpy(m, op->m, sizeof(m));
        else or_gate_matrix8(oc, op->angle, m);
        const double r0[4] = {m[0], m[1], m[2], m[3]}, r1[4] = {m[4], m[5], m[6], m[7]};
        pass_2x2(s, n, n - 1 - op->q[0], 0, r0, r1);
      } break;
      case QG_OP_CNOT: case QG_OP_CZ: case QG_OP_CY: case QG_OP_CRX: case QG_OP_CRY: case QG_OP_CRZ:
      case QG_OP_RYDBERG_CZ: {
        const int base = oc == QG_OP_CNOT ? QG_OP_X : (oc == QG_OP_CZ || oc == QG_OP_RYDBERG_CZ) ? QG_OP_Z
                         : oc == QG_OP_CY ? QG_OP_Y : oc == QG_OP_CRX ? QG_OP_RX : oc == QG_OP_CRY ? QG_OP_RY
                                                                                 : QG_OP_RZ;
        or_gate_matrix8(base, op->angle, m);
        /* the transpose: y0 = x0 g00 + x1 g10, y1 = x0 g01 + x1 g11 */
        const double r0[4] = {m[0], m[1], m[4], m[5]}, r1[4] = {m[2], m[3], m[6], m[7]};
        pass_2x2(s, n, n - 1 - op->q[1], 1ULL << (n - 1 - op->q[0]), r0, r1);
      } break;
      case QG_OP_RYDBERG_CPHASE:
        pass_phase(s, n, (1ULL << (n - 1 - op->q[0])) | (1ULL << (n - 1 - op->q[1])), cos(op->angle),
                   sin(op->angle));
        break;
      case QG_OP_SWAP:
        pass_swap(s, n, op->q[0], op->q[1]);
        break;
      default:
        return k + 1;
    }
  }
  return 0;
}

int sv_threads(void) {
#ifdef _OPENMP
  extern int omp_get_max_threads(void);
  return omp_get_max_threads();
#else
  return 1;
#endif
}
