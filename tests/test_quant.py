"""The sampler's integer probability helpers (qclojure_gb300/csrc/quant.cuh) against the FP64
expressions they replace, bit for bit: the quantisation floor(p 2^62) and the exact
square of a float as a double. The header is compiled for the host with FP contraction
off (as the oracle is), over random inputs (uniform, log-uniform, raw float bit patterns)
and edge cases (zero, subnormals, the 2^-62 boundary, one, values just below 4), and the
fixed-point fast path for complex64 and complex128 parts: wherever its guard lets it answer,
bit for bit the FP64 expression, including sums placed on grid points of 2^-62."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

PROGRAM = r'''
#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdint>
#include <random>
#include "quant.cuh"

static uint64_t ref_quant(double p) {
  double v = p * 4611686018427387904.0;
  return v > 0 ? (uint64_t)v : 0ULL;
}
static int check_q(double p, long* bad) {
  if (qg_quant62(p) != ref_quant(p)) {
    if (*bad < 5) std::printf("quant %.17g: %llu vs %llu\n", p, (unsigned long long)qg_quant62(p),
                              (unsigned long long)ref_quant(p));
    ++*bad;
  }
  return 0;
}
static int check_s(float x, long* bad) {
  const double r = (double)x * (double)x, g = qg_sq_float(x);
  if (std::memcmp(&r, &g, 8) != 0) {
    if (*bad < 5) std::printf("square %.9g: %.17g vs %.17g\n", x, g, r);
    ++*bad;
  }
  return 0;
}
int main() {
  long bad = 0;
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> u01(0.0, 1.0), u04(0.0, 3.999999);
  std::uniform_real_distribution<double> lg(-70.0, 1.9);
  // quantisation
  const double edge[] = {0.0, -0.0, 1.0, 2.0, 3.9999999999999996, 0x1p-62, 0x1p-63, 0x1.fffffffffffffp-62,
                         0x1.0000000000001p-62, 0x1p-61, 0x1p-1022, 0x1p-1074, 0.5, 0.25, 1.0 - 0x1p-53, -1.0};
  for (double p : edge) check_q(p, &bad);
  for (long i = 0; i < 4000000; ++i) {
    check_q(u01(rng), &bad);
    check_q(u04(rng), &bad);
    check_q(std::exp2(lg(rng)), &bad);
  }
  // squares of floats: random bit patterns (all exponents, subnormals included) and edges
  const float fedge[] = {0.0f, -0.0f, 1.0f, -1.0f, 0x1p-149f, 0x1p-126f, 0x1.fffffep-127f, 0x1.fffffep127f,
                         0.70710677f, 1e-20f, 3.4e38f};
  for (float x : fedge) check_s(x, &bad);
  for (long i = 0; i < 8000000; ++i) {
    uint32_t b = (uint32_t)rng();
    if (((b >> 23) & 0xFF) == 0xFF) b &= ~(1u << 30);  // finite
    float x;
    std::memcpy(&x, &b, 4);
    check_s(x, &bad);
    check_s((float)u01(rng), &bad);
  }
  // the combination the complex64 probabilities use: one rounded FP64 sum
  for (long i = 0; i < 2000000; ++i) {
    // amplitudes of magnitude at most 1, so p stays below 4 (the host conversion's range)
    const float a = (float)(u01(rng) - 0.5), b = (float)(std::exp2(lg(rng) - 2.0) * (i & 1 ? 1 : -1));
    const double r = (double)a * (double)a + (double)b * (double)b, g = qg_sq_float(a) + qg_sq_float(b);
    if (std::memcmp(&r, &g, 8) != 0) ++bad;
    check_q(g, &bad);
  }
  // the fixed-point fast path: whenever it answers, its value is the FP64 expression's
  long fast = 0, total = 0;
  auto chk_f = [&](float a, float b) {
    const double r = (double)a * (double)a + (double)b * (double)b;
    uint64_t q;
    ++total;
    if (qg_quant62_sq_fast(a, b, &q)) {
      ++fast;
      if (q != ref_quant(r)) {
        if (bad < 5) std::printf("fast f %a %a: %llu vs %llu\n", a, b, (unsigned long long)q,
                                 (unsigned long long)ref_quant(r));
        ++bad;
      }
    }
  };
  auto chk_d = [&](double a, double b) {
    const double r = a * a + b * b;
    uint64_t q;
    ++total;
    if (qg_quant62_sq_fast(a, b, &q)) {
      ++fast;
      if (q != ref_quant(r)) {
        if (bad < 5) std::printf("fast d %a %a: %llu vs %llu\n", a, b, (unsigned long long)q,
                                 (unsigned long long)ref_quant(r));
        ++bad;
      }
    }
  };
  std::uniform_real_distribution<double> lgp(-45.0, -8.0), sgn(-1.0, 1.0);
  for (long i = 0; i < 3000000; ++i) {  // parts of every magnitude around the fast range
    const double a = std::exp2(lgp(rng)) * (sgn(rng) < 0 ? -1 : 1), b = std::exp2(lgp(rng)) * (sgn(rng) < 0 ? -1 : 1);
    chk_d(a, b);
    chk_f((float)a, (float)b);
    chk_d(a, 0.0);
    chk_f((float)b, 0.0f);
  }
  // sums placed on a grid point of 2^-62 (the guard's boundary): im chosen so that
  // re^2 + im^2 lands within rounding of Q 2^-62
  std::uniform_int_distribution<int> lq(10, 50);
  for (long i = 0; i < 3000000; ++i) {
    const double Q = (i & 3) ? std::floor(std::exp2((double)lq(rng)) * (1.0 + u01(rng))) : std::exp2((double)lq(rng));
    const double pt = std::ldexp(Q, -62);
    const double re = std::sqrt(pt) * u01(rng);
    const double im = std::sqrt(pt - re * re);
    chk_d(re, im);
    chk_d(-im, re);
    chk_d(std::nextafter(im, 1.0), re);
    chk_d(std::nextafter(im, 0.0), re);
    const float rf = (float)re, imf = (float)std::sqrt(pt - (double)rf * (double)rf);
    chk_f(rf, imf);
    chk_f(std::nextafterf(imf, 1.0f), rf);
    chk_f(std::nextafterf(imf, 0.0f), -rf);
  }
  const double fedge2[] = {0.0, -0.0, 0x1p-11, 0x1.fffffffffffffp-11, 0x1p-10, 0x1p-31, 0x1p-41, 0x1p-600, 0x1p-1074,
                           0x1.6a09e667f3bcdp-21, INFINITY, NAN};
  for (double a : fedge2)
    for (double b : fedge2) {
      chk_d(a, b);
      chk_f((float)a, (float)b);
    }
  // zeros and tiny parts take the fast path (a zero sum has no lower margin to keep)
  {
    uint64_t q = 1;
    const float fz[] = {0.0f, -0.0f, 0x1p-149f, 0x1p-60f};
    const double dz[] = {0.0, -0.0, 0x1p-1074, 0x1p-60};
    for (float a : fz)
      for (float b : fz) {
        if (!qg_quant62_sq_fast(a, b, &q) || q != 0) ++bad;
        if (qg_part_big(a)) ++bad;
      }
    for (double a : dz)
      for (double b : dz) {
        if (!qg_quant62_sq_fast(a, b, &q) || q != 0) ++bad;
        if (qg_part_big(a)) ++bad;
      }
    if (bad) std::printf("zeros not on the fast path\n");
  }
  // the group test agrees with the fast path's own range flag on finite parts
  for (long i = 0; i < 1000000; ++i) {
    const double a = std::exp2(lgp(rng)) * (sgn(rng) < 0 ? -1 : 1);
    bool bd, bf;
    qg_sq_fix(a, &bd);
    qg_sq_fix((float)a, &bf);
    if (bd != qg_part_big(a) || bf != qg_part_big((float)a)) {
      if (bad < 5) std::printf("range flag %a\n", a);
      ++bad;
    }
  }
  // states of 20 and more qubits: parts about 2^-11 and smaller take the fast path
  long fast_typ = 0, tot_typ = 0;
  std::normal_distribution<double> nd(0.0, std::exp2(-16.0));
  for (long i = 0; i < 1000000; ++i) {
    const double a = nd(rng), b = nd(rng);
    uint64_t q;
    tot_typ += 2;
    fast_typ += qg_quant62_sq_fast(a, b, &q) + qg_quant62_sq_fast((float)a, (float)b, &q);
    chk_d(a, b);
    chk_f((float)a, (float)b);
  }
  std::printf("fast %ld of %ld; typical %ld of %ld\n", fast, total, fast_typ, tot_typ);
  if (tot_typ - fast_typ > tot_typ / 10000) {
    std::printf("too many fallbacks at 2^-16\n");
    ++bad;
  }
  std::printf(bad ? "MISMATCHES %ld\n" : "ok\n", bad);
  return bad ? 1 : 0;
}
'''


def test_quant_helpers_match_fp64(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "quant_check.cpp"
    exe = tmp_path / "quant_check"
    src.write_text(PROGRAM)
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(ROOT / "qclojure_gb300" / "csrc"),
                    str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0 and out.stdout.strip().endswith("ok"), out.stdout
