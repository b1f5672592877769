"""The sampler's integer probability helpers (qclojure_gb300/csrc/quant.cuh) against the FP64
expressions they replace, bit for bit: the quantisation floor(p 2^62) and the exact
square of a float as a double. The header is compiled for the host with FP contraction
off (as the oracle is), over random inputs (uniform, log-uniform, raw float bit patterns)
and edge cases (zero, subnormals, the 2^-62 boundary, one, values just below 4)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

PROGRAM = r'''
#include <cmath>
#include <cstdio>
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
