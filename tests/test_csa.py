"""The carry-save counting schedule of the pass-kernel generator (qclojure_gb300/csrc/csa.h),
executed on the CPU: for 1 to 100 one-bit words of 32 lanes (random, all ones, all zeros),
the planes it leaves must hold every lane's count, and it must use at most one adder per
word plus one per plane."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

PROGRAM = r'''
#include <cstdint>
#include <cstdio>
#include <random>
#include <vector>
#include "csa.h"

int main() {
  std::mt19937 rng(5);
  long bad = 0;
  for (int E = 1; E <= 100; ++E) {
    int planes = 0;
    while ((1 << planes) <= E) ++planes;
    const qg::CsaPlan plan = qg::csa_plan(E, planes);
    int adders = 0;
    for (const auto& o : plan.ops) adders += o.kind != qg::CsaOp::IN;
    if (adders > E + planes) {
      std::printf("E=%d: %d adders\n", E, adders);
      ++bad;
    }
    for (int trial = 0; trial < 40; ++trial) {
      std::vector<uint32_t> in(E), w(plan.words, 0xDEADBEEFu);
      for (int e = 0; e < E; ++e) in[e] = trial == 0 ? 0xFFFFFFFFu : trial == 1 ? 0u : (uint32_t)rng();
      for (const auto& o : plan.ops) {
        if (o.kind == qg::CsaOp::IN) {
          w[o.s] = in[o.a];
        } else if (o.kind == qg::CsaOp::FULL) {
          const uint32_t a = w[o.a], b = w[o.b], c = w[o.c];
          w[o.s] = a ^ b ^ c;
          if (o.cy >= 0) w[o.cy] = (a & b) | (c & (a ^ b));
        } else {
          const uint32_t a = w[o.a], b = w[o.b];
          w[o.s] = a ^ b;
          if (o.cy >= 0) w[o.cy] = a & b;
        }
      }
      for (int lane = 0; lane < 32; ++lane) {
        int want = 0, got = 0;
        for (int e = 0; e < E; ++e) want += (in[e] >> lane) & 1;
        for (int p = 0; p < planes; ++p)
          if (plan.planes[p] >= 0) got |= (int)((w[plan.planes[p]] >> lane) & 1) << p;
        if (got != want) {
          if (bad < 5) std::printf("E=%d lane %d: %d vs %d\n", E, lane, got, want);
          ++bad;
        }
      }
    }
  }
  std::printf(bad ? "MISMATCHES %ld\n" : "ok\n", bad);
  return bad ? 1 : 0;
}
'''


def test_csa_schedule_counts(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    src = tmp_path / "csa_check.cpp"
    exe = tmp_path / "csa_check"
    src.write_text(PROGRAM)
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(ROOT / "qclojure_gb300" / "csrc"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip().endswith("ok"), out.stdout
