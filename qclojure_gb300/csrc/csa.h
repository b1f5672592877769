// Carry-save counting of one-bit vectors (host side of the pass-kernel generator).
//
// A parity run in table form (the sweep kernels) adds E words v_0 .. v_{E-1}, bit j of
// v_e being 1 when op e's parity is odd for register j, into bit planes: plane p holds
// bit p of every register's count (the count selects the run's phase). Adding each
// word into the planes with a ripple carry costs two operations per plane per word.
// Here the words go through a streaming carry-save counter instead: each weight keeps
// at most two pending words, and a third arriving word triggers a full adder (sum
// a ^ b ^ c stays, the majority carries to the next weight), so E words cost about E
// full adders in all. At the end, half adders bring every weight down to one word,
// which is that plane. Counts never exceed E < 2^planes, so a carry into weight
// `planes` is zero and is not formed.
//
// csa_plan returns the schedule as abstract operations on numbered words, which the
// generator prints as CUDA and tests/test_csa.py executes on the CPU against direct
// counts.
#pragma once

#include <vector>

namespace qg {

struct CsaOp {
  enum Kind { IN, FULL, HALF } kind;
  int a, b, c;  // IN: a = the input's index; FULL: three words; HALF: a, b
  int s, cy;    // result words: the sum (IN: the input word) and the carry (-1: not formed)
};

struct CsaPlan {
  std::vector<CsaOp> ops;
  std::vector<int> planes;  // word of plane p, -1 for a plane that is zero
  int words = 0;
};

inline CsaPlan csa_plan(int inputs, int planes) {
  CsaPlan p;
  std::vector<std::vector<int>> pend((size_t)planes);
  struct Adder {
    CsaPlan& p;
    std::vector<std::vector<int>>& pend;
    int planes;
    void add(int w, int word) {
      if (w >= planes) return;  // provably zero
      pend[w].push_back(word);
      if (pend[w].size() == 3) {
        CsaOp o{CsaOp::FULL, pend[w][0], pend[w][1], pend[w][2], p.words++, -1};
        if (w + 1 < planes) o.cy = p.words++;
        p.ops.push_back(o);
        pend[w].assign(1, o.s);
        if (o.cy >= 0) add(w + 1, o.cy);
      }
    }
  } ad{p, pend, planes};
  for (int e = 0; e < inputs; ++e) {
    const CsaOp in{CsaOp::IN, e, -1, -1, p.words++, -1};
    p.ops.push_back(in);
    ad.add(0, in.s);
  }
  for (int w = 0; w < planes; ++w) {
    if (pend[w].size() == 2) {
      CsaOp o{CsaOp::HALF, pend[w][0], pend[w][1], -1, p.words++, -1};
      if (w + 1 < planes) o.cy = p.words++;
      p.ops.push_back(o);
      pend[w].assign(1, o.s);
      if (o.cy >= 0) ad.add(w + 1, o.cy);
    }
    p.planes.push_back(pend[w].empty() ? -1 : pend[w][0]);
  }
  return p;
}

}  // namespace qg
