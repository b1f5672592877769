// Noisy trajectories: the hardware simulator's shot loop as batched device states.
//
// The reference (adapter/backend/hardware_simulator.clj:84-193) runs every shot as a
// fresh pass over the circuit: after each operation whose :operation-type has a
// gate-noise entry it applies one Kraus operator of that entry's channel to the
// operation's :target (noise.clj:53-102), drawn with probabilities max_ij |K_ij|^2
// (channel.clj:194-232), renormalising after every operator (channel.clj:127-171);
// the shot ends with one sampled outcome and readout noise (noise.clj:107-202).
//
// The draws here depend only on (seed, shot, site), never on the state, so every
// trajectory is the same program with different Kraus matrices: the circuit with one
// QG_OP_KRAUS per noise site is compiled once into tiled passes, and a batch of
// trajectories runs as one launch per pass over all its states, each state reading its
// own op records (the template's records with the chosen operators patched in); shots
// with equal choices share one state. The
// renormalisations are deferred to the end of the shot (every operator is linear, so
// the final direction is the same) and done by the kernel that also samples the shot.
// States of fewer than 5 qubits run padded with idle low qubits, which stay |0>.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "qgpu_internal.h"

namespace qg {
namespace {

constexpr uint32_t kStreamMeasure = 2u;           // the shot's outcome
constexpr uint32_t kStreamReadout = 0x20000000u;  // + qubit: readout flips
constexpr uint32_t kStreamKraus = 0x40000000u;    // + site: Kraus operator choice
constexpr int kMinQubits = 5;                     // tiled passes need 2^5 amplitudes per tile
constexpr double kNormTolerance = 1e-12;          // normalize-state leaves smaller norms alone

double uniform01(uint64_t x) { return (double)(x >> 11) * 0x1p-53; }

struct Channel {
  bool built = false;
  std::vector<std::array<double, 8>> ops;      // Kraus matrices with their coefficients applied
  std::vector<double> probs;                   // max_ij |K_ij|^2 of each operator
  std::vector<std::array<double, 8>> applied;  // the matrices the trajectories apply (ops when empty)
};

// calculate-decoherence-params (channel.clj:234-250)
int decoherence(double t1, double t2, double gate_ns, double* g1, double* g2, std::string* err) {
  if (!(t1 > 0)) { *err = "Assert failed: (pos? t1)"; return QG_ERR_INVALID_ARG; }
  if (!(t2 > 0)) { *err = "Assert failed: (pos? t2)"; return QG_ERR_INVALID_ARG; }
  if (!(gate_ns > 0)) { *err = "Assert failed: (pos? gate-time)"; return QG_ERR_INVALID_ARG; }
  const double us = gate_ns / 1000.0;
  *g1 = 1.0 - std::exp(-(us / t1));
  *g2 = 1.0 - std::exp(-(us / t2));
  return QG_OK;
}

std::array<double, 8> mat(double a, double ai, double b, double bi, double c, double ci, double d, double di) {
  return {a, ai, b, bi, c, ci, d, di};
}

// The channel of one gate-noise entry, as apply-gate-noise builds it (noise.clj:73-99).
int build_channel(const qg_gate_noise& e, Channel* ch, std::string* err) {
  ch->ops.clear();
  ch->applied.clear();
  switch (e.noise_type) {
    case QG_NOISE_DEPOLARIZING: {  // channel.clj:40-63
      const double p = e.strength;
      if (!(p >= 0.0 && p <= 1.0)) {
        *err = "Assert failed: (s/valid? :org.soulspace.qclojure.domain.channel/noise-probability p)";
        return QG_ERR_INVALID_ARG;
      }
      if (!(p <= 0.75)) {
        *err = "Assert failed: (<= p 0.75)";
        return QG_ERR_INVALID_ARG;
      }
      const double a = std::sqrt(1.0 - p), b = std::sqrt(p / 3.0);
      ch->ops = {mat(a, 0, 0, 0, 0, 0, a, 0), mat(0, 0, b, 0, b, 0, 0, 0), mat(0, 0, 0, -b, 0, b, 0, 0),
                 mat(b, 0, 0, 0, 0, 0, -b, 0)};
      // the operators are multiples of I, X, Y, Z: applying the unit Paulis gives the
      // same renormalised state without shrinking the norm by the coefficients
      ch->applied = {mat(1, 0, 0, 0, 0, 0, 1, 0), mat(0, 0, 1, 0, 1, 0, 0, 0), mat(0, 0, 0, -1, 0, 1, 0, 0),
                     mat(1, 0, 0, 0, 0, 0, -1, 0)};
    } break;
    case QG_NOISE_AMPLITUDE_DAMPING:  // channel.clj:65-84; decoherence when t1 and gate-time are set
    case QG_NOISE_PHASE_DAMPING: {     // channel.clj:86-104; decoherence when t2 and gate-time are set
      const bool amp = e.noise_type == QG_NOISE_AMPLITUDE_DAMPING;
      double g = e.strength;
      const bool has_t1 = e.present & QG_NOISE_HAS_T1, has_t2 = e.present & QG_NOISE_HAS_T2;
      const bool has_gt = e.present & QG_NOISE_HAS_GATE_TIME;
      if (amp && has_t1 && has_gt) {
        double g1, g2;
        int rc = decoherence(e.t1_us, has_t2 ? e.t2_us : e.t1_us, e.gate_time_ns, &g1, &g2, err);
        if (rc != QG_OK) return rc;
        g = g1;
      } else if (!amp && has_t2 && has_gt) {
        double g1, g2;
        int rc = decoherence(has_t1 ? e.t1_us : e.t2_us, e.t2_us, e.gate_time_ns, &g1, &g2, err);
        if (rc != QG_OK) return rc;
        g = g2;
      }
      if (!(g >= 0.0 && g <= 1.0)) {
        *err = "Assert failed: (s/valid? :org.soulspace.qclojure.domain.channel/damping-parameter gamma)";
        return QG_ERR_INVALID_ARG;
      }
      const double k = std::sqrt(1.0 - g), r = std::sqrt(g);
      ch->ops = {mat(1.0, 0, 0, 0, 0, 0, k, 0), amp ? mat(0, 0, r, 0, 0, 0, 0, 0) : mat(0, 0, 0, 0, 0, 0, r, 0)};
    } break;
    case QG_NOISE_COHERENT: {  // channel.clj:106-125: one operator, applied directly
      const double t = e.coherent_angle, c = std::cos(t / 2.0), s = std::sin(t / 2.0);
      if (e.coherent_axis == 0) ch->ops = {mat(c, 0, -s, 0, s, 0, c, 0)};
      else if (e.coherent_axis == 1) ch->ops = {mat(c, 0, s, 0, -s, 0, c, 0)};
      else if (e.coherent_axis == 2) ch->ops = {mat(std::cos(t), 0, 0, 0, 0, 0, std::cos(-t), 0)};
      else {
        *err = "Assert failed: (s/valid? :org.soulspace.qclojure.domain.channel/rotation-axis axis)";
        return QG_ERR_INVALID_ARG;
      }
    } break;
    default:
      break;
  }
  if (ch->applied.empty()) ch->applied = ch->ops;
  ch->probs.clear();
  for (const auto& m : ch->ops) {
    double mx = 0;
    for (int j = 0; j < 4; ++j) mx = std::max(mx, m[2 * j] * m[2 * j] + m[2 * j + 1] * m[2 * j + 1]);
    ch->probs.push_back(mx);
  }
  ch->built = true;
  return QG_OK;
}

// apply-quantum-channel's choice (channel.clj:212-231): the first operator whose
// cumulative probability exceeds the draw, else the last one.
int choose(const Channel& ch, double u) {
  const int k = (int)ch.ops.size();
  if (k <= 1) return 0;
  double cum = 0.0;
  for (int i = 0; i < k; ++i) {
    const double nc = cum + ch.probs[i];
    if (u < nc || i >= k - 1) return i;
    cum = nc;
  }
  return k - 1;
}

struct Readout {
  bool on = false;
  double p01 = 0, p10 = 0;
  bool corr = false;
  std::vector<double> factor;  // [source * n + target], NaN where no factor is given
};

// calculate-final-bitstring (noise.clj:107-160): qubits in order; a qubit's flip
// probability is its base probability times the factors from earlier flipped qubits.
uint64_t apply_readout(uint64_t bits, int n, const Readout& r, uint64_t seed, uint64_t shot) {
  if (!r.on) return bits;
  int hist[64];
  int nh = 0;
  for (int q = 0; q < n; ++q) {
    const int b = n - 1 - q;
    const int bit = (int)((bits >> b) & 1ULL);
    const double base = bit ? r.p10 : r.p01;
    double f = 1.0;
    if (r.corr)
      for (int h = 0; h < nh; ++h) {
        const double c = r.factor[(size_t)hist[h] * n + q];
        if (!std::isnan(c)) f *= c;
      }
    const double eff = std::min(1.0, std::max(0.0, base * f));
    if (uniform01(draw64(seed, shot, kStreamReadout + (uint32_t)q)) < eff) {
      bits ^= 1ULL << b;
      hist[nh++] = q;
    }
  }
  return bits;
}

struct Site {
  int entry;
  int pass;    // tiled pass holding its op
  int64_t at;  // index of its op within the pass
};

// Run body(begin, end) over [0, count) on the host's cores.
template <class F>
void parallel_for(uint64_t count, uint64_t grain, F body) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const uint64_t parts = std::min<uint64_t>(hw, std::max<uint64_t>(1, count / std::max<uint64_t>(1, grain)));
  if (parts <= 1) {
    body(0, count);
    return;
  }
  std::vector<std::thread> th;
  const uint64_t per = (count + parts - 1) / parts;
  for (uint64_t t = 0; t < parts; ++t) {
    const uint64_t b = t * per, e = std::min(count, b + per);
    if (b < e) th.emplace_back(body, b, e);
  }
  for (auto& x : th) x.join();
}

double ms_between(std::chrono::steady_clock::time_point a) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
}

}  // namespace

}  // namespace qg

using namespace qg;

extern "C" int qg_noisy_run(void* ctx, const qg_circuit* circuit, const qg_noise_model* noise, uint64_t shots,
                            uint64_t seed, int32_t precision, int32_t max_trajectories, uint64_t* outcomes,
                            double* trajectories, double* final_state, qg_noisy_stats* stats) {
  const auto t0 = std::chrono::steady_clock::now();
  if (!ctx || !circuit || !noise || (shots && !outcomes)) return QG_ERR_INVALID_ARG;
  if (precision != QG_C128 && precision != QG_C64) return QG_ERR_INVALID_ARG;
  if (noise->num_entries < 0 || (noise->num_entries > 0 && !noise->entries)) return QG_ERR_INVALID_ARG;
  if (circuit->num_ops < 0 || (circuit->num_ops > 0 && !circuit->ops)) return QG_ERR_INVALID_ARG;
  if (circuit->num_ops > 0 && noise->num_entries > 0 && (!noise->op_entry || !noise->op_target))
    return QG_ERR_INVALID_ARG;
  if (noise->num_correlations < 0 ||
      (noise->num_correlations > 0 && (!noise->corr_source || !noise->corr_target || !noise->corr_factor)))
    return QG_ERR_INVALID_ARG;
  std::string err;
  auto fail = [&](int rc, const std::string& msg) {
    ctx_report_error(ctx, msg);
    return rc;
  };
  const int n = circuit->num_qubits;
  // validate the clean circuit at its own size first (operand range, unknown gates)
  {
    std::vector<GOp> gops;
    std::vector<std::vector<int>> measures;
    std::vector<int> measure_at;
    int rc = lower_circuit(circuit, &gops, &measures, &measure_at, &err);
    if (rc != QG_OK) return fail(rc, err);
    if (!measures.empty()) return fail(QG_ERR_UNSUPPORTED, "mid-circuit measurements are not supported in noisy trajectories");
  }
  if (n > 30) return fail(QG_ERR_OOM, "noisy trajectories are limited to 30 qubits");
  if (max_trajectories < 0) max_trajectories = 0;

  // readout model
  Readout ro;
  if (noise->has_readout) {
    ro.on = true;
    ro.p01 = noise->prob_0_to_1;
    ro.p10 = noise->prob_1_to_0;
    if (!(ro.p01 >= 0 && ro.p01 <= 1) || !(ro.p10 >= 0 && ro.p10 <= 1))
      return fail(QG_ERR_INVALID_ARG,
                  "Assert failed: (s/valid? :org.soulspace.qclojure.domain.noise/noise-model noise-model)");
    if (noise->num_correlations > 0) {
      ro.corr = true;
      ro.factor.assign((size_t)n * n, std::nan(""));
      for (int i = 0; i < noise->num_correlations; ++i) {
        const int a = noise->corr_source[i], b = noise->corr_target[i];
        if (a >= 0 && a < n && b >= 0 && b < n) ro.factor[(size_t)a * n + b] = noise->corr_factor[i];
      }
    }
  }

  // the template: every operation, then a Kraus operator after each noisy one
  std::vector<Channel> chans((size_t)noise->num_entries);
  std::vector<qg_op> tops;
  std::vector<Site> sites;
  tops.reserve((size_t)circuit->num_ops * 2);
  for (int k = 0; k < circuit->num_ops; ++k) {
    tops.push_back(circuit->ops[k]);
    const int e = noise->num_entries > 0 ? noise->op_entry[k] : -1;
    if (e < 0) continue;
    if (e >= noise->num_entries) return fail(QG_ERR_INVALID_ARG, "noise entry out of range");
    const qg_gate_noise& ge = noise->entries[e];
    if (ge.noise_type < QG_NOISE_DEPOLARIZING || ge.noise_type > QG_NOISE_COHERENT) continue;
    if (!chans[e].built) {
      int rc = build_channel(ge, &chans[e], &err);
      if (rc != QG_OK) return fail(rc, err);
    }
    const int q = noise->op_target[k];
    if (q < 0 || q >= n) return fail(QG_ERR_QUBIT_RANGE, "Assert failed: (< qubit-index (:num-qubits state))");
    qg_op ko;
    std::memset(&ko, 0, sizeof(ko));
    ko.opcode = QG_OP_KRAUS;
    ko.nq = 1;
    ko.q[0] = (uint8_t)q;
    std::memcpy(ko.m, chans[e].applied[0].data(), sizeof(ko.m));
    tops.push_back(ko);
    sites.push_back({e, -1, -1});
  }
  const int n_run = std::max(n, kMinQubits), shift = n_run - n;
  qg_circuit tc;
  tc.num_qubits = n_run;
  tc.num_ops = (int32_t)tops.size();
  tc.ops = tops.data();
  Program prog;
  int rc = ctx_compile_tiled(ctx, &tc, precision, &prog, &err);
  if (rc != QG_OK) return fail(rc, err);

  // passes, their op counts and where each site's op landed
  std::vector<size_t> pass_steps;
  for (size_t i = 0; i < prog.steps.size(); ++i) {
    if (prog.steps[i].kind != Step::TILE_PASS) return fail(QG_ERR_DEVICE, "noisy program is not fully tiled");
    pass_steps.push_back(i);
  }
  const size_t P = pass_steps.size();
  std::vector<int64_t> nops(P), rec_off(P + 1, 0);
  for (size_t p = 0; p < P; ++p) {
    const PassDesc& pd = prog.steps[pass_steps[p]].pass;
    nops[p] = pd.op_end - pd.op_begin;
    rec_off[p + 1] = rec_off[p] + nops[p];
    for (int64_t j = pd.op_begin; j < pd.op_end; ++j) {
      const uint32_t tag = prog.tops[(size_t)j].tag;
      if (tag == 0) continue;
      if (tag > sites.size() || sites[tag - 1].pass >= 0) return fail(QG_ERR_DEVICE, "noise site lost in scheduling");
      sites[tag - 1].pass = (int)p;
      sites[tag - 1].at = j - pd.op_begin;
    }
  }
  for (const Site& s : sites)
    if (s.pass < 0) return fail(QG_ERR_DEVICE, "noise site lost in scheduling");
  const int64_t R = rec_off[P];  // op records per trajectory
  const size_t rec = kop_record_bytes();
  const int arith = prog.arith;

  // encoded records: the template per pass, and every operator of every site
  std::vector<unsigned char> tmpl((size_t)R * rec);
  for (size_t p = 0; p < P; ++p) {
    const PassDesc& pd = prog.steps[pass_steps[p]].pass;
    encode_kops(precision, arith, prog.tops.data() + pd.op_begin, nops[p], tmpl.data() + rec * (size_t)rec_off[p]);
  }
  std::vector<std::vector<unsigned char>> variants(sites.size());
  for (size_t s = 0; s < sites.size(); ++s) {
    const Channel& ch = chans[sites[s].entry];
    const PassDesc& pd = prog.steps[pass_steps[sites[s].pass]].pass;
    TOp t = prog.tops[(size_t)(pd.op_begin + sites[s].at)];
    variants[s].resize(rec * ch.applied.size());
    for (size_t v = 0; v < ch.applied.size(); ++v) {
      set_op_matrix(&t, ch.applied[v].data());
      encode_kops(precision, arith, &t, 1, variants[s].data() + rec * v);
    }
  }

  // Batches of shots. Shots whose Kraus choices coincide end in the same state, so each
  // batch simulates only its distinct choice vectors and samples every shot from its
  // vector's state (with the shot's own draw). Batch size: device memory for one state
  // per shot, host op records for one state per shot.
  const int dev = ctx_device_of(ctx);
  cudaSetDevice(dev);
  const size_t state_bytes = (precision == QG_C64 ? 8ull : 16ull) << n_run;
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return fail(QG_ERR_DEVICE, "cudaMemGetInfo failed");
  const size_t budget = std::min(free_b / 2, (size_t)64 << 30);
  const size_t per = state_bytes + rec * (size_t)R + 64;
  if (budget < per) return fail(QG_ERR_OOM, "one trajectory does not fit the device memory budget");
  uint64_t B = std::min<uint64_t>(shots ? shots : 1, 65536);
  B = std::min<uint64_t>(B, std::max<size_t>(1, budget / per));
  B = std::min<uint64_t>(B, std::max<size_t>(1, ((size_t)1 << 30) / std::max<size_t>(1, rec * (size_t)R)));
  const size_t S = sites.size();

  cudaStream_t st;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return fail(QG_ERR_DEVICE, "stream");
  void* slab = nullptr;
  void** d_ptrs = nullptr;
  unsigned char* d_kops = nullptr;
  uint64_t* d_out = nullptr;
  double* d_norm = nullptr;
  int32_t* d_state_of = nullptr;
  unsigned char* h_kops = nullptr;
  size_t h_cap = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double device_ms = 0;
  int batches = 0;
  int64_t distinct = 0;
  auto cleanup = [&]() {
    cudaStreamSynchronize(st);
    if (slab) cudaFree(slab);
    if (d_ptrs) cudaFree(d_ptrs);
    if (d_kops) cudaFree(d_kops);
    if (d_out) cudaFree(d_out);
    if (d_norm) cudaFree(d_norm);
    if (d_state_of) cudaFree(d_state_of);
    if (h_kops) cudaFreeHost(h_kops);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaStreamDestroy(st);
  };
  auto cuda_check = [&](cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
  };
  bool ok = cuda_check(cudaMalloc(&slab, state_bytes * B), "alloc trajectories") &&
            cuda_check(cudaMalloc((void**)&d_ptrs, sizeof(void*) * B), "alloc pointers") &&
            cuda_check(cudaMalloc((void**)&d_kops, rec * (size_t)R * B + 16), "alloc op records") &&
            cuda_check(cudaMalloc((void**)&d_out, sizeof(uint64_t) * B), "alloc outcomes") &&
            cuda_check(cudaMalloc((void**)&d_norm, sizeof(double) * B), "alloc norms") &&
            cuda_check(cudaMalloc((void**)&d_state_of, sizeof(int32_t) * B), "alloc shot states") &&
            cuda_check(cudaEventCreate(&e0), "event") && cuda_check(cudaEventCreate(&e1), "event");
  if (ok) {
    std::vector<void*> ptrs(B);
    for (uint64_t m = 0; m < B; ++m) ptrs[m] = (unsigned char*)slab + state_bytes * m;
    ok = cuda_check(cudaMemcpyAsync(d_ptrs, ptrs.data(), sizeof(void*) * B, cudaMemcpyHostToDevice, st), "H2D") &&
         cuda_check(cudaStreamSynchronize(st), "sync");
  }
  std::vector<uint64_t> h_out(B);
  std::vector<double> h_norm(B);
  std::vector<int32_t> state_of(B);
  std::vector<uint8_t> choices(B * std::max<size_t>(S, 1));
  std::vector<uint64_t> reps;
  std::unordered_map<std::string, int32_t> seen;
  std::vector<double> host_state;
  int result = QG_OK;
  for (uint64_t base = 0; ok && base < shots; base += B) {
    const uint64_t nb = std::min<uint64_t>(B, shots - base);
    // Kraus choices of every shot, and the distinct choice vectors
    reps.clear();
    seen.clear();
    parallel_for(nb, 256, [&](uint64_t b, uint64_t e) {
      for (uint64_t m = b; m < e; ++m) {
        uint8_t* cv = choices.data() + m * S;
        for (size_t s = 0; s < S; ++s) {
          const Channel& ch = chans[sites[s].entry];
          cv[s] = (uint8_t)(ch.ops.size() > 1
                                ? choose(ch, uniform01(draw64(seed, base + m, kStreamKraus + (uint32_t)s)))
                                : 0);
        }
      }
    });
    for (uint64_t m = 0; m < nb; ++m) {
      const uint8_t* cv = choices.data() + m * S;
      auto it = seen.emplace(std::string((const char*)cv, S), (int32_t)reps.size());
      if (it.second) reps.push_back(m);
      state_of[m] = it.first->second;
    }
    const uint64_t U = reps.size();
    distinct += (int64_t)U;
    const size_t need = rec * (size_t)R * U + 16;
    if (need > h_cap) {  // pinned staging for the records, grown on demand
      if (h_kops) cudaFreeHost(h_kops);
      h_kops = nullptr;
      h_cap = std::max(need, std::min(rec * (size_t)R * B + 16, h_cap * 2));
      if (!cuda_check(cudaMallocHost((void**)&h_kops, h_cap), "alloc host records")) {
        ok = false;
        break;
      }
    }
    // op records of the distinct states: pass-major, states contiguous within a pass
    parallel_for(U, 64, [&](uint64_t b, uint64_t e) {
      for (uint64_t u = b; u < e; ++u) {
        const uint8_t* cv = choices.data() + reps[u] * S;
        for (size_t p = 0; p < P; ++p) {
          unsigned char* dst = h_kops + rec * (size_t)(rec_off[p] * (int64_t)U + (int64_t)u * nops[p]);
          std::memcpy(dst, tmpl.data() + rec * (size_t)rec_off[p], rec * (size_t)nops[p]);
        }
        for (size_t s = 0; s < S; ++s) {
          const Site& si = sites[s];
          unsigned char* dst =
              h_kops + rec * (size_t)(rec_off[si.pass] * (int64_t)U + (int64_t)u * nops[si.pass] + si.at);
          std::memcpy(dst, variants[s].data() + rec * (size_t)cv[s], rec);
        }
      }
    });
    ok = cuda_check(cudaEventRecord(e0, st), "event") &&
         cuda_check(cudaMemcpyAsync(d_kops, h_kops, rec * (size_t)R * U, cudaMemcpyHostToDevice, st), "H2D records") &&
         cuda_check(cudaMemcpyAsync(d_state_of, state_of.data(), sizeof(int32_t) * nb, cudaMemcpyHostToDevice, st),
                    "H2D shot states") &&
         cuda_check(launch_batch_zero(slab, precision, n_run, (int)U, st), "zero states");
    for (size_t p = 0; ok && p < P; ++p) {
      PassDesc pd = prog.steps[pass_steps[p]].pass;
      pd.op_begin = 0;
      pd.op_end = nops[p];
      ok = cuda_check(launch_tile_pass(precision, arith, tile_pass_io(prog, pass_steps[p]), n_run, pd, d_ptrs, (int)U,
                                       d_kops + rec * (size_t)(rec_off[p] * (int64_t)U), nops[p], nullptr, st),
                      "trajectory pass");
    }
    ok = ok && cuda_check(launch_traj_normalise(precision, d_ptrs, (int)U, n_run, d_norm, st), "renormalise") &&
         cuda_check(launch_traj_sample(precision, d_ptrs, d_state_of, (int)nb, n_run, shift, seed, base,
                                       kStreamMeasure, d_out, st),
                    "trajectory sampling") &&
         cuda_check(cudaEventRecord(e1, st), "event") &&
         cuda_check(cudaMemcpyAsync(h_out.data(), d_out, sizeof(uint64_t) * nb, cudaMemcpyDeviceToHost, st), "D2H") &&
         cuda_check(cudaMemcpyAsync(h_norm.data(), d_norm, sizeof(double) * U, cudaMemcpyDeviceToHost, st), "D2H") &&
         cuda_check(cudaStreamSynchronize(st), "sync");
    if (!ok) break;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    device_ms += ms;
    ++batches;
    for (uint64_t m = 0; m < nb; ++m) {
      // measure-state rejects a state whose probabilities do not sum to one (state.clj:901)
      if (!(std::sqrt(h_norm[state_of[m]]) > kNormTolerance)) {
        result = QG_ERR_NOT_NORMALIZED;
        err = "State is not properly normalized (trajectory " + std::to_string(base + m) + ")";
        break;
      }
    }
    if (result != QG_OK) break;
    parallel_for(nb, 1024, [&](uint64_t b, uint64_t e) {
      for (uint64_t m = b; m < e; ++m) outcomes[base + m] = apply_readout(h_out[m], n, ro, seed, base + m);
    });
    // final states: the first max_trajectories shots, and the last shot
    const uint64_t N = 1ULL << n, Nr = 1ULL << n_run;
    for (uint64_t m = 0; m < nb; ++m) {
      const uint64_t traj = base + m;
      double* dst_t = (trajectories && traj < (uint64_t)max_trajectories) ? trajectories + 2 * N * traj : nullptr;
      double* dst_f = (final_state && traj == shots - 1) ? final_state : nullptr;
      if (!dst_t && !dst_f) continue;
      host_state.resize(2 * Nr);
      const unsigned char* src = (const unsigned char*)slab + state_bytes * (size_t)state_of[m];
      if (precision == QG_C64) {
        std::vector<float> f(2 * Nr);
        ok = cuda_check(cudaMemcpy(f.data(), src, state_bytes, cudaMemcpyDeviceToHost), "D2H state");
        for (uint64_t i = 0; i < 2 * Nr; ++i) host_state[i] = f[i];
      } else {
        ok = cuda_check(cudaMemcpy(host_state.data(), src, state_bytes, cudaMemcpyDeviceToHost), "D2H state");
      }
      if (!ok) break;
      for (double* dst : {dst_t, dst_f}) {
        if (!dst) continue;
        for (uint64_t i = 0; i < N; ++i) {
          dst[2 * i] = host_state[2 * (i << shift)];
          dst[2 * i + 1] = host_state[2 * (i << shift) + 1];
        }
      }
    }
  }
  cleanup();
  if (!ok) return fail(QG_ERR_DEVICE, err);
  if (result != QG_OK) return fail(result, err);
  if (stats) {
    stats->device_ms = device_ms;
    stats->total_ms = ms_between(t0);
    stats->batches = batches;
    stats->batch_size = (int32_t)B;
    stats->noise_sites = (int64_t)sites.size();
    stats->passes = (int64_t)P;
    stats->distinct_states = distinct;
  }
  return QG_OK;
}
