// Runtime of libqgpu.so: contexts, device-resident states, the job queue and
// every extern "C" entry point declared in include/qgpu.h.
//
// Job semantics follow src/org/soulspace/qclojure/adapter/backend/ideal_simulator.clj:
// submit returns at once (:120-136), status goes :queued -> :running ->
// :completed | :failed | :cancelled (:138-141), failures carry a message
// (:93-96), cancel answers :cancelled / :cannot-cancel / :not-found
// (:154-163), queue-status counts jobs by status (:165-176). Worker threads
// (one CUDA stream each) run jobs; a job is admitted only when its state fits
// the HBM budget, so several jobs overlap on the device.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <array>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "qgpu_internal.h"

namespace qg {

using Clock = std::chrono::steady_clock;

static double ms_since(Clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

struct Ctx;

// ---------------------------------------------------------------------------
// Device state
// ---------------------------------------------------------------------------
struct State {
  Ctx* ctx = nullptr;
  int n = 0;
  int prec = QG_C128;
  void* d = nullptr;
  size_t bytes = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  double* d_part = nullptr;  // reduction partials: 4 * reduce_blocks doubles
  void** d_self = nullptr;   // device copy of d (the tiled kernel takes an array of states)
  int nblocks = 0;
  std::string err;
};

static size_t amp_bytes(int prec) { return prec == QG_C64 ? 8 : 16; }

static int cuda_fail(std::string* err, cudaError_t e, const char* what) {
  if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
  return QG_ERR_DEVICE;
}
#define CK(expr, what)                                   \
  do {                                                   \
    cudaError_t e_ = (expr);                             \
    if (e_ != cudaSuccess) return cuda_fail(err, e_, what); \
  } while (0)

static int state_alloc(State* s, int n, int prec, cudaStream_t stream, std::string* err) {
  s->n = n;
  s->prec = prec;
  s->bytes = amp_bytes(prec) << n;
  s->stream = stream;
  s->nblocks = reduce_blocks_for(n);
  CK(cudaMallocAsync(&s->d, s->bytes, stream), "cudaMallocAsync(state)");
  CK(cudaMallocAsync((void**)&s->d_part, sizeof(double) * 4 * s->nblocks, stream), "cudaMallocAsync(partials)");
  CK(cudaMallocAsync((void**)&s->d_self, sizeof(void*), stream), "cudaMallocAsync(self)");
  CK(cudaMemcpyAsync(s->d_self, &s->d, sizeof(void*), cudaMemcpyHostToDevice, stream), "H2D self");
  return QG_OK;
}

static void state_release(State* s) {
  if (s->d) cudaFreeAsync(s->d, s->stream);
  if (s->d_part) cudaFreeAsync(s->d_part, s->stream);
  if (s->d_self) cudaFreeAsync(s->d_self, s->stream);
  s->d_self = nullptr;
  s->d = nullptr;
  s->d_part = nullptr;
}

// Sum (sum, comp) pairs from the device in a fixed order.
static int fetch_dd(State* s, const double* d_part, int count, double* out, std::string* err) {
  std::vector<double> h(2 * (size_t)count);
  CK(cudaMemcpyAsync(h.data(), d_part, sizeof(double) * 2 * count, cudaMemcpyDeviceToHost, s->stream), "D2H partials");
  CK(cudaStreamSynchronize(s->stream), "sync");
  long double acc = 0;
  double hi = 0, lo = 0;
  for (int i = 0; i < count; ++i) {
    // TwoSum in double keeps the compensation; long double only for the final fold
    double x = h[2 * i];
    double t = hi + x, bp = t - hi;
    lo += (hi - (t - bp)) + (x - bp);
    hi = t;
    lo += h[2 * i + 1];
  }
  acc = (long double)hi + (long double)lo;
  *out = (double)acc;
  return QG_OK;
}

static int upload_c128(State* s, const double* host, std::string* err) {
  const uint64_t N = 1ULL << s->n;
  if (s->prec == QG_C128) {
    CK(cudaMemcpyAsync(s->d, host, s->bytes, cudaMemcpyHostToDevice, s->stream), "H2D state");
    return QG_OK;
  }
  // complex64: stage complex128 chunks through a device buffer
  const uint64_t chunk = std::min<uint64_t>(N, 1ULL << 24);
  double* tmp = nullptr;
  CK(cudaMallocAsync((void**)&tmp, chunk * 16, s->stream), "cudaMallocAsync(stage)");
  for (uint64_t off = 0; off < N; off += chunk) {
    uint64_t c = std::min(chunk, N - off);
    CK(cudaMemcpyAsync(tmp, host + 2 * off, c * 16, cudaMemcpyHostToDevice, s->stream), "H2D stage");
    CK(launch_c128_to_c64(tmp, (float*)s->d + 2 * off, c, s->stream), "convert");
  }
  CK(cudaFreeAsync(tmp, s->stream), "cudaFreeAsync");
  return QG_OK;
}

static int download_c128(State* s, double* host, std::string* err) {
  const uint64_t N = 1ULL << s->n;
  if (s->prec == QG_C128) {
    CK(cudaMemcpyAsync(host, s->d, s->bytes, cudaMemcpyDeviceToHost, s->stream), "D2H state");
    CK(cudaStreamSynchronize(s->stream), "sync");
    return QG_OK;
  }
  const uint64_t chunk = std::min<uint64_t>(N, 1ULL << 24);
  double* tmp = nullptr;
  CK(cudaMallocAsync((void**)&tmp, chunk * 16, s->stream), "cudaMallocAsync(stage)");
  for (uint64_t off = 0; off < N; off += chunk) {
    uint64_t c = std::min(chunk, N - off);
    CK(launch_c64_to_c128((const float*)s->d + 2 * off, tmp, c, s->stream), "convert");
    CK(cudaMemcpyAsync(host + 2 * off, tmp, c * 16, cudaMemcpyDeviceToHost, s->stream), "D2H stage");
  }
  CK(cudaFreeAsync(tmp, s->stream), "cudaFreeAsync");
  CK(cudaStreamSynchronize(s->stream), "sync");
  return QG_OK;
}

// ---------------------------------------------------------------------------
// Program execution (shared by jobs and qg_state_apply)
// ---------------------------------------------------------------------------
struct ExecStats {
  double device_ms = 0;
  int passes = 0;
  int specialised = 0;                     // tiled passes that ran as specialised kernels
  double compile_ms = 0;                   // host time to obtain them (0 on a cache hit)
  std::vector<float>* pass_ms = nullptr;  // per-step CUDA-event times when profiling
  std::vector<int>* pass_kind = nullptr;
};

static int do_measure(State* s, const std::vector<int>& qubits, uint64_t seed, uint64_t draw_index,
                      uint64_t* outcome_out, double* prob_out, std::string* err) {
  const int n = s->n;
  const int m_orig = (int)qubits.size();
  // unique bits in order of first appearance
  std::vector<int> ubits;
  std::vector<int> orig_to_u(m_orig);
  for (int k = 0; k < m_orig; ++k) {
    int b = n - 1 - qubits[k];
    auto it = std::find(ubits.begin(), ubits.end(), b);
    if (it == ubits.end()) {
      orig_to_u[k] = (int)ubits.size();
      ubits.push_back(b);
    } else {
      orig_to_u[k] = (int)(it - ubits.begin());
    }
  }
  const int m = (int)ubits.size();
  if (m > 15) {
    *err = "measurement of more than 15 distinct qubits is not supported";
    return QG_ERR_UNSUPPORTED;
  }
  const int nout = 1 << m;
  int nbx = std::max(1, 1024 / nout);
  uint64_t work = (1ULL << n) >> m;
  if ((uint64_t)nbx * 256 > work) nbx = (int)std::max<uint64_t>(1, (work + 255) / 256);
  int* d_bits = nullptr;
  double* d_pm = nullptr;
  unsigned long long* d_qm = nullptr;
  CK(cudaMallocAsync((void**)&d_bits, sizeof(int) * 16, s->stream), "alloc");
  CK(cudaMallocAsync((void**)&d_pm, sizeof(double) * 2 * nout * nbx, s->stream), "alloc");
  CK(cudaMallocAsync((void**)&d_qm, sizeof(unsigned long long) * nout * nbx, s->stream), "alloc");
  CK(cudaMemcpyAsync(d_bits, ubits.data(), sizeof(int) * m, cudaMemcpyHostToDevice, s->stream), "H2D bits");
  CK(launch_marginal_host(s->d, s->prec, n, ubits.data(), d_bits, m, nbx, d_pm, d_qm, s->stream), "marginal");
  std::vector<double> hpm(2 * (size_t)nout * nbx);
  std::vector<unsigned long long> hqm((size_t)nout * nbx);
  CK(cudaMemcpyAsync(hpm.data(), d_pm, sizeof(double) * hpm.size(), cudaMemcpyDeviceToHost, s->stream), "D2H");
  CK(cudaMemcpyAsync(hqm.data(), d_qm, sizeof(unsigned long long) * hqm.size(), cudaMemcpyDeviceToHost, s->stream),
     "D2H");
  CK(cudaStreamSynchronize(s->stream), "sync");
  cudaFreeAsync(d_bits, s->stream);
  cudaFreeAsync(d_pm, s->stream);
  cudaFreeAsync(d_qm, s->stream);
  std::vector<double> Pu(nout);
  std::vector<uint64_t> Qu(nout);
  for (int o = 0; o < nout; ++o) {
    double hi = 0, lo = 0;
    uint64_t q = 0;
    for (int b = 0; b < nbx; ++b) {
      size_t slot = (size_t)o * nbx + b;
      double x = hpm[2 * slot];
      double t = hi + x, bp = t - hi;
      lo += (hi - (t - bp)) + (x - bp);
      hi = t;
      lo += hpm[2 * slot + 1];
      q += hqm[slot];
    }
    Pu[o] = hi + lo;
    Qu[o] = q;
  }
  // outcomes in the reference's index order (bit k <-> qubits[k])
  const uint64_t norig = 1ULL << m_orig;
  auto to_u = [&](uint64_t o, bool* ok) {
    uint64_t u = 0;
    uint64_t seen = 0, val = 0;
    for (int k = 0; k < m_orig; ++k) {
      int ui = orig_to_u[k];
      uint64_t bit = (o >> k) & 1;
      if (seen & (1ULL << ui)) {
        if (((val >> ui) & 1) != bit) { *ok = false; return (uint64_t)0; }
      } else {
        seen |= 1ULL << ui;
        val |= bit << ui;
      }
    }
    u = val;
    *ok = true;
    return u;
  };
  uint64_t T = 0;
  for (int o = 0; o < nout; ++o) T += Qu[o];
  uint64_t sel = norig - 1;
  if (T > 0) {
    unsigned __int128 prod = (unsigned __int128)draw64(seed, draw_index, 1u) * T;
    uint64_t u = (uint64_t)(prod >> 64), c = 0;
    for (uint64_t o = 0; o < norig; ++o) {
      bool ok;
      uint64_t ui = to_u(o, &ok);
      if (!ok) continue;
      c += Qu[ui];
      if (c > u) { sel = o; break; }
    }
  }
  bool ok;
  uint64_t usel = to_u(sel, &ok);
  double ps = ok ? Pu[usel] : 0.0;
  double nf = ps > 0 ? 1.0 / std::sqrt(ps) : 1.0;
  GOp g;
  std::memset(&g, 0, sizeof(g));
  g.kind = OK_COLLAPSE;
  for (int k = 0; k < m; ++k) {
    g.mask |= 1ULL << ubits[k];
    if (ok && ((usel >> k) & 1)) g.val |= 1ULL << ubits[k];
  }
  if (!ok) g.val = ~0ULL;  // impossible outcome: everything collapses to zero (never chosen with T > 0)
  g.m[0] = nf;
  CK(launch_plain_op(s->d, s->prec, n, g, s->stream), "collapse");
  if (outcome_out) *outcome_out = sel;
  if (prob_out) *prob_out = ps;
  return QG_OK;
}

// Specialised pass kernels are used for states of at least this many qubits
// (QG_PASS_KERNELS_AUTO). A pass kernel compiles in about 0.1 s of host time
// (in parallel over the host cores); an interpreted 29-qubit double-float pass
// takes about 13 ms on the device, so from here on even a circuit that runs once
// gains, while smaller one-off jobs (the serving stream) would lose.
// qg_autotune_crossover measures the crossover for a context and replaces it.
constexpr int kPassKernelMinQubits = 29;
// Large jobs below the crossover that wait in the queue get their pass kernels compiled
// on background host threads meanwhile; a job that starts after its compile finished
// runs them, one that starts before runs interpreted. Host cores are otherwise idle
// while the device works through the queue, so the compile costs the job nothing.
constexpr int kPrecompileMinQubits = 20;
constexpr int kPrecompileThreads = 2;

static std::shared_ptr<const PassKernels> maybe_pass_kernels(const State* s, const Program& prog);
static std::shared_ptr<const PassKernels> forced_pass_kernels(const State* s, const Program& prog);

// specialise: -1 the context's policy (maybe_pass_kernels), 0 never, 1 always.
static int exec_program(State* s, const Program& prog, uint64_t seed, const std::atomic<bool>* cancel,
                        ExecStats* stats, std::string* err, int specialise = -1) {
  double* d_dense = nullptr;
  void* d_kops = nullptr;
  std::shared_ptr<const PassKernels> pk;
  {
    const auto t0 = Clock::now();
    if (specialise < 0) {
      pk = maybe_pass_kernels(s, prog);
    } else if (specialise > 0) {
      pk = forced_pass_kernels(s, prog);
    }
    if (stats) stats->compile_ms = ms_since(t0);
  }
  if (!prog.tops.empty()) {
    std::vector<unsigned char> kops(kop_record_bytes() * prog.tops.size());
    encode_kops(s->prec, prog.arith, prog.tops.data(), (int64_t)prog.tops.size(), kops.data());
    CK(cudaMallocAsync(&d_kops, kops.size(), s->stream), "alloc ops");
    CK(cudaMemcpyAsync(d_kops, kops.data(), kops.size(), cudaMemcpyHostToDevice, s->stream), "H2D ops");
    CK(cudaStreamSynchronize(s->stream), "sync");  // the host buffer dies at scope end
  }
  if (!prog.dense.empty()) {
    CK(cudaMallocAsync((void**)&d_dense, sizeof(double) * prog.dense.size(), s->stream), "alloc dense");
    CK(cudaMemcpyAsync(d_dense, prog.dense.data(), sizeof(double) * prog.dense.size(), cudaMemcpyHostToDevice,
                       s->stream),
       "H2D dense");
  }
  float* d_tc = nullptr;  // tensor-core block operands, then one int: the kernels' error word
  int* d_tc_err = nullptr;
  if (!prog.dense_tc.empty()) {
    const size_t wb = sizeof(float) * prog.dense_tc.size(), wb_al = (wb + 255) / 256 * 256;
    CK(cudaMallocAsync((void**)&d_tc, wb_al + 256, s->stream), "alloc dense tc");
    CK(cudaMemcpyAsync(d_tc, prog.dense_tc.data(), wb, cudaMemcpyHostToDevice, s->stream), "H2D dense tc");
    d_tc_err = (int*)((char*)d_tc + wb_al);
    CK(cudaMemsetAsync(d_tc_err, 0, sizeof(int), s->stream), "clear dense tc error");
    CK(cudaStreamSynchronize(s->stream), "sync");  // the program's host vector may go away
  }
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0), "event");
  CK(cudaEventCreate(&e1), "event");
  CK(cudaEventRecord(e0, s->stream), "event");
  uint64_t measure_index = 0;
  int rc = QG_OK;
  const bool profile = stats && stats->pass_ms;
  std::vector<cudaEvent_t> evs;
  std::vector<int> spec_step;
  if (profile) {
    spec_step.assign(prog.steps.size(), 0);
    evs.resize(prog.steps.size() + 1);
    for (auto& ev : evs) CK(cudaEventCreate(&ev), "event");
  }
  for (size_t i = 0; i < prog.steps.size() && rc == QG_OK; ++i) {
    if (cancel && cancel->load()) {
      rc = QG_ERR_CANCELLED;
      break;
    }
    const Step& st = prog.steps[i];
    if (profile) cudaEventRecord(evs[i], s->stream);
    cudaError_t e = cudaSuccess;
    if (st.kind == Step::PLAIN_OP && st.op.kind == OK_DENSE && (st.op.flags & kDenseTcFlag)) {
      e = launch_dense_tc(s->d, s->n, st.op.dk, st.op.dbits, d_tc + st.op.doff, d_tc_err, s->stream);
      if (profile) spec_step[i] = 2;
    } else if (st.kind == Step::PLAIN_OP) {
      e = launch_plain_op(s->d, s->prec, s->n, st.op, s->stream);
    } else if (st.kind == Step::TILE_PASS) {
      if (pk && pass_kernel_ready(*pk, i)) {
        e = launch_pass_kernel(*pk, i, s->n, st.pass, s->d, s->prec, s->stream);
        if (stats) ++stats->specialised;
        if (profile) spec_step[i] = 1;
      } else {
        e = launch_tile_pass(s->prec, prog.arith, tile_pass_io(prog, i), s->n, st.pass, s->d_self, 1, d_kops, 0,
                             d_dense, s->stream);
      }
    } else {
      rc = do_measure(s, st.mqubits, seed, measure_index++, nullptr, nullptr, err);
    }
    if (e != cudaSuccess) rc = cuda_fail(err, e, "gate pass");
    if (profile) cudaEventRecord(evs[i + 1], s->stream);
  }
  cudaEventRecord(e1, s->stream);
  cudaError_t se = cudaEventSynchronize(e1);
  if (se != cudaSuccess && rc == QG_OK) rc = cuda_fail(err, se, "gate passes");
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (profile) {
    stats->pass_ms->clear();
    stats->pass_kind->clear();
    for (size_t i = 0; i < prog.steps.size(); ++i) {
      float t = 0;
      if (rc == QG_OK) cudaEventElapsedTime(&t, evs[i], evs[i + 1]);
      stats->pass_ms->push_back(t);
      const Step::Kind k = prog.steps[i].kind;
      stats->pass_kind->push_back(k == Step::PLAIN_OP ? (spec_step[i] == 2 ? 4 : 0)
                                  : k == Step::TILE_PASS ? (spec_step[i] ? 3 : 1) : 2);
    }
    for (auto& ev : evs) cudaEventDestroy(ev);
  }
  if (d_tc) {
    int tc_err = 0;
    if (cudaMemcpyAsync(&tc_err, d_tc_err, sizeof(int), cudaMemcpyDeviceToHost, s->stream) == cudaSuccess &&
        cudaStreamSynchronize(s->stream) == cudaSuccess && tc_err != 0 && rc == QG_OK) {
      *err = "dense block kernel: a bounded wait gave up (tensor-core pass did not complete)";
      rc = QG_ERR_DEVICE;
    }
    cudaFreeAsync(d_tc, s->stream);
  }
  if (d_dense) cudaFreeAsync(d_dense, s->stream);
  if (d_kops) cudaFreeAsync(d_kops, s->stream);
  if (stats) {
    stats->device_ms = ms;
    stats->passes = prog.hbm_passes;
  }
  return rc;
}

// reorder = false keeps passes in circuit order even for tolerance-held policies:
// sweeps batch circuits whose pass structure must not depend on their graphs.
static int compile_program(const qg_circuit* c, int precision, int fusion, int fuse_k, int arith, Program* prog,
                           std::string* err, bool reorder = true, const qg_tuning* tune = nullptr) {
  NvtxRange nvtx("qg compile");
  if (tune) {
    prog->rbits = tune->reg_bits;
    prog->bufs = tune->buffers;
    prog->ctas = tune->ctas_per_sm;
  }
  // complex128 dense fused blocks follow the arithmetic setting: double-float blocks on
  // the FP32 pipes, or FP64 (FMA inside the block product) for the exact setting
  prog->arith = arith == QG_ARITH_DOUBLE_FLOAT ? QG_ARITH_DOUBLE_FLOAT : QG_ARITH_EXACT;
  std::vector<GOp> gops;
  std::vector<std::vector<int>> measures;
  std::vector<int> measure_at;
  int rc = lower_circuit(c, &gops, &measures, &measure_at, err);
  if (rc != QG_OK) return rc;
  const bool tolerance_held = precision == QG_C64 || prog->arith == QG_ARITH_DOUBLE_FLOAT;
  if (fusion == QG_FUSE_TILED && tolerance_held)
    factor_global_phases(&gops, &measure_at, reorder ? kFactorRotations : kFactorNone);
  return schedule(c->num_qubits, precision, fusion, fuse_k, gops, measures, measure_at, prog, err,
                  reorder && fusion == QG_FUSE_TILED && tolerance_held, tune ? tune->tile_bits : 0);
}

// ---------------------------------------------------------------------------
// Result extraction on a device state
// ---------------------------------------------------------------------------
static int st_norm2(State* s, double* out, std::string* err) {
  CK(launch_norm2(s->d, s->prec, s->n, s->d_part, s->nblocks, s->stream), "norm2");
  return fetch_dd(s, s->d_part, s->nblocks, out, err);
}

static int st_pauli(State* s, const char* pauli, double* out, std::string* err) {
  uint64_t xm = 0, zm = 0;
  int ny = 0;
  for (int q = 0; q < s->n; ++q) {
    uint64_t b = 1ULL << (s->n - 1 - q);
    char ch = pauli[q];
    if (ch == 'X') xm |= b;
    else if (ch == 'Y') { xm |= b; zm |= b; ++ny; }
    else if (ch == 'Z') zm |= b;
    else if (ch != 'I') {
      *err = "Pauli strings use the characters I, X, Y, Z";
      return QG_ERR_INVALID_ARG;
    }
  }
  CK(launch_pauli_expect(s->d, s->prec, s->n, xm, zm, ny & 3, s->d_part, s->nblocks, s->stream), "pauli");
  return fetch_dd(s, s->d_part, s->nblocks, out, err);
}

static int st_expect1q(State* s, const double* o8, int target, double* out, std::string* err) {
  if (target < 0 || target >= s->n) {
    *err = "observable target out of range";
    return QG_ERR_QUBIT_RANGE;
  }
  CK(launch_expect_1q(s->d, s->prec, s->n, s->n - 1 - target, o8, s->d_part, s->nblocks, s->stream), "expect");
  return fetch_dd(s, s->d_part, s->nblocks, out, err);
}

static int st_inner(State* a, State* b, double* re, double* im, std::string* err) {
  if (a->n != b->n || a->prec != b->prec) {
    *err = "states differ in size or precision";
    return QG_ERR_INVALID_ARG;
  }
  CK(cudaStreamSynchronize(b->stream), "sync");
  CK(launch_inner(a->d, b->d, a->prec, a->n, a->d_part, a->nblocks, a->stream), "inner");
  int rc = fetch_dd(a, a->d_part, a->nblocks, re, err);
  if (rc != QG_OK) return rc;
  return fetch_dd(a, a->d_part + 2 * a->nblocks, a->nblocks, im, err);
}

// out[0] = max_i |a_i - b_i|, out[1] = 1 - |<b|a>|^2 / (<a|a><b|b>), out[2] = total variation
// distance of the outcome distributions, 1/2 sum_i | |a_i|^2 - |b_i|^2 |.
static int st_compare(State* a, State* b, double* out, std::string* err) {
  if (a->n != b->n || b->prec != QG_C128) {
    *err = "the reference state must be complex128 of the same size";
    return QG_ERR_INVALID_ARG;
  }
  CK(cudaStreamSynchronize(b->stream), "sync");
  const int nb = a->nblocks;
  double* d_buf = nullptr;
  CK(cudaMallocAsync((void**)&d_buf, sizeof(double) * 13 * nb, a->stream), "alloc partials");
  int rc = QG_OK;
  double v[6] = {0, 0, 0, 0, 0, 0};
  std::vector<double> mx(nb);
  if (launch_compare(a->d, a->prec, b->d, a->n, d_buf, d_buf + 12 * nb, nb, a->stream) != cudaSuccess) {
    *err = "compare launch failed";
    rc = QG_ERR_DEVICE;
  }
  for (int k = 0; k < 6 && rc == QG_OK; ++k) rc = fetch_dd(a, d_buf + 2 * k * nb, nb, &v[k], err);
  if (rc == QG_OK &&
      (cudaMemcpyAsync(mx.data(), d_buf + 12 * nb, sizeof(double) * nb, cudaMemcpyDeviceToHost, a->stream) !=
           cudaSuccess ||
       cudaStreamSynchronize(a->stream) != cudaSuccess)) {
    *err = "D2H maxima";
    rc = QG_ERR_DEVICE;
  }
  cudaFreeAsync(d_buf, a->stream);
  if (rc != QG_OK) return rc;
  double m = 0;
  for (double x : mx) m = std::max(m, x);
  const double dd = v[0], zr = v[1], zi = v[2], na = v[3], nbn = v[4], tv = v[5];
  out[0] = std::sqrt(m);
  out[1] = (na > 0 && nbn > 0) ? (nbn * dd - (zr * zr + zi * zi)) / (na * nbn) : 1.0;
  out[2] = 0.5 * tv;
  return QG_OK;
}

static int st_sample(State* s, uint64_t shots, uint64_t seed, std::vector<uint64_t>* outcomes, std::string* err) {
  size_t scratch = sampler_scratch_bytes(s->n, shots);
  void* d_scratch = nullptr;
  uint64_t* d_out = nullptr;
  double* d_total = nullptr;
  CK(cudaMallocAsync(&d_scratch, scratch, s->stream), "alloc sampler");
  CK(cudaMallocAsync((void**)&d_out, sizeof(uint64_t) * std::max<uint64_t>(shots, 1), s->stream), "alloc outcomes");
  CK(cudaMallocAsync((void**)&d_total, sizeof(double) * 2, s->stream), "alloc total");
  CK(launch_sample(s->d, s->prec, s->n, shots, seed, d_scratch, d_out, d_total, s->stream), "sample");
  double total = 0;
  outcomes->resize(shots);
  CK(cudaMemcpyAsync(&total, d_total, sizeof(double), cudaMemcpyDeviceToHost, s->stream), "D2H total");
  if (shots) {
    CK(cudaMemcpyAsync(outcomes->data(), d_out, sizeof(uint64_t) * shots, cudaMemcpyDeviceToHost, s->stream),
       "D2H outcomes");
  }
  CK(cudaStreamSynchronize(s->stream), "sync");
  cudaFreeAsync(d_scratch, s->stream);
  cudaFreeAsync(d_out, s->stream);
  cudaFreeAsync(d_total, s->stream);
  // state.clj:901-903 rejects |sum p - 1| > 1e-8; a complex64 state carries FP32
  // rounding (about 1e-7 per gate), so its check allows 1e-4 instead.
  const double norm_tol = s->prec == QG_C64 ? 1e-4 : 1e-8;
  if (std::fabs(total - 1.0) > norm_tol) {
    *err = "State is not properly normalized (total probability " + std::to_string(total) + ")";
    outcomes->clear();
    return QG_ERR_NOT_NORMALIZED;
  }
  return QG_OK;
}

static int st_probs(State* s, double* host, std::string* err) {
  const uint64_t N = 1ULL << s->n;
  const uint64_t chunk = std::min<uint64_t>(N, 1ULL << 25);
  double* d_p = nullptr;
  CK(cudaMallocAsync((void**)&d_p, sizeof(double) * N, s->stream), "alloc probs");
  CK(launch_probabilities(s->d, s->prec, s->n, d_p, s->stream), "probabilities");
  for (uint64_t off = 0; off < N; off += chunk) {
    uint64_t c = std::min(chunk, N - off);
    CK(cudaMemcpyAsync(host + off, d_p + off, sizeof(double) * c, cudaMemcpyDeviceToHost, s->stream), "D2H probs");
  }
  CK(cudaStreamSynchronize(s->stream), "sync");
  cudaFreeAsync(d_p, s->stream);
  return QG_OK;
}

static int st_gather(State* s, const std::vector<uint64_t>& idx, std::vector<double>* out, std::string* err) {
  out->assign(2 * idx.size(), 0.0);
  if (idx.empty()) return QG_OK;
  const uint64_t N = 1ULL << s->n;
  for (uint64_t i : idx)
    if (i >= N) {
      *err = "basis state index out of range";
      return QG_ERR_INVALID_ARG;
    }
  uint64_t* d_idx = nullptr;
  double* d_out = nullptr;
  CK(cudaMallocAsync((void**)&d_idx, sizeof(uint64_t) * idx.size(), s->stream), "alloc");
  CK(cudaMallocAsync((void**)&d_out, sizeof(double) * 2 * idx.size(), s->stream), "alloc");
  CK(cudaMemcpyAsync(d_idx, idx.data(), sizeof(uint64_t) * idx.size(), cudaMemcpyHostToDevice, s->stream), "H2D");
  CK(launch_gather(s->d, s->prec, d_idx, (int64_t)idx.size(), d_out, s->stream), "gather");
  CK(cudaMemcpyAsync(out->data(), d_out, sizeof(double) * out->size(), cudaMemcpyDeviceToHost, s->stream), "D2H");
  CK(cudaStreamSynchronize(s->stream), "sync");
  cudaFreeAsync(d_idx, s->stream);
  cudaFreeAsync(d_out, s->stream);
  return QG_OK;
}

// ---------------------------------------------------------------------------
// Jobs
// ---------------------------------------------------------------------------
struct SpecCopy {
  uint32_t flags = 0;
  uint64_t shots = 1;
  std::vector<double> coeffs;
  std::string paulis;
  std::vector<double> observables;
  std::vector<int32_t> obs_targets;
  std::vector<uint64_t> basis_states;
  std::vector<uint64_t> prob_targets;
  std::vector<double> references;
  int n_terms = 0, n_obs = 0, n_refs = 0;
};

struct Job {
  uint64_t id = 0;
  int n = 0;
  std::vector<qg_op> ops;
  SpecCopy spec;
  std::vector<double> initial;
  uint64_t seed = 0;
  int precision = QG_C128, fusion = QG_FUSE_TILED, arith = QG_ARITH_EXACT;
  std::atomic<int> status{QG_JOB_QUEUED};
  std::atomic<bool> cancel{false};
  int error_code = QG_OK;
  std::string error;
  Clock::time_point submitted, started, finished;
  double exec_ms = 0, device_ms = 0, queue_ms = 0;
  int passes = 0;
  // results
  std::vector<uint64_t> shots;
  std::vector<std::pair<uint64_t, uint64_t>> counts;
  std::vector<double> probs;          // full probability vector (when small or requested)
  std::vector<double> target_probs;
  std::vector<double> amplitudes;
  std::vector<double> expectations, variances;
  std::vector<double> term_values;
  double energy = 0;
  std::vector<double> fidelities;
  std::vector<double> density;
  double accuracy[3] = {0, 0, 0};     // QG_RES_ACCURACY: max |d amp|, 1 - F, TVD
  int has = 0;
  std::unique_ptr<State> state;       // final state kept on the device
  bool state_pinned = false;          // requested by :state-vector; never evicted
  uint64_t batch = 0;
  std::unique_ptr<Program> prog;      // compiled by the worker that admitted the job
  int batched_with = 0;               // jobs that shared its small-job launch (0: run alone)
  int specialised = 0;                // tiled passes run as specialised kernels
};

struct Ctx {
  int device = 0;
  qg_config cfg{};
  std::mutex mu;
  std::condition_variable cv;       // queue / admission
  std::condition_variable done_cv;  // job completion
  std::map<uint64_t, std::shared_ptr<Job>> jobs;
  std::deque<uint64_t> queue;
  std::map<uint64_t, std::vector<uint64_t>> batches;
  std::vector<std::thread> workers;
  // compiled small jobs (one tile per state) waiting for the batcher, which runs
  // everything ready of one qubit count in one launch
  std::deque<std::shared_ptr<Job>> ready;
  std::condition_variable ready_cv;
  std::thread batcher;
  bool stop = false;
  bool batch_stop = false;  // set after the workers have exited
  int small_queued = 0;     // queued jobs of the small-job lane
  int compiling = 0;        // small jobs admitted and being compiled
  uint64_t next_id = 1;
  uint64_t hbm_budget = 0, hbm_in_use = 0, hbm_total = 0;
  int sm_count = 0;
  std::string last_error;
  std::mutex err_mu;
  // pass-kernel shapes chosen by qg_autotune / qg_tuning_set, per (qubits, precision)
  std::mutex tune_mu;
  std::map<std::pair<int, int>, qg_tuning> tunings;
  // smallest state that runs specialised under QG_PASS_KERNELS_AUTO, per precision
  // (kPassKernelMinQubits until qg_autotune_crossover measures it)
  std::atomic<int> spec_min_qubits[2] = {{kPassKernelMinQubits}, {kPassKernelMinQubits}};
  // device-resident loops of small jobs, per (qubits, precision, arithmetic)
  std::mutex loop_mu;
  std::condition_variable loop_cv;
  std::map<std::tuple<int, int, int>, std::unique_ptr<struct JobLoop>> loops;
  std::thread loop_poller;
  bool loop_stop = false;
  uint64_t loop_jobs = 0;
  // background compiles of queued large jobs' pass kernels (precompile_loop)
  std::mutex pre_mu;
  std::condition_variable pre_cv;
  std::deque<std::shared_ptr<Job>> pre_queue;
  std::vector<std::thread> pre_threads;
  bool pre_stop = false;
  uint64_t precompiled = 0;
};

// True when programs of this kind run as specialised pass kernels (the condition
// maybe_pass_kernels applies at run time), so a tuned shape applies to them.
static bool will_specialise(const Ctx* c, int n, int prec, int arith, int fusion) {
  if (fusion != QG_FUSE_TILED) return false;
  if (prec == QG_C128 && arith != QG_ARITH_DOUBLE_FLOAT) return false;
  const int mode = c->cfg.pass_kernels;
  if (mode == QG_PASS_KERNELS_OFF) return false;
  return mode == QG_PASS_KERNELS_ALWAYS || n >= c->spec_min_qubits[prec == QG_C64 ? 1 : 0].load();
}
// The tuned shape for programs of this kind, if one was chosen (copied into *out).
static const qg_tuning* tuning_for(Ctx* c, int n, int prec, int arith, int fusion, qg_tuning* out) {
  if (!c || !will_specialise(c, n, prec, arith, fusion)) return nullptr;
  std::lock_guard<std::mutex> lk(c->tune_mu);
  auto it = c->tunings.find({n, prec});
  if (it == c->tunings.end()) return nullptr;
  *out = it->second;
  return out;
}

static std::shared_ptr<const PassKernels> maybe_pass_kernels(const State* s, const Program& prog) {
  const Ctx* c = s->ctx;
  if (!c || prog.tops.empty()) return nullptr;
  if (s->prec == QG_C128 && prog.arith != QG_ARITH_DOUBLE_FLOAT) return nullptr;
  const int mode = c->cfg.pass_kernels;
  if (mode == QG_PASS_KERNELS_OFF) return nullptr;
  if (mode != QG_PASS_KERNELS_ALWAYS && s->n < c->spec_min_qubits[s->prec == QG_C64 ? 1 : 0].load()) {
    // below the crossover a one-off program runs interpreted, unless its kernels were
    // compiled meanwhile (a queued job's background compile, precompile_loop)
    return s->n >= kPrecompileMinQubits ? pass_kernels_cached(prog, s->prec, c->device) : nullptr;
  }
  std::string why;
  return pass_kernels_for(prog, s->prec, c->device, &why);
}

// The program's pass kernels whatever the context's policy (nullptr when none compile).
static std::shared_ptr<const PassKernels> forced_pass_kernels(const State* s, const Program& prog) {
  if (!s->ctx || prog.tops.empty()) return nullptr;
  if (s->prec == QG_C128 && prog.arith != QG_ARITH_DOUBLE_FLOAT) return nullptr;
  std::string why;
  return pass_kernels_for(prog, s->prec, s->ctx->device, &why);
}

static void set_ctx_error(Ctx* c, const std::string& e) {
  std::lock_guard<std::mutex> g(c->err_mu);
  c->last_error = e;
}

// ---------------------------------------------------------------------------
// Context services for the noisy-trajectory runner (noisy.cpp)
// ---------------------------------------------------------------------------
int ctx_device_of(void* ctx) { return ((Ctx*)ctx)->device; }
int ctx_arithmetic_of(void* ctx) { return ((Ctx*)ctx)->cfg.arithmetic; }
void ctx_report_error(void* ctx, const std::string& msg) { set_ctx_error((Ctx*)ctx, msg); }
int ctx_compile_tiled(void* ctx, const qg_circuit* c, int precision, Program* prog, std::string* err) {
  Ctx* cx = (Ctx*)ctx;
  return compile_program(c, precision, QG_FUSE_TILED, cx->cfg.fuse_k, cx->cfg.arithmetic, prog, err, true);
}

static size_t job_bytes(int n, int prec) {
  size_t st = amp_bytes(prec) << n;
  return st + st / 4 + (64ULL << 20);  // state + sampler/probability scratch headroom
}

static void finish_job(Ctx* c, Job* j, int status) {
  j->finished = Clock::now();
  j->exec_ms = std::chrono::duration<double, std::milli>(j->finished - j->started).count();
  {
    std::lock_guard<std::mutex> g(c->mu);
    j->status.store(status);
  }
  c->done_cv.notify_all();
}

// Evict final states of completed jobs (oldest first) until `need` bytes fit. Caller holds mu.
static bool make_room(Ctx* c, size_t need) {
  if (c->hbm_in_use + need <= c->hbm_budget) return true;
  std::vector<std::shared_ptr<Job>> cands;
  for (auto& kv : c->jobs) {
    Job* j = kv.second.get();
    if (j->state && !j->state_pinned && j->status.load() == QG_JOB_COMPLETED) cands.push_back(kv.second);
  }
  std::sort(cands.begin(), cands.end(), [](auto& a, auto& b) { return a->finished < b->finished; });
  for (auto& j : cands) {
    if (c->hbm_in_use + need <= c->hbm_budget) break;
    cudaStreamSynchronize(j->state->stream);
    size_t b = job_bytes(j->n, j->state->prec);
    state_release(j->state.get());
    cudaStreamSynchronize(j->state->stream);
    if (j->state->own_stream) cudaStreamDestroy(j->state->stream);
    j->state.reset();
    c->hbm_in_use -= std::min(c->hbm_in_use, b);
  }
  return c->hbm_in_use + need <= c->hbm_budget;
}

static int compile_job(Ctx* c, Job* j, std::string* err) {
  auto prog = std::make_unique<Program>();
  qg_circuit circ{j->n, (int32_t)j->ops.size(), j->ops.data()};
  qg_tuning tu;
  const qg_tuning* tune = tuning_for(c, j->n, j->precision, j->arith, j->fusion, &tu);
  const int rc = compile_program(&circ, j->precision, j->fusion, c->cfg.fuse_k, j->arith, prog.get(), err, true, tune);
  if (rc == QG_OK) j->prog = std::move(prog);
  return rc;
}

// Jobs of the small-job lane: tiled fusion and 5..12 qubits (one tile per state).
static bool small_eligible(const Job* j) {
  return j->fusion == QG_FUSE_TILED && j->n >= 5 && j->n <= kMaxSmallJobQubits;
}

// A small job's state is one tile (5..12 qubits) and its program is tiled passes only.
static bool small_job(const Job* j) {
  if (!j->prog || j->fusion != QG_FUSE_TILED || j->n < 5 || j->n > kMaxSmallJobQubits) return false;
  for (const Step& s : j->prog->steps)
    if (s.kind != Step::TILE_PASS) return false;
  return true;
}

// Allocate the job's state on `stream` and set it to |0...0> or the initial state.
static int init_job_state(Ctx* c, Job* j, cudaStream_t stream, State* st, std::string* err) {
  st->ctx = c;
  int rc = state_alloc(st, j->n, j->precision, stream, err);
  if (rc != QG_OK) return rc;
  if (!j->initial.empty()) return upload_c128(st, j->initial.data(), err);
  cudaError_t e = launch_set_basis(st->d, st->prec, st->n, 0, stream);
  return e == cudaSuccess ? QG_OK : cuda_fail(err, e, "zero-state");
}

static int job_results(Ctx* c, Job* j, std::unique_ptr<State> st, cudaStream_t stream, int rc, std::string err);

static int run_job(Ctx* c, Job* j, cudaStream_t stream) {
  std::string err;
  int rc = j->prog ? QG_OK : compile_job(c, j, &err);
  if (rc != QG_OK) {
    j->error_code = rc;
    j->error = err;
    return rc;
  }
  auto st = std::make_unique<State>();
  rc = init_job_state(c, j, stream, st.get(), &err);
  ExecStats stats;
  if (rc == QG_OK) {
    NvtxRange nvtx("qg launch");
    rc = exec_program(st.get(), *j->prog, j->seed, &j->cancel, &stats, &err);
  }
  j->device_ms = stats.device_ms;
  j->passes = stats.passes;
  j->specialised = stats.specialised;
  return job_results(c, j, std::move(st), stream, rc, std::move(err));
}

// Result extraction on the final state (result.clj:179-457), then keep the state
// for later reads or release it.
static int job_results(Ctx* c, Job* j, std::unique_ptr<State> st, cudaStream_t stream, int rc, std::string err) {
  NvtxRange nvtx("qg extract");
  const SpecCopy& sp = j->spec;
  const uint64_t N = 1ULL << j->n;
  if (rc == QG_OK && (sp.flags & QG_RES_MEASUREMENTS)) {
    rc = st_sample(st.get(), sp.shots, j->seed, &j->shots, &err);
    if (rc == QG_OK) {
      std::vector<uint64_t> sorted = j->shots;
      std::sort(sorted.begin(), sorted.end());
      j->counts.clear();
      for (size_t i = 0; i < sorted.size();) {
        size_t k = i;
        while (k < sorted.size() && sorted[k] == sorted[i]) ++k;
        j->counts.emplace_back(sorted[i], (uint64_t)(k - i));
        i = k;
      }
      j->has |= QG_RES_MEASUREMENTS;
    }
  }
  if (rc == QG_OK && (sp.flags & QG_RES_PROBABILITIES)) {
    if (!sp.prob_targets.empty()) {
      std::vector<double> amps;
      rc = st_gather(st.get(), sp.prob_targets, &amps, &err);
      j->target_probs.resize(sp.prob_targets.size());
      for (size_t i = 0; rc == QG_OK && i < sp.prob_targets.size(); ++i) {
        double re = amps[2 * i], im = amps[2 * i + 1];
        j->target_probs[i] = re * re + im * im;
      }
    } else if (j->n <= 26) {
      j->probs.resize(N);
      rc = st_probs(st.get(), j->probs.data(), &err);
    }
    if (rc == QG_OK) j->has |= QG_RES_PROBABILITIES;
  }
  if (rc == QG_OK && (sp.flags & QG_RES_AMPLITUDES)) {
    rc = st_gather(st.get(), sp.basis_states, &j->amplitudes, &err);
    if (rc == QG_OK) j->has |= QG_RES_AMPLITUDES;
  }
  if (rc == QG_OK && (sp.flags & (QG_RES_EXPECTATION | QG_RES_VARIANCE))) {
    j->expectations.assign(sp.n_obs, 0.0);
    j->variances.assign(sp.n_obs, 0.0);
    for (int k = 0; rc == QG_OK && k < sp.n_obs; ++k) {
      const double* o = &sp.observables[8 * k];
      int t = sp.obs_targets.empty() ? -1 : sp.obs_targets[k];
      if (t < 0) {
        if (j->n == 1) t = 0;
        else {
          err = "observables without a target qubit must match the register size; pass a target";
          rc = QG_ERR_UNSUPPORTED;
          break;
        }
      }
      double e;
      rc = st_expect1q(st.get(), o, t, &e, &err);
      if (rc != QG_OK) break;
      // O^2 (observables.clj:305-320 squares the full observable)
      double o2[8];
      for (int r = 0; r < 2; ++r)
        for (int cc = 0; cc < 2; ++cc) {
          double re = 0, im = 0;
          for (int q = 0; q < 2; ++q) {
            double ar = o[2 * (2 * r + q)], ai = o[2 * (2 * r + q) + 1];
            double br = o[2 * (2 * q + cc)], bi = o[2 * (2 * q + cc) + 1];
            re += ar * br - ai * bi;
            im += ar * bi + ai * br;
          }
          o2[2 * (2 * r + cc)] = re;
          o2[2 * (2 * r + cc) + 1] = im;
        }
      double e2;
      rc = st_expect1q(st.get(), o2, t, &e2, &err);
      j->expectations[k] = e;
      j->variances[k] = e2 - e * e;
    }
    if (rc == QG_OK) j->has |= (sp.flags & (QG_RES_EXPECTATION | QG_RES_VARIANCE));
  }
  if (rc == QG_OK && (sp.flags & QG_RES_HAMILTONIAN)) {
    j->term_values.assign(sp.n_terms, 0.0);
    double energy = 0;
    for (int k = 0; rc == QG_OK && k < sp.n_terms; ++k) {
      double v;
      rc = st_pauli(st.get(), sp.paulis.data() + (size_t)k * j->n, &v, &err);
      j->term_values[k] = v;
      double term = sp.coeffs[k] * v;
      energy = (k == 0) ? term : energy + term;  // (reduce + ...) in term order
    }
    j->energy = energy;
    if (rc == QG_OK) j->has |= QG_RES_HAMILTONIAN;
  }
  if (rc == QG_OK && (sp.flags & QG_RES_FIDELITY)) {
    j->fidelities.assign(sp.n_refs, 0.0);
    for (int k = 0; rc == QG_OK && k < sp.n_refs; ++k) {
      State ref;
      ref.ctx = c;
      rc = state_alloc(&ref, j->n, j->precision, stream, &err);
      if (rc == QG_OK) rc = upload_c128(&ref, sp.references.data() + 2 * N * (size_t)k, &err);
      double re = 0, im = 0;
      if (rc == QG_OK) rc = st_inner(st.get(), &ref, &re, &im, &err);
      cudaStreamSynchronize(stream);
      state_release(&ref);
      j->fidelities[k] = std::sqrt(re * re + im * im);
    }
    if (rc == QG_OK) j->has |= QG_RES_FIDELITY;
  }
  if (rc == QG_OK && (sp.flags & QG_RES_ACCURACY)) {
    // the same circuit again: complex128, exact FP64 arithmetic, the reference's gate order
    NvtxRange nvtx("qg accuracy");
    Program exact;
    qg_circuit circ{j->n, (int32_t)j->ops.size(), j->ops.data()};
    rc = compile_program(&circ, QG_C128, QG_FUSE_TILED, c->cfg.fuse_k, QG_ARITH_EXACT, &exact, &err, false);
    State ref;
    ref.ctx = c;
    if (rc == QG_OK) rc = state_alloc(&ref, j->n, QG_C128, stream, &err);
    if (rc == QG_OK) {
      cudaError_t e = launch_set_basis(ref.d, QG_C128, j->n, 0, stream);
      if (e != cudaSuccess) rc = cuda_fail(&err, e, "accuracy reference zero-state");
    }
    if (rc == QG_OK && !j->initial.empty()) rc = upload_c128(&ref, j->initial.data(), &err);
    ExecStats xs;
    if (rc == QG_OK) rc = exec_program(&ref, exact, j->seed, nullptr, &xs, &err, 0);
    double d3[3] = {0, 0, 0};
    if (rc == QG_OK) rc = st_compare(st.get(), &ref, d3, &err);
    cudaStreamSynchronize(stream);
    state_release(&ref);
    cudaStreamSynchronize(stream);
    if (rc == QG_OK) {
      std::memcpy(j->accuracy, d3, sizeof(d3));
      j->has |= QG_RES_ACCURACY;
    }
  }
  if (rc == QG_OK && (sp.flags & QG_RES_DENSITY_MATRIX)) {
    if (j->n > 12) {
      err = "density matrix limited to 12 qubits (4^n entries)";
      rc = QG_ERR_UNSUPPORTED;
    } else {
      double* d_rho = nullptr;
      cudaError_t e = cudaMallocAsync((void**)&d_rho, sizeof(double) * 2 * N * N, stream);
      if (e == cudaSuccess) e = launch_density(st->d, st->prec, st->n, d_rho, stream);
      j->density.resize(2 * N * N);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(j->density.data(), d_rho, sizeof(double) * 2 * N * N, cudaMemcpyDeviceToHost, stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
      if (d_rho) cudaFreeAsync(d_rho, stream);
      if (e != cudaSuccess) rc = cuda_fail(&err, e, "density matrix");
      else j->has |= QG_RES_DENSITY_MATRIX;
    }
  }
  cudaError_t se = cudaStreamSynchronize(stream);
  if (se != cudaSuccess && rc == QG_OK) rc = cuda_fail(&err, se, "job");
  if (rc == QG_OK) {
    j->has |= QG_RES_STATE_VECTOR;  // final state available while kept
    j->state_pinned = (sp.flags & QG_RES_STATE_VECTOR) != 0;
    // the kept state gets its own stream so it outlives this worker's queue
    cudaStream_t own;
    if (cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking) == cudaSuccess) {
      st->stream = own;
      st->own_stream = true;
    }
    j->state = std::move(st);
  } else {
    state_release(st.get());
    cudaStreamSynchronize(stream);
    j->error_code = rc;
    j->error = err;
  }
  return rc;
}

// Release the job's HBM reservation unless its final state is kept, and publish the outcome.
static void complete_job(Ctx* c, Job* j, int rc) {
  const size_t need = job_bytes(j->n, j->precision);
  {
    std::lock_guard<std::mutex> g(c->mu);
    if (need <= c->hbm_budget && !j->state) c->hbm_in_use -= std::min(c->hbm_in_use, need);
  }
  c->cv.notify_all();
  if (rc == QG_OK) finish_job(c, j, QG_JOB_COMPLETED);
  else if (rc == QG_ERR_CANCELLED) finish_job(c, j, QG_JOB_CANCELLED);
  else finish_job(c, j, QG_JOB_FAILED);
}

// Workers of the small-job lane compile small jobs and hand them to the batcher,
// so small jobs never wait behind large ones; the other workers run large jobs.
// ---------------------------------------------------------------------------
// Device-resident loops for small jobs (k_job_loop). One loop per (qubits, precision,
// arithmetic): a ring of slots in mapped host memory that the host fills in order and
// publishes by raising the tail; the loop's CTAs claim slots in that order, run each
// job whole in shared memory and set the slot's done flag; a poller thread extracts
// the results of finished jobs. A loop kernel returns after kLoopIdleNs without work
// (its only waits are these polls) and is started again when the next job arrives;
// the poller also restarts one that left while a published job was still unclaimed.
// ---------------------------------------------------------------------------
constexpr uint32_t kLoopSlots = 256;
constexpr uint64_t kLoopIdleNs = 3000000;  // 3 ms

struct JobLoop {
  int n = 0, prec = 0, arith = 0;
  void* host = nullptr;  // pinned, mapped: kLoopSlots slots, then the tail word
  JobLoopSlot* h_slots = nullptr;
  JobLoopSlot* d_slots = nullptr;
  uint32_t* h_tail = nullptr;
  uint32_t* d_tail = nullptr;
  uint32_t* d_head = nullptr;    // device: claimed count, then the served count
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;    // recorded after the latest loop launch
  bool launched = false;
  uint32_t published = 0;
  uint64_t launches = 0;
  int since_launch = 0;          // jobs published to the running loop kernel
  int outstanding = 0;
  std::vector<std::shared_ptr<Job>> job;      // per slot (null: free)
  std::vector<std::unique_ptr<State>> state;  // per slot
  std::vector<void*> buf;                     // per slot: op records, then per-pass op counts
};

static bool loops_enabled(const Ctx* c) { return c->cfg.small_job_loop != QG_JOB_LOOP_OFF; }

// Caller holds loop_mu.
static JobLoop* get_loop(Ctx* c, int n, int prec, int arith, std::string* err) {
  auto key = std::make_tuple(n, prec, arith);
  auto it = c->loops.find(key);
  if (it != c->loops.end()) return it->second.get();
  auto L = std::make_unique<JobLoop>();
  L->n = n;
  L->prec = prec;
  L->arith = arith;
  const size_t bytes = sizeof(JobLoopSlot) * kLoopSlots + 64;
  cudaError_t e = cudaHostAlloc(&L->host, bytes, cudaHostAllocMapped | cudaHostAllocPortable);
  void* dhost = nullptr;
  if (e == cudaSuccess) e = cudaHostGetDevicePointer(&dhost, L->host, 0);
  if (e == cudaSuccess) e = cudaMalloc((void**)&L->d_head, 2 * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(L->d_head, 0, 2 * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L->done, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    cuda_fail(err, e, "small-job loop setup");
    if (L->host) cudaFreeHost(L->host);
    if (L->d_head) cudaFree(L->d_head);
    return nullptr;
  }
  std::memset(L->host, 0, bytes);
  L->h_slots = (JobLoopSlot*)L->host;
  L->d_slots = (JobLoopSlot*)dhost;
  L->h_tail = (uint32_t*)((char*)L->host + sizeof(JobLoopSlot) * kLoopSlots);
  L->d_tail = (uint32_t*)((char*)dhost + sizeof(JobLoopSlot) * kLoopSlots);
  L->job.resize(kLoopSlots);
  L->state.resize(kLoopSlots);
  L->buf.assign(kLoopSlots, nullptr);
  JobLoop* raw = L.get();
  c->loops[key] = std::move(L);
  return raw;
}

// Caller holds loop_mu.
static cudaError_t start_loop(JobLoop* L) {
  cudaError_t e = launch_job_loop(L->prec, L->arith, L->n, L->d_slots, kLoopSlots, L->d_tail, L->d_head,
                                  L->d_head + 1, kLoopIdleNs, L->stream);
  if (e == cudaSuccess) e = cudaEventRecord(L->done, L->stream);
  if (e == cudaSuccess) {
    L->launched = true;
    ++L->launches;
    L->since_launch = 0;
  }
  return e;
}

// Publish a compiled small job to its loop: its state and op records go to the device
// first (on the lane's stream), then the slot is filled and the tail raised.
static int loop_submit(Ctx* c, const std::shared_ptr<Job>& j, cudaStream_t stream, std::string* err) {
  NvtxRange nvtx("qg loop publish");
  auto st = std::make_unique<State>();
  int rc = init_job_state(c, j.get(), stream, st.get(), err);
  if (rc != QG_OK) return rc;
  const Program& pr = *j->prog;
  const size_t rec = kop_record_bytes();
  std::vector<int32_t> nops;
  for (const Step& s : pr.steps) nops.push_back((int32_t)(s.pass.op_end - s.pass.op_begin));
  const size_t b_ops = rec * std::max<size_t>(pr.tops.size(), 1);
  std::vector<unsigned char> host(b_ops + sizeof(int32_t) * std::max<size_t>(nops.size(), 1), 0);
  encode_kops(j->precision, pr.arith, pr.tops.data(), (int64_t)pr.tops.size(), host.data());
  if (!nops.empty()) std::memcpy(host.data() + b_ops, nops.data(), sizeof(int32_t) * nops.size());
  void* d = nullptr;
  CK(cudaMallocAsync(&d, host.size(), stream), "small-job records");
  cudaError_t e = cudaMemcpyAsync(d, host.data(), host.size(), cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) {
    cudaFreeAsync(d, stream);
    return cuda_fail(err, e, "small-job records");
  }
  std::unique_lock<std::mutex> lk(c->loop_mu);
  JobLoop* L = get_loop(c, j->n, j->precision, pr.arith, err);
  if (!L) {
    cudaFreeAsync(d, stream);
    return QG_ERR_DEVICE;
  }
  const uint32_t idx = L->published;
  const uint32_t slot = idx % kLoopSlots;
  c->loop_cv.wait(lk, [&] { return !L->job[slot]; });
  JobLoopSlot& sl = L->h_slots[slot];
  sl.rec.state = st->d;
  sl.rec.op_begin = 0;
  sl.rec.npasses = (int32_t)nops.size();
  sl.rec.pass_begin = 0;
  sl.kops = d;
  sl.pass_nops = (const int32_t*)((unsigned char*)d + b_ops);
  *(volatile int32_t*)&sl.done = 0;
  L->job[slot] = j;
  L->state[slot] = std::move(st);
  L->buf[slot] = d;
  ++L->outstanding;
  std::atomic_thread_fence(std::memory_order_seq_cst);  // the slot before the tail
  *(volatile uint32_t*)L->h_tail = idx + 1;
  L->published = idx + 1;
  std::atomic_thread_fence(std::memory_order_seq_cst);
  if (!L->launched || cudaEventQuery(L->done) == cudaSuccess) {
    e = start_loop(L);
    if (e != cudaSuccess) {
      // unpublish is not possible once the tail moved; the poller retries the start
      cuda_fail(err, e, "small-job loop launch");
    }
  }
  j->batched_with = ++L->since_launch;
  lk.unlock();
  c->loop_cv.notify_all();
  return QG_OK;
}

// Collect finished loop jobs, extract their results, restart loops that left while a
// published job was unclaimed. Runs until the context stops and no job is outstanding.
static void loop_poller_loop(Ctx* c) {
  cudaSetDevice(c->device);
  cudaStream_t stream;
  cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
  struct Finished {
    std::shared_ptr<Job> job;
    std::unique_ptr<State> state;
    void* buf;
  };
  for (;;) {
    std::vector<Finished> fin;
    {
      std::unique_lock<std::mutex> lk(c->loop_mu);
      int outstanding = 0;
      for (auto& kv : c->loops) {
        JobLoop* L = kv.second.get();
        if (L->outstanding == 0) continue;
        for (uint32_t sidx = 0; sidx < kLoopSlots; ++sidx) {
          if (!L->job[sidx]) continue;
          if (*(volatile int32_t*)&L->h_slots[sidx].done == 1) {
            std::atomic_thread_fence(std::memory_order_acquire);
            fin.push_back({std::move(L->job[sidx]), std::move(L->state[sidx]), L->buf[sidx]});
            L->job[sidx].reset();
            L->buf[sidx] = nullptr;
            --L->outstanding;
          }
        }
        // a loop that left (idle budget) while a published job was still unclaimed
        if (L->outstanding > 0 && L->launched && cudaEventQuery(L->done) == cudaSuccess) {
          bool pending = false;
          for (uint32_t sidx = 0; sidx < kLoopSlots && !pending; ++sidx)
            pending = L->job[sidx] && *(volatile int32_t*)&L->h_slots[sidx].done == 0;
          if (pending) start_loop(L);
        }
        outstanding += L->outstanding;
      }
      if (fin.empty()) {
        if (c->loop_stop && outstanding == 0) break;
        c->loop_cv.wait_for(lk, std::chrono::microseconds(50));
        continue;
      }
      c->loop_jobs += fin.size();
    }
    c->loop_cv.notify_all();  // slots are free again
    for (Finished& f : fin) {
      cudaFreeAsync(f.buf, stream);
      Job* j = f.job.get();
      j->passes = j->prog->hbm_passes;
      const int rc = job_results(c, j, std::move(f.state), stream, QG_OK, std::string());
      complete_job(c, j, rc);
    }
  }
  cudaStreamSynchronize(stream);
  cudaStreamDestroy(stream);
}

static void loops_shutdown(Ctx* c) {
  {
    std::lock_guard<std::mutex> g(c->loop_mu);
    c->loop_stop = true;
  }
  c->loop_cv.notify_all();
  if (c->loop_poller.joinable()) c->loop_poller.join();
  for (auto& kv : c->loops) {
    JobLoop* L = kv.second.get();
    cudaStreamSynchronize(L->stream);  // a loop kernel leaves within its idle budget
    cudaEventDestroy(L->done);
    cudaStreamDestroy(L->stream);
    cudaFree(L->d_head);
    cudaFreeHost(L->host);
  }
  c->loops.clear();
}


static void worker_loop(Ctx* c, bool small_lane) {
  cudaSetDevice(c->device);
  cudaStream_t stream;
  cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
  for (;;) {
    std::shared_ptr<Job> j;
    {
      std::unique_lock<std::mutex> lk(c->mu);
      for (;;) {
        if (c->stop) break;
        // first queued job of this lane that fits (jobs that can never fit fail at once)
        bool picked = false;
        for (auto it = c->queue.begin(); it != c->queue.end(); ++it) {
          auto jj = c->jobs.find(*it);
          if (jj == c->jobs.end() || jj->second->status.load() != QG_JOB_QUEUED) {
            if (jj != c->jobs.end() && small_eligible(jj->second.get())) --c->small_queued;
            c->queue.erase(it);
            picked = true;  // rescan
            break;
          }
          if (small_eligible(jj->second.get()) != small_lane) continue;
          size_t need = job_bytes(jj->second->n, jj->second->precision);
          if (need > c->hbm_budget) {
            j = jj->second;
            c->queue.erase(it);
            if (small_lane) --c->small_queued;
            picked = true;
            break;
          }
          if (make_room(c, need)) {
            c->hbm_in_use += need;
            j = jj->second;
            c->queue.erase(it);
            if (small_lane) --c->small_queued;
            picked = true;
            break;
          }
        }
        if (j) break;
        if (!picked) c->cv.wait(lk);
      }
      if (!j) break;
      j->started = Clock::now();
      j->queue_ms = std::chrono::duration<double, std::milli>(j->started - j->submitted).count();
      if (j->cancel.load()) {
        j->status.store(QG_JOB_CANCELLED);
      } else {
        j->status.store(QG_JOB_RUNNING);
        if (small_lane) ++c->compiling;
      }
    }
    if (j->status.load() == QG_JOB_CANCELLED) {
      complete_job(c, j.get(), QG_ERR_CANCELLED);  // releases the HBM reservation
      continue;
    }
    const size_t need = job_bytes(j->n, j->precision);
    int rc = QG_OK;
    if (need > c->hbm_budget) {
      j->error_code = QG_ERR_OOM;
      j->error = "state of " + std::to_string(j->n) + " qubits does not fit the HBM budget";
      rc = QG_ERR_OOM;
      if (small_lane) {
        std::lock_guard<std::mutex> g(c->mu);
        --c->compiling;
      }
    } else {
      if (small_lane) {
        // compile here (the lane's workers compile in parallel) and hand the job to the batcher
        std::string err;
        rc = compile_job(c, j.get(), &err);
        const bool small = rc == QG_OK && small_job(j.get());
        if (small && loops_enabled(c)) {
          // a device-resident loop claims it; the poller completes it
          rc = loop_submit(c, j, stream, &err);
          {
            std::lock_guard<std::mutex> g(c->mu);
            --c->compiling;
          }
          c->ready_cv.notify_all();
          if (rc == QG_OK) continue;
          j->error_code = rc;
          j->error = err;
          complete_job(c, j.get(), rc);
          continue;
        }
        const bool batch = small;
        {
          std::lock_guard<std::mutex> g(c->mu);
          if (batch) c->ready.push_back(j);
          --c->compiling;
        }
        c->ready_cv.notify_all();
        if (batch) continue;
        if (rc != QG_OK) {
          j->error_code = rc;
          j->error = err;
        }
      }
      if (rc == QG_OK) rc = run_job(c, j.get(), stream);  // mid-circuit measurements run per job
    }
    complete_job(c, j.get(), rc);
  }
  cudaStreamSynchronize(stream);
  cudaStreamDestroy(stream);
}


// ---------------------------------------------------------------------------
// Continuous batching of small jobs. Workers admit jobs as they arrive (HBM
// budget) and compile them; small ones (one tile per state) wait in `ready`.
// The batcher takes everything ready, groups it by qubit count, precision and
// arithmetic, and runs each group in one k_tile_jobs launch (one CTA per job)
// while larger jobs run on the workers' streams. Jobs that arrive meanwhile go
// into the next batch.
// ---------------------------------------------------------------------------
constexpr size_t kMaxBatchJobs = 4096;
constexpr int kBatchWindowUs = 2000;   // longest wait for jobs still being admitted
constexpr int kSmallLaneWorkers = 4;

static void run_batch(Ctx* c, std::vector<std::shared_ptr<Job>>& batch, cudaStream_t stream) {
  std::map<std::tuple<int, int, int>, std::vector<Job*>> groups;
  for (auto& j : batch) {
    if (j->cancel.load()) {
      complete_job(c, j.get(), QG_ERR_CANCELLED);
      continue;
    }
    groups[std::make_tuple(j->n, j->precision, j->prog->arith)].push_back(j.get());
  }
  const size_t rec = kop_record_bytes();
  for (auto& kv : groups) {
    std::vector<Job*>& js = kv.second;
    const int n = std::get<0>(kv.first), prec = std::get<1>(kv.first), arith = std::get<2>(kv.first);
    const size_t m = js.size();
    std::vector<std::unique_ptr<State>> sts(m);
    std::vector<int> rcs(m, QG_OK);
    std::vector<std::string> errs(m);
    std::vector<TileJobRec> recs;
    std::vector<int32_t> nops;
    std::vector<size_t> members;
    size_t total_ops = 0;
    for (size_t i = 0; i < m; ++i) {
      sts[i] = std::make_unique<State>();
      rcs[i] = init_job_state(c, js[i], stream, sts[i].get(), &errs[i]);
      if (rcs[i] != QG_OK) continue;
      TileJobRec r;
      r.state = sts[i]->d;
      r.op_begin = (int64_t)total_ops;
      r.pass_begin = (int32_t)nops.size();
      r.npasses = 0;
      for (const Step& s : js[i]->prog->steps) {
        nops.push_back((int32_t)(s.pass.op_end - s.pass.op_begin));
        ++r.npasses;
      }
      total_ops += js[i]->prog->tops.size();
      recs.push_back(r);
      members.push_back(i);
    }
    float ms = 0;
    if (!recs.empty()) {
      // one upload: op records (16-byte aligned), job records, per-pass op counts
      const size_t b_ops = rec * total_ops, b_recs = sizeof(TileJobRec) * recs.size();
      std::vector<unsigned char> host(b_ops + b_recs + sizeof(int32_t) * nops.size() + 16);
      size_t off = 0;
      for (size_t q : members) {
        const Program& pr = *js[q]->prog;
        encode_kops(prec, pr.arith, pr.tops.data(), (int64_t)pr.tops.size(), host.data() + off);
        off += rec * pr.tops.size();
      }
      std::memcpy(host.data() + b_ops, recs.data(), b_recs);
      if (!nops.empty()) std::memcpy(host.data() + b_ops + b_recs, nops.data(), sizeof(int32_t) * nops.size());
      unsigned char* d = nullptr;
      cudaEvent_t e0 = nullptr, e1 = nullptr;
      cudaError_t e = cudaMallocAsync((void**)&d, host.size(), stream);
      if (e == cudaSuccess) e = cudaMemcpyAsync(d, host.data(), host.size(), cudaMemcpyHostToDevice, stream);
      if (e == cudaSuccess) e = cudaEventCreate(&e0);
      if (e == cudaSuccess) e = cudaEventCreate(&e1);
      if (e == cudaSuccess) e = cudaEventRecord(e0, stream);
      if (e == cudaSuccess)
        e = launch_tile_jobs(prec, arith, n, reinterpret_cast<const TileJobRec*>(d + b_ops), (int)recs.size(), d,
                             reinterpret_cast<const int32_t*>(d + b_ops + b_recs), stream);
      if (e == cudaSuccess) e = cudaEventRecord(e1, stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
      if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
      if (d) cudaFreeAsync(d, stream);
      if (e != cudaSuccess)
        for (size_t q : members) rcs[q] = cuda_fail(&errs[q], e, "small-job batch");
    }
    for (size_t i = 0; i < m; ++i) {
      Job* j = js[i];
      j->device_ms = ms;
      j->passes = j->prog->hbm_passes;
      j->batched_with = (int)recs.size();
      const int rc = job_results(c, j, std::move(sts[i]), stream, rcs[i], std::move(errs[i]));
      complete_job(c, j, rc);
    }
  }
}

static void batcher_loop(Ctx* c) {
  cudaSetDevice(c->device);
  cudaStream_t stream;
  cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
  for (;;) {
    std::vector<std::shared_ptr<Job>> batch;
    {
      std::unique_lock<std::mutex> lk(c->mu);
      c->ready_cv.wait(lk, [&] { return c->batch_stop || !c->ready.empty(); });
      if (c->ready.empty()) break;  // batch_stop and nothing left
      // gathering window: small jobs already queued or being compiled join this batch
      const auto deadline = Clock::now() + std::chrono::microseconds(kBatchWindowUs);
      while (!c->batch_stop && (c->compiling > 0 || c->small_queued > 0) && c->ready.size() < kMaxBatchJobs &&
             c->ready_cv.wait_until(lk, deadline) != std::cv_status::timeout) {
      }
      while (!c->ready.empty() && batch.size() < kMaxBatchJobs) {
        batch.push_back(c->ready.front());
        c->ready.pop_front();
      }
    }
    run_batch(c, batch, stream);
  }
  cudaStreamSynchronize(stream);
  cudaStreamDestroy(stream);
}

static std::shared_ptr<Job> find_job(Ctx* c, uint64_t id) {
  std::lock_guard<std::mutex> g(c->mu);
  auto it = c->jobs.find(id);
  return it == c->jobs.end() ? nullptr : it->second;
}

static int copy_spec(const qg_result_spec* in, int n, SpecCopy* out, std::string* err) {
  if (!in) return QG_OK;
  out->flags = in->flags;
  out->shots = in->shots ? in->shots : 1;
  if (in->flags & QG_RES_HAMILTONIAN) {
    if (in->n_terms < 0 || (in->n_terms > 0 && (!in->coefficients || !in->pauli_strings))) {
      *err = "hamiltonian terms need coefficients and pauli strings";
      return QG_ERR_INVALID_ARG;
    }
    out->n_terms = in->n_terms;
    out->coeffs.assign(in->coefficients, in->coefficients + in->n_terms);
    out->paulis.assign(in->pauli_strings, (size_t)in->n_terms * n);
    for (char ch : out->paulis)
      if (ch != 'I' && ch != 'X' && ch != 'Y' && ch != 'Z') {
        *err = "Pauli strings use the characters I, X, Y, Z and have num-qubits characters";
        return QG_ERR_INVALID_ARG;
      }
  }
  if (in->flags & (QG_RES_EXPECTATION | QG_RES_VARIANCE)) {
    if (in->n_observables < 0 || (in->n_observables > 0 && !in->observables)) {
      *err = "expectation needs observables";
      return QG_ERR_INVALID_ARG;
    }
    out->n_obs = in->n_observables;
    out->observables.assign(in->observables, in->observables + 8 * (size_t)in->n_observables);
    if (in->observable_targets)
      out->obs_targets.assign(in->observable_targets, in->observable_targets + in->n_observables);
  }
  if (in->flags & QG_RES_AMPLITUDES) {
    if (in->n_basis_states < 0 || (in->n_basis_states > 0 && !in->basis_states)) {
      *err = "amplitudes need basis-states";
      return QG_ERR_INVALID_ARG;
    }
    out->basis_states.assign(in->basis_states, in->basis_states + in->n_basis_states);
  }
  if ((in->flags & QG_RES_PROBABILITIES) && in->n_probability_targets > 0) {
    if (!in->probability_targets) {
      *err = "probability targets missing";
      return QG_ERR_INVALID_ARG;
    }
    out->prob_targets.assign(in->probability_targets, in->probability_targets + in->n_probability_targets);
    for (uint64_t t : out->prob_targets)
      if (t >= (1ULL << n)) {
        *err = "probability target out of range";
        return QG_ERR_INVALID_ARG;
      }
  }
  if (in->flags & QG_RES_FIDELITY) {
    if (in->n_references < 0 || (in->n_references > 0 && !in->references)) {
      *err = "fidelity needs reference states";
      return QG_ERR_INVALID_ARG;
    }
    if (n > 28) {
      *err = "fidelity references limited to 28 qubits";
      return QG_ERR_UNSUPPORTED;
    }
    out->n_refs = in->n_references;
    out->references.assign(in->references, in->references + 2 * ((size_t)in->n_references << n));
  }
  return QG_OK;
}

// Validate a circuit and its options into a Job (not yet queued).
static int prepare_job(Ctx* c, const qg_circuit* circ, const qg_options* opt, std::shared_ptr<Job>* out) {
  if (!circ) return QG_ERR_INVALID_ARG;
  std::string err;
  // validate now (ideal_simulator.clj relies on :pre checks in backend.clj:228-230)
  {
    std::vector<GOp> g;
    std::vector<std::vector<int>> m;
    std::vector<int> at;
    int rc = lower_circuit(circ, &g, &m, &at, &err);
    if (rc != QG_OK) {
      set_ctx_error(c, err);
      return rc;
    }
  }
  auto j = std::make_shared<Job>();
  j->n = circ->num_qubits;
  j->ops.assign(circ->ops, circ->ops + circ->num_ops);
  j->seed = c->cfg.seed;
  j->precision = c->cfg.precision;
  j->fusion = c->cfg.fusion;
  j->arith = c->cfg.arithmetic;
  if (opt) {
    int rc = copy_spec(opt->spec, j->n, &j->spec, &err);
    if (rc != QG_OK) {
      set_ctx_error(c, err);
      return rc;
    }
    if (opt->initial_state) j->initial.assign(opt->initial_state, opt->initial_state + 2 * (1ULL << j->n));
    if (opt->seed) j->seed = opt->seed;
    if (opt->precision == QG_C128 || opt->precision == QG_C64) j->precision = opt->precision;
    if (opt->fusion >= QG_FUSE_PLAIN && opt->fusion <= QG_FUSE_DENSE) j->fusion = opt->fusion;
    if (opt->arithmetic == QG_ARITH_EXACT || opt->arithmetic == QG_ARITH_DOUBLE_FLOAT) j->arith = opt->arithmetic;
  }
  if (c->cfg.max_qubits > 0 && j->n > c->cfg.max_qubits) {
    set_ctx_error(c, "circuit exceeds max-qubits of this backend");
    return QG_ERR_OOM;
  }
  *out = std::move(j);
  return QG_OK;
}

// Queue prepared jobs in one step (a batch arrives together) and assign their ids.
// A queued job whose kernels a background compile could have ready by the time it runs.
static bool precompile_eligible(const Ctx* c, const Job* j) {
  if (j->n < kPrecompileMinQubits || j->fusion != QG_FUSE_TILED) return false;
  if (c->cfg.pass_kernels != QG_PASS_KERNELS_AUTO || pass_kernels_unavailable()) return false;
  if (j->precision == QG_C128 && j->arith != QG_ARITH_DOUBLE_FLOAT) return false;
  return j->n < c->spec_min_qubits[j->precision == QG_C64 ? 1 : 0].load();  // above it the run compiles anyway
}

// Background compile of queued large jobs' pass kernels (into the per-device kernel
// cache); a job already started or finished is skipped.
static void precompile_loop(Ctx* c) {
  cudaSetDevice(c->device);
  for (;;) {
    std::shared_ptr<Job> j;
    {
      std::unique_lock<std::mutex> lk(c->pre_mu);
      c->pre_cv.wait(lk, [&] { return c->pre_stop || !c->pre_queue.empty(); });
      if (c->pre_stop) break;
      // the queued job with the most interpreted work (2^n amplitudes x gates) first: a
      // compile costs all host cores for seconds, and the largest jobs save the most
      // device time by it (a 28-qubit job hundreds of milliseconds, a 20-qubit job a few)
      auto best = c->pre_queue.begin();
      double best_w = -1.0;
      for (auto it = c->pre_queue.begin(); it != c->pre_queue.end(); ++it) {
        const double w = std::ldexp((double)(*it)->ops.size(), (*it)->n);
        if ((*it)->status.load() == QG_JOB_QUEUED && w > best_w) {
          best_w = w;
          best = it;
        }
      }
      j = *best;
      c->pre_queue.erase(best);
    }
    if (j->status.load() != QG_JOB_QUEUED) continue;
    NvtxRange nvtx("qg precompile");
    Program prog;
    std::string err;
    qg_circuit circ{j->n, (int32_t)j->ops.size(), j->ops.data()};
    qg_tuning tu;  // the same program the run will compile (compile_job)
    const qg_tuning* tune = tuning_for(c, j->n, j->precision, j->arith, j->fusion, &tu);
    if (compile_program(&circ, j->precision, j->fusion, c->cfg.fuse_k, j->arith, &prog, &err, true, tune) != QG_OK)
      continue;
    std::string why;
    if (pass_kernels_for(prog, j->precision, c->device, &why, false)) {
      std::lock_guard<std::mutex> lk(c->pre_mu);
      ++c->precompiled;
    }
  }
}

static void enqueue_jobs(Ctx* c, std::vector<std::shared_ptr<Job>>& js, uint64_t batch, uint64_t* ids_out) {
  const auto now = Clock::now();
  {
    std::lock_guard<std::mutex> g(c->mu);
    for (size_t i = 0; i < js.size(); ++i) {
      Job* j = js[i].get();
      j->submitted = now;
      j->batch = batch;
      j->id = c->next_id++;
      c->jobs[j->id] = js[i];
      c->queue.push_back(j->id);
      if (small_eligible(j)) ++c->small_queued;
      if (batch) c->batches[batch].push_back(j->id);
      if (ids_out) ids_out[i] = j->id;
    }
  }
  c->cv.notify_all();
  bool pre = false;
  {
    std::lock_guard<std::mutex> g(c->pre_mu);
    for (auto& j : js)
      if (precompile_eligible(c, j.get())) {
        c->pre_queue.push_back(j);
        pre = true;
      }
  }
  if (pre) c->pre_cv.notify_one();
}

static int submit_one(Ctx* c, const qg_circuit* circ, const qg_options* opt, uint64_t* id_out) {
  if (!circ || !id_out) return QG_ERR_INVALID_ARG;
  std::vector<std::shared_ptr<Job>> js(1);
  const int rc = prepare_job(c, circ, opt, &js[0]);
  if (rc != QG_OK) return rc;
  enqueue_jobs(c, js, 0, id_out);
  return QG_OK;
}

}  // namespace qg

using namespace qg;

// ===========================================================================
// extern "C" entry points
// ===========================================================================
extern "C" {

int qg_job_loop_info(void* ctx, qg_loop_info* out) {
  if (!ctx || !out) return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  cudaSetDevice(c->device);
  std::lock_guard<std::mutex> g(c->loop_mu);
  std::memset(out, 0, sizeof(*out));
  for (auto& kv : c->loops) {
    JobLoop* L = kv.second.get();
    ++out->loops;
    if (L->launched && cudaEventQuery(L->done) == cudaErrorNotReady) ++out->running;
    out->launches += L->launches;
  }
  cudaGetLastError();
  out->jobs = c->loop_jobs;
  return QG_OK;
}


int qg_abi_version(void) { return QG_ABI_VERSION; }

int qg_device_count(int32_t* count) {
  if (!count) return QG_ERR_INVALID_ARG;
  int c = 0;
  cudaError_t e = cudaGetDeviceCount(&c);
  *count = e == cudaSuccess ? c : 0;
  return QG_OK;
}

int qg_ctx_create(const qg_config* cfg, void** ctx_out) {
  if (!ctx_out) return QG_ERR_INVALID_ARG;
  *ctx_out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return QG_ERR_NO_DEVICE;
  auto* c = new Ctx();
  if (cfg) c->cfg = *cfg;
  if (c->cfg.workers < 1) c->cfg.workers = 2;
  if (c->cfg.fuse_k < 1 || c->cfg.fuse_k > 5) c->cfg.fuse_k = 4;
  if (c->cfg.precision != QG_C64) c->cfg.precision = QG_C128;
  if (c->cfg.fusion < QG_FUSE_PLAIN || c->cfg.fusion > QG_FUSE_DENSE) c->cfg.fusion = QG_FUSE_TILED;
  if (c->cfg.arithmetic != QG_ARITH_DOUBLE_FLOAT) c->cfg.arithmetic = QG_ARITH_EXACT;
  if (c->cfg.seed == 0) c->cfg.seed = 0x5eed5eedULL;
  c->device = c->cfg.device;
  if (c->device < 0 || c->device >= ndev) {
    delete c;
    return QG_ERR_INVALID_ARG;
  }
  cudaSetDevice(c->device);
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
    delete c;
    return QG_ERR_DEVICE;
  }
  c->hbm_total = tot;
  const size_t reserve = 4ULL << 30;
  c->hbm_budget = c->cfg.hbm_budget_bytes ? c->cfg.hbm_budget_bytes : (fr > reserve ? fr - reserve : fr / 2);
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
  // keep freed blocks in the stream-ordered pool for reuse
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, c->device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  for (int w = 0; w < c->cfg.workers; ++w) c->workers.emplace_back(worker_loop, c, false);
  for (int w = 0; w < kSmallLaneWorkers; ++w) c->workers.emplace_back(worker_loop, c, true);
  c->batcher = std::thread(batcher_loop, c);
  c->loop_poller = std::thread(loop_poller_loop, c);
  for (int t = 0; t < kPrecompileThreads; ++t) c->pre_threads.emplace_back(precompile_loop, c);
  *ctx_out = c;
  return QG_OK;
}

int qg_ctx_destroy(void* ctx) {
  if (!ctx) return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  {
    std::lock_guard<std::mutex> g(c->pre_mu);
    c->pre_stop = true;
  }
  c->pre_cv.notify_all();
  for (auto& t : c->pre_threads) t.join();
  {
    std::lock_guard<std::mutex> g(c->mu);
    c->stop = true;
    for (auto& kv : c->jobs) kv.second->cancel.store(true);
  }
  c->cv.notify_all();
  for (auto& t : c->workers) t.join();
  {
    std::lock_guard<std::mutex> g(c->mu);
    c->batch_stop = true;
  }
  c->ready_cv.notify_all();
  if (c->batcher.joinable()) c->batcher.join();
  cudaSetDevice(c->device);
  loops_shutdown(c);
  for (auto& kv : c->jobs)
    if (kv.second->state) {
      State* s = kv.second->state.get();
      state_release(s);
      cudaStreamSynchronize(s->stream);
      if (s->own_stream) cudaStreamDestroy(s->stream);
    }
  cudaDeviceSynchronize();
  delete c;
  return QG_OK;
}

int qg_ctx_capabilities(void* ctx, int32_t* mq128, int32_t* mq64, uint64_t* hbm_total, int32_t* sms) {
  if (!ctx) return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  auto maxq = [&](int prec) {
    int q = 1;
    while (q < QG_MAX_QUBITS && job_bytes(q + 1, prec) <= c->hbm_budget) ++q;
    return q;
  };
  if (mq128) *mq128 = maxq(QG_C128);
  if (mq64) *mq64 = maxq(QG_C64);
  if (hbm_total) *hbm_total = c->hbm_total;
  if (sms) *sms = c->sm_count;
  return QG_OK;
}

int qg_submit(void* ctx, const qg_circuit* circuit, const qg_options* options, uint64_t* job_out) {
  if (!ctx) return QG_ERR_INVALID_ARG;
  NvtxRange nvtx("qg admit");
  return submit_one((Ctx*)ctx, circuit, options, job_out);
}

int qg_job_status(void* ctx, uint64_t job, int32_t* status_out) {
  if (!ctx || !status_out) return QG_ERR_INVALID_ARG;
  auto j = find_job((Ctx*)ctx, job);
  *status_out = j ? j->status.load() : QG_JOB_NOT_FOUND;
  return QG_OK;
}

int qg_wait(void* ctx, uint64_t job, int64_t timeout_ms, int32_t* status_out) {
  if (!ctx) return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  auto j = find_job(c, job);
  if (!j) {
    if (status_out) *status_out = QG_JOB_NOT_FOUND;
    return QG_ERR_NOT_FOUND;
  }
  std::unique_lock<std::mutex> lk(c->mu);
  auto pred = [&] {
    int s = j->status.load();
    return s == QG_JOB_COMPLETED || s == QG_JOB_FAILED || s == QG_JOB_CANCELLED;
  };
  bool ok = true;
  if (timeout_ms < 0) c->done_cv.wait(lk, pred);
  else ok = c->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred);
  if (status_out) *status_out = j->status.load();
  return ok ? QG_OK : QG_ERR_TIMEOUT;
}

int qg_cancel(void* ctx, uint64_t job, int32_t* outcome) {
  if (!ctx || !outcome) return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  std::lock_guard<std::mutex> g(c->mu);
  auto it = c->jobs.find(job);
  if (it == c->jobs.end()) {
    *outcome = QG_CANCEL_NOT_FOUND;
    return QG_OK;
  }
  Job* j = it->second.get();
  int s = j->status.load();
  if (s == QG_JOB_QUEUED) {
    j->cancel.store(true);
    j->status.store(QG_JOB_CANCELLED);
    j->finished = Clock::now();
    *outcome = QG_CANCEL_CANCELLED;
    c->done_cv.notify_all();
  } else if (s == QG_JOB_RUNNING) {
    j->cancel.store(true);  // the worker stops between passes
    *outcome = QG_CANCEL_CANCELLED;
  } else {
    *outcome = QG_CANCEL_CANNOT;
  }
  return QG_OK;
}

int qg_queue_status(void* ctx, qg_queue_info* out) {
  if (!ctx || !out) return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  std::memset(out, 0, sizeof(*out));
  std::lock_guard<std::mutex> g(c->mu);
  for (auto& kv : c->jobs) {
    ++out->total_jobs;
    switch (kv.second->status.load()) {
      case QG_JOB_QUEUED: ++out->queued; break;
      case QG_JOB_RUNNING: ++out->running; break;
      case QG_JOB_COMPLETED: ++out->completed; break;
      case QG_JOB_FAILED: ++out->failed; break;
      default: ++out->cancelled; break;
    }
  }
  size_t fr = 0, tot = 0;
  cudaSetDevice(c->device);
  cudaMemGetInfo(&fr, &tot);
  out->hbm_free_bytes = fr;
  out->hbm_budget_bytes = c->hbm_budget;
  out->hbm_in_use_bytes = c->hbm_in_use;
  out->workers = (int32_t)c->workers.size();
  {
    std::lock_guard<std::mutex> g2(c->pre_mu);
    out->precompiled_jobs = (int32_t)c->precompiled;
  }
  return QG_OK;
}

int qg_job_details(void* ctx, uint64_t job, qg_job_info* out) {
  if (!ctx || !out) return QG_ERR_INVALID_ARG;
  auto j = find_job((Ctx*)ctx, job);
  if (!j) return QG_ERR_NOT_FOUND;
  std::memset(out, 0, sizeof(*out));
  out->status = j->status.load();
  out->num_qubits = j->n;
  out->precision = j->precision;
  out->num_passes = j->passes;
  out->execution_time_ms = j->exec_ms;
  out->device_time_ms = j->device_ms;
  out->queue_time_ms = j->queue_ms;
  out->shots = j->shots.size();
  out->num_distinct_outcomes = (int64_t)j->counts.size();
  out->has_results = j->has & (j->state ? ~0 : ~QG_RES_STATE_VECTOR);
  out->error_code = j->error_code;
  out->batched_with = j->batched_with;
  out->specialised_passes = j->specialised;
  return QG_OK;
}

// common guard for result getters
static int completed_job(void* ctx, uint64_t job, std::shared_ptr<Job>* out) {
  if (!ctx) return QG_ERR_INVALID_ARG;
  auto j = find_job((Ctx*)ctx, job);
  if (!j) return QG_ERR_NOT_FOUND;
  int s = j->status.load();
  if (s == QG_JOB_CANCELLED) return QG_ERR_CANCELLED;
  if (s != QG_JOB_COMPLETED) return QG_ERR_NOT_COMPLETED;
  *out = j;
  return QG_OK;
}

int qg_result_counts(void* ctx, uint64_t job, uint64_t* outcomes, uint64_t* counts, int64_t cap, int64_t* n_out) {
  std::shared_ptr<Job> j;
  int rc = completed_job(ctx, job, &j);
  if (rc != QG_OK) return rc;
  if (!(j->has & QG_RES_MEASUREMENTS)) return QG_ERR_NO_RESULT;
  if (n_out) *n_out = (int64_t)j->counts.size();
  if (cap < (int64_t)j->counts.size()) return QG_ERR_BUFFER_TOO_SMALL;
  for (size_t i = 0; i < j->counts.size(); ++i) {
    if (outcomes) outcomes[i] = j->counts[i].first;
    if (counts) counts[i] = j->counts[i].second;
  }
  return QG_OK;
}

int qg_result_shots(void* ctx, uint64_t job, uint64_t* outcomes, int64_t cap) {
  std::shared_ptr<Job> j;
  int rc = completed_job(ctx, job, &j);
  if (rc != QG_OK) return rc;
  if (!(j->has & QG_RES_MEASUREMENTS)) return QG_ERR_NO_RESULT;
  if (cap < (int64_t)j->shots.size()) return QG_ERR_BUFFER_TOO_SMALL;
  if (!outcomes) return QG_ERR_INVALID_ARG;
  std::memcpy(outcomes, j->shots.data(), sizeof(uint64_t) * j->shots.size());
  return QG_OK;
}

int qg_result_probabilities(void* ctx, uint64_t job, double* out, int64_t cap) {
  std::shared_ptr<Job> j;
  int rc = completed_job(ctx, job, &j);
  if (rc != QG_OK) return rc;
  const uint64_t N = 1ULL << j->n;
  if (!out) return QG_ERR_INVALID_ARG;
  if (cap < (int64_t)N) return QG_ERR_BUFFER_TOO_SMALL;
  if (!j->probs.empty()) {
    std::memcpy(out, j->probs.data(), sizeof(double) * N);
    return QG_OK;
  }
  if (!j->state) return QG_ERR_NO_RESULT;
  std::string err;
  cudaSetDevice(((Ctx*)ctx)->device);
  rc = st_probs(j->state.get(), out, &err);
  if (rc != QG_OK) set_ctx_error((Ctx*)ctx, err);
  return rc;
}

int qg_result_target_probabilities(void* ctx, uint64_t job, double* out, int64_t cap) {
  std::shared_ptr<Job> j;
  int rc = completed_job(ctx, job, &j);
  if (rc != QG_OK) return rc;
  if (j->target_probs.empty() && !(j->has & QG_RES_PROBABILITIES)) return QG_ERR_NO_RESULT;
  if (cap < (int64_t)j->target_probs.size()) return QG_ERR_BUFFER_TOO_SMALL;
  if (!j->target_probs.empty()) std::memcpy(out, j->target_probs.data(), sizeof(double) * j->target_probs.size());
  return QG_OK;
}

int qg_result_state(void* ctx, uint64_t job, double* out, int64_t cap) {
  std::shared_ptr<Job> j;
  int rc = completed_job(ctx, job, &j);
  if (rc != QG_OK) return rc;
  if (!out) return QG_ERR_INVALID_ARG;
  if (!j->state) {
    set_ctx_error((Ctx*)ctx, "final state evicted; request :state-vector in the result spec to retain it");
    return QG_ERR_NO_RESULT;
  }
  if (cap < (int64_t)(1ULL << j->n)) return QG_ERR_BUFFER_TOO_SMALL;
  std::string err;
  cudaSetDevice(((Ctx*)ctx)->device);
  rc = download_c128(j->state.get(), out, &err);
  if (rc != QG_OK) set_ctx_error((Ctx*)ctx, err);
  return rc;
}

int qg_result_amplitudes(void* ctx, uint64_t job, double* out, int64_t cap) {
  std::shared_ptr<Job> j;
  int rc = completed_job(ctx, job, &j);
  if (rc != QG_OK) return rc;
  if (!(j->has & QG_RES_AMPLITUDES)) return QG_ERR_NO_RESULT;
  if (cap < (int64_t)(j->amplitudes.size() / 2)) return QG_ERR_BUFFER_TOO_SMALL;
  if (!j->amplitudes.empty()) std::memcpy(out, j->amplitudes.data(), sizeof(double) * j->amplitudes.size());
  return QG_OK;
}

int qg_result_expectations(void* ctx, uint64_t job, double* expectation, double* variance, int64_t cap) {
  std::shared_ptr<Job> j;
  int rc = completed_job(ctx, job, &j);
  if (rc != QG_OK) return rc;
  if (!(j->has & (QG_RES_EXPECTATION | QG_RES_VARIANCE))) return QG_ERR_NO_RESULT;
  if (cap < (int64_t)j->expectations.size()) return QG_ERR_BUFFER_TOO_SMALL;
  for (size_t i = 0; i < j->expectations.size(); ++i) {
    if (expectation) expectation[i] = j->expectations[i];
    if (variance) variance[i] = j->variances[i];
  }
  return QG_OK;
}

int qg_result_hamiltonian(void* ctx, uint64_t job, double* energy, double* term_values, int64_t cap) {
  std::shared_ptr<Job> j;
  int rc = completed_job(ctx, job, &j);
  if (rc != QG_OK) return rc;
  if (!(j->has & QG_RES_HAMILTONIAN)) return QG_ERR_NO_RESULT;
  if (energy) *energy = j->energy;
  if (term_values) {
    if (cap < (int64_t)j->term_values.size()) return QG_ERR_BUFFER_TOO_SMALL;
    std::memcpy(term_values, j->term_values.data(), sizeof(double) * j->term_values.size());
  }
  return QG_OK;
}

int qg_result_fidelities(void* ctx, uint64_t job, double* out, int64_t cap) {
  std::shared_ptr<Job> j;
  int rc = completed_job(ctx, job, &j);
  if (rc != QG_OK) return rc;
  if (!(j->has & QG_RES_FIDELITY)) return QG_ERR_NO_RESULT;
  if (cap < (int64_t)j->fidelities.size()) return QG_ERR_BUFFER_TOO_SMALL;
  if (!j->fidelities.empty()) std::memcpy(out, j->fidelities.data(), sizeof(double) * j->fidelities.size());
  return QG_OK;
}

int qg_result_accuracy(void* ctx, uint64_t job, double* out3) {
  if (!out3) return QG_ERR_INVALID_ARG;
  std::shared_ptr<Job> j;
  int rc = completed_job(ctx, job, &j);
  if (rc != QG_OK) return rc;
  if (!(j->has & QG_RES_ACCURACY)) return QG_ERR_NO_RESULT;
  std::memcpy(out3, j->accuracy, sizeof(j->accuracy));
  return QG_OK;
}

int qg_result_density_matrix(void* ctx, uint64_t job, double* out, int64_t cap) {
  std::shared_ptr<Job> j;
  int rc = completed_job(ctx, job, &j);
  if (rc != QG_OK) return rc;
  if (!(j->has & QG_RES_DENSITY_MATRIX)) return QG_ERR_NO_RESULT;
  if (cap < (int64_t)(j->density.size() / 2)) return QG_ERR_BUFFER_TOO_SMALL;
  std::memcpy(out, j->density.data(), sizeof(double) * j->density.size());
  return QG_OK;
}

int qg_last_error(void* ctx, uint64_t job, char* buf, int64_t len) {
  if (!ctx || !buf || len <= 0) return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  std::string msg;
  if (job) {
    auto j = find_job(c, job);
    if (!j) return QG_ERR_NOT_FOUND;
    msg = j->error;
  } else {
    std::lock_guard<std::mutex> g(c->err_mu);
    msg = c->last_error;
  }
  std::snprintf(buf, (size_t)len, "%s", msg.c_str());
  return QG_OK;
}

int qg_job_free(void* ctx, uint64_t job) {
  if (!ctx) return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  std::shared_ptr<Job> j;
  {
    std::lock_guard<std::mutex> g(c->mu);
    auto it = c->jobs.find(job);
    if (it == c->jobs.end()) return QG_ERR_NOT_FOUND;
    int s = it->second->status.load();
    if (s == QG_JOB_RUNNING || s == QG_JOB_QUEUED) return QG_ERR_NOT_COMPLETED;
    j = it->second;
    c->jobs.erase(it);
    if (j->state) {
      c->hbm_in_use -= std::min(c->hbm_in_use, job_bytes(j->n, j->state->prec));
    }
  }
  if (j->state) {
    cudaSetDevice(c->device);
    cudaStream_t st = j->state->stream;
    state_release(j->state.get());
    cudaStreamSynchronize(st);
    if (j->state->own_stream) cudaStreamDestroy(st);
    j->state.reset();
  }
  c->cv.notify_all();
  return QG_OK;
}

int qg_cleanup_completed(void* ctx, int64_t max_age_ms, int64_t* removed) {
  if (!ctx) return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  std::vector<uint64_t> old;
  {
    std::lock_guard<std::mutex> g(c->mu);
    auto now = Clock::now();
    for (auto& kv : c->jobs) {
      Job* j = kv.second.get();
      if (j->status.load() != QG_JOB_COMPLETED) continue;
      double age = std::chrono::duration<double, std::milli>(now - j->finished).count();
      if (age > (double)max_age_ms) old.push_back(kv.first);
    }
  }
  for (uint64_t id : old) qg_job_free(ctx, id);
  if (removed) *removed = (int64_t)old.size();
  return QG_OK;
}

int qg_batch_submit(void* ctx, const qg_circuit* circuits, int32_t count, const qg_options* options,
                    uint64_t* batch_out, uint64_t* jobs_out) {
  if (!ctx || !circuits || count < 0 || !batch_out) return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  // all or nothing: every circuit is validated before any job is queued
  std::vector<std::shared_ptr<Job>> js((size_t)count);
  for (int i = 0; i < count; ++i) {
    const int rc = prepare_job(c, &circuits[i], options, &js[(size_t)i]);
    if (rc != QG_OK) return rc;
  }
  uint64_t bid;
  {
    std::lock_guard<std::mutex> g(c->mu);
    bid = c->next_id++;
    c->batches[bid];
  }
  enqueue_jobs(c, js, bid, jobs_out);
  *batch_out = bid;
  return QG_OK;
}

int qg_batch_status(void* ctx, uint64_t batch, int32_t* statuses, int32_t cap, int32_t* n_out) {
  if (!ctx) return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  std::lock_guard<std::mutex> g(c->mu);
  auto it = c->batches.find(batch);
  if (it == c->batches.end()) return QG_ERR_NOT_FOUND;
  if (n_out) *n_out = (int32_t)it->second.size();
  if (cap < (int32_t)it->second.size()) return QG_ERR_BUFFER_TOO_SMALL;
  for (size_t i = 0; i < it->second.size(); ++i) {
    auto jt = c->jobs.find(it->second[i]);
    statuses[i] = jt == c->jobs.end() ? QG_JOB_NOT_FOUND : jt->second->status.load();
  }
  return QG_OK;
}

int qg_batch_jobs(void* ctx, uint64_t batch, uint64_t* jobs, int32_t cap, int32_t* n_out) {
  if (!ctx) return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  std::lock_guard<std::mutex> g(c->mu);
  auto it = c->batches.find(batch);
  if (it == c->batches.end()) return QG_ERR_NOT_FOUND;
  if (n_out) *n_out = (int32_t)it->second.size();
  if (cap < (int32_t)it->second.size()) return QG_ERR_BUFFER_TOO_SMALL;
  for (size_t i = 0; i < it->second.size(); ++i) jobs[i] = it->second[i];
  return QG_OK;
}

// ---- device-resident state ---------------------------------------------------
int qg_state_create(void* ctx, int32_t n, int32_t precision, void** state_out) {
  if (!ctx || !state_out || n < 1 || n > QG_MAX_QUBITS) return QG_ERR_INVALID_ARG;
  if (precision != QG_C128 && precision != QG_C64) return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  cudaSetDevice(c->device);
  auto* s = new State();
  s->ctx = c;
  s->own_stream = true;
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete s;
    return QG_ERR_DEVICE;
  }
  std::string err;
  int rc = state_alloc(s, n, precision, s->stream, &err);
  if (rc == QG_OK) {
    cudaError_t e = launch_set_basis(s->d, precision, n, 0, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) rc = cuda_fail(&err, e, "zero-state");
  }
  if (rc != QG_OK) {
    set_ctx_error(c, err);
    state_release(s);
    cudaStreamSynchronize(s->stream);
    cudaStreamDestroy(s->stream);
    delete s;
    return rc == QG_ERR_DEVICE ? QG_ERR_OOM : rc;
  }
  *state_out = s;
  return QG_OK;
}

int qg_state_destroy(void* state) {
  if (!state) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  cudaSetDevice(s->ctx->device);
  state_release(s);
  cudaStreamSynchronize(s->stream);
  if (s->own_stream) cudaStreamDestroy(s->stream);
  delete s;
  return QG_OK;
}

int qg_state_num_qubits(void* state, int32_t* n, int32_t* precision) {
  if (!state) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  if (n) *n = s->n;
  if (precision) *precision = s->prec;
  return QG_OK;
}

static int state_err(State* s, int rc, const std::string& err) {
  if (rc != QG_OK) set_ctx_error(s->ctx, err);
  return rc;
}

int qg_state_set_basis(void* state, uint64_t index) {
  if (!state) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  if (index >= (1ULL << s->n)) return QG_ERR_INVALID_ARG;
  cudaSetDevice(s->ctx->device);
  cudaError_t e = launch_set_basis(s->d, s->prec, s->n, index, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  std::string err;
  return state_err(s, e == cudaSuccess ? QG_OK : cuda_fail(&err, e, "set_basis"), err);
}

int qg_state_upload(void* state, const double* host) {
  if (!state || !host) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  cudaSetDevice(s->ctx->device);
  std::string err;
  int rc = upload_c128(s, host, &err);
  if (rc == QG_OK && cudaStreamSynchronize(s->stream) != cudaSuccess) rc = QG_ERR_DEVICE;
  return state_err(s, rc, err);
}

int qg_state_download(void* state, double* host) {
  if (!state || !host) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  cudaSetDevice(s->ctx->device);
  std::string err;
  return state_err(s, download_c128(s, host, &err), err);
}

int qg_state_apply(void* state, const qg_circuit* circuit, int32_t fusion, uint64_t seed, int32_t* passes_out) {
  if (!state || !circuit) return QG_ERR_INVALID_ARG;
  NvtxRange nvtx("qg apply");
  State* s = (State*)state;
  if (circuit->num_qubits != s->n) {
    set_ctx_error(s->ctx, "circuit and state have mismatched number of qubits");
    return QG_ERR_INVALID_ARG;
  }
  cudaSetDevice(s->ctx->device);
  std::string err;
  Program prog;
  qg_tuning tu;
  const qg_tuning* tune = tuning_for(s->ctx, s->n, s->prec, s->ctx->cfg.arithmetic, fusion, &tu);
  int rc = compile_program(circuit, s->prec, fusion, s->ctx->cfg.fuse_k, s->ctx->cfg.arithmetic, &prog, &err, true,
                           tune);
  if (rc != QG_OK) return state_err(s, rc, err);
  ExecStats st;
  rc = exec_program(s, prog, seed, nullptr, &st, &err);
  if (passes_out) *passes_out = st.passes;
  return state_err(s, rc, err);
}

int qg_state_prepare(void* state, const qg_circuit* circuit, int32_t fusion, double* compile_ms_out,
                     int32_t* specialised_out) {
  if (!state || !circuit) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  if (circuit->num_qubits != s->n) {
    set_ctx_error(s->ctx, "circuit and state have mismatched number of qubits");
    return QG_ERR_INVALID_ARG;
  }
  cudaSetDevice(s->ctx->device);
  std::string err;
  Program prog;
  qg_tuning tu;
  const qg_tuning* tune = tuning_for(s->ctx, s->n, s->prec, s->ctx->cfg.arithmetic, fusion, &tu);
  int rc = compile_program(circuit, s->prec, fusion, s->ctx->cfg.fuse_k, s->ctx->cfg.arithmetic, &prog, &err, true,
                           tune);
  if (rc != QG_OK) return state_err(s, rc, err);
  const auto t0 = Clock::now();
  auto pk = maybe_pass_kernels(s, prog);
  if (compile_ms_out) *compile_ms_out = ms_since(t0);
  int cnt = 0;
  if (pk)
    for (size_t i = 0; i < prog.steps.size(); ++i) cnt += pass_kernel_ready(*pk, i) ? 1 : 0;
  if (specialised_out) *specialised_out = cnt;
  return QG_OK;
}

int qg_state_probabilities(void* state, double* host_out) {
  if (!state || !host_out) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  cudaSetDevice(s->ctx->device);
  std::string err;
  return state_err(s, st_probs(s, host_out, &err), err);
}

int qg_state_sample(void* state, uint64_t shots, uint64_t seed, uint64_t* host_outcomes) {
  if (!state || (shots && !host_outcomes)) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  cudaSetDevice(s->ctx->device);
  std::string err;
  std::vector<uint64_t> out;
  int rc = st_sample(s, shots, seed, &out, &err);
  if (rc == QG_OK && shots) std::memcpy(host_outcomes, out.data(), sizeof(uint64_t) * shots);
  return state_err(s, rc, err);
}

// Same kernels and outcomes as qg_state_sample; the scratch is the file-scope array
// of noalloc.cu and the outcomes go to caller-owned device memory. Every scratch
// word is written by an earlier kernel of the same call before it is read, so
// nothing needs clearing between calls.
static int st_sample_noalloc(State* s, uint64_t shots, uint64_t seed, uint64_t* d_out, std::string* err) {
  if (s->n > kNoAllocSampleMaxQubits) {
    *err = "qg_state_sample_noalloc: " + std::to_string(s->n) + " qubits exceed its fixed scratch (at most " +
           std::to_string(kNoAllocSampleMaxQubits) + " qubits)";
    return QG_ERR_INVALID_ARG;
  }
  if (shots) {
    cudaPointerAttributes pa{};
    CK(cudaPointerGetAttributes(&pa, d_out), "outcome buffer attributes");
    const bool device_ok = pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged ||
                           (pa.type == cudaMemoryTypeHost && pa.devicePointer != nullptr);
    if (!device_ok || (pa.type == cudaMemoryTypeDevice && pa.device != s->ctx->device)) {
      *err = "qg_state_sample_noalloc: outcomes must be device memory of the state's device";
      return QG_ERR_INVALID_ARG;
    }
  }
  void* scratch = nullptr;
  size_t cap = 0;
  CK(noalloc_sample_scratch(s->ctx->device, &scratch, &cap), "sampler scratch address");
  const size_t need = sampler_scratch_bytes(s->n, shots);
  const size_t total_off = (need + 255) / 256 * 256;
  if (total_off + sizeof(double) > cap) {
    *err = "qg_state_sample_noalloc: sampler scratch too small";
    return QG_ERR_INVALID_ARG;
  }
  double* d_total = (double*)((char*)scratch + total_off);
  CK(launch_sample(s->d, s->prec, s->n, shots, seed, scratch, d_out, d_total, s->stream), "sample");
  double total = 0;
  CK(cudaMemcpyAsync(&total, d_total, sizeof(double), cudaMemcpyDeviceToHost, s->stream), "D2H total");
  CK(cudaStreamSynchronize(s->stream), "sync");
  const double norm_tol = s->prec == QG_C64 ? 1e-4 : 1e-8;
  if (std::fabs(total - 1.0) > norm_tol) {
    *err = "State is not properly normalized (total probability " + std::to_string(total) + ")";
    return QG_ERR_NOT_NORMALIZED;
  }
  return QG_OK;
}

int qg_state_sample_noalloc(void* state, uint64_t shots, uint64_t seed, uint64_t* device_outcomes) {
  if (!state || (shots && !device_outcomes)) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  cudaSetDevice(s->ctx->device);
  std::string err;
  return state_err(s, st_sample_noalloc(s, shots, seed, device_outcomes, &err), err);
}

int qg_state_pauli_expectation(void* state, const char* pauli, double* out) {
  if (!state || !pauli || !out) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  cudaSetDevice(s->ctx->device);
  std::string err;
  return state_err(s, st_pauli(s, pauli, out, &err), err);
}

int qg_state_hamiltonian(void* state, int32_t n_terms, const double* coeffs, const char* paulis, double* out) {
  if (!state || !out || n_terms < 0 || (n_terms && (!coeffs || !paulis))) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  cudaSetDevice(s->ctx->device);
  std::string err;
  double energy = 0;
  for (int k = 0; k < n_terms; ++k) {
    double v;
    int rc = st_pauli(s, paulis + (size_t)k * s->n, &v, &err);
    if (rc != QG_OK) return state_err(s, rc, err);
    double term = coeffs[k] * v;
    energy = k == 0 ? term : energy + term;
  }
  *out = energy;
  return QG_OK;
}

int qg_state_expectation_1q(void* state, const double* obs8, int32_t target, double* out) {
  if (!state || !obs8 || !out) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  cudaSetDevice(s->ctx->device);
  std::string err;
  return state_err(s, st_expect1q(s, obs8, target, out, &err), err);
}

int qg_state_norm2(void* state, double* out) {
  if (!state || !out) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  cudaSetDevice(s->ctx->device);
  std::string err;
  return state_err(s, st_norm2(s, out, &err), err);
}

int qg_state_inner(void* a, void* b, double* re, double* im) {
  if (!a || !b || !re || !im) return QG_ERR_INVALID_ARG;
  State* s = (State*)a;
  cudaSetDevice(s->ctx->device);
  std::string err;
  return state_err(s, st_inner(s, (State*)b, re, im, &err), err);
}

int qg_state_compare(void* state, void* reference, double* out3) {
  if (!state || !reference || !out3) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  cudaSetDevice(s->ctx->device);
  std::string err;
  return state_err(s, st_compare(s, (State*)reference, out3, &err), err);
}

int qg_state_measure(void* state, const int32_t* qubits, int32_t count, uint64_t seed, uint64_t* outcome_out,
                     double* probability_out) {
  if (!state || !qubits || count < 1 || count > 20) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  std::vector<int> qs(qubits, qubits + count);
  for (int q : qs)
    if (q < 0 || q >= s->n) return QG_ERR_QUBIT_RANGE;
  cudaSetDevice(s->ctx->device);
  std::string err;
  int rc = do_measure(s, qs, seed, 0, outcome_out, probability_out, &err);
  if (rc == QG_OK && cudaStreamSynchronize(s->stream) != cudaSuccess) rc = QG_ERR_DEVICE;
  return state_err(s, rc, err);
}

int qg_state_device_ptr(void* state, void** dptr, void** stream) {
  if (!state) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  if (dptr) *dptr = s->d;
  if (stream) *stream = (void*)s->stream;
  return QG_OK;
}

int qg_state_synchronize(void* state) {
  if (!state) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  return cudaStreamSynchronize(s->stream) == cudaSuccess ? QG_OK : QG_ERR_DEVICE;
}

int qg_state_profile(void* state, const qg_circuit* circuit, int32_t fusion, uint64_t seed, float* pass_ms,
                     int32_t* pass_kind, int32_t cap, int32_t* n_passes) {
  if (!state || !circuit || cap < 0) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  if (circuit->num_qubits != s->n) return QG_ERR_INVALID_ARG;
  cudaSetDevice(s->ctx->device);
  std::string err;
  Program prog;
  qg_tuning tu;
  const qg_tuning* tune = tuning_for(s->ctx, s->n, s->prec, s->ctx->cfg.arithmetic, fusion, &tu);
  int rc = compile_program(circuit, s->prec, fusion, s->ctx->cfg.fuse_k, s->ctx->cfg.arithmetic, &prog, &err, true,
                           tune);
  if (rc != QG_OK) return state_err(s, rc, err);
  std::vector<float> ms;
  std::vector<int> kinds;
  ExecStats st;
  st.pass_ms = &ms;
  st.pass_kind = &kinds;
  rc = exec_program(s, prog, seed, nullptr, &st, &err);
  if (n_passes) *n_passes = (int32_t)ms.size();
  if (rc != QG_OK) return state_err(s, rc, err);
  if ((int32_t)ms.size() > cap) return QG_ERR_BUFFER_TOO_SMALL;
  for (size_t i = 0; i < ms.size(); ++i) {
    if (pass_ms) pass_ms[i] = ms[i];
    if (pass_kind) pass_kind[i] = kinds[i];
  }
  return QG_OK;
}

int qg_pass_kernels_build(const qg_circuit* circuit, int32_t precision, int32_t arithmetic, int32_t* kernels_out,
                          double* compile_ms_out, char* err_buf, int64_t err_len) {
  if (!circuit || (precision != QG_C128 && precision != QG_C64)) return QG_ERR_INVALID_ARG;
  std::string err;
  Program prog;
  const bool table = (arithmetic & QG_PASS_BUILD_TABLE) != 0;
  const int arith =
      (arithmetic & ~QG_PASS_BUILD_TABLE) == QG_ARITH_DOUBLE_FLOAT ? QG_ARITH_DOUBLE_FLOAT : QG_ARITH_EXACT;
  // a sweep keeps every circuit's gates in order (its states share one pass structure)
  int rc = compile_program(circuit, precision, QG_FUSE_TILED, 4, arith, &prog, &err, !table);
  if (rc == QG_OK) {
    int kernels = 0;
    double ms = 0;
    const int r = pass_kernels_build_only(prog, precision, &kernels, &ms, &err, table);
    if (kernels_out) *kernels_out = kernels;
    if (compile_ms_out) *compile_ms_out = ms;
    if (r < 0) rc = QG_ERR_DEVICE;
    else if (r == 0 && pass_kernels_unavailable()) rc = QG_ERR_UNSUPPORTED;
  }
  if (err_buf && err_len > 0) {
    const size_t n = std::min<size_t>(err.size(), (size_t)err_len - 1);
    std::memcpy(err_buf, err.data(), n);
    err_buf[n] = 0;
  }
  return rc;
}

int qg_diag_dense_tc_stall(int32_t on) {
  g_dense_tc_stall.store(on ? 1 : 0);
  return QG_OK;
}

// The sampler's scratch holds the chunk sums first, then the block sums, then the block
// prefixes with the total T after them (sampler_scratch_bytes_at).
static int st_sample_sums(State* s, uint64_t* h_csum, uint64_t count, uint64_t* h_total, std::string* err) {
  const uint64_t N = 1ULL << s->n, ch = N < 32 ? N : 32, nch = N / ch, cpb = nch < 256 ? nch : 256,
                 nb = nch / cpb;
  if (count != nch) {
    *err = "qg_diag_sample_sums: count must be " + std::to_string(nch);
    return QG_ERR_INVALID_ARG;
  }
  void* d_scratch = nullptr;
  double* d_total = nullptr;
  CK(cudaMallocAsync(&d_scratch, sampler_scratch_bytes(s->n, 0), s->stream), "alloc sampler");
  CK(cudaMallocAsync((void**)&d_total, sizeof(double) * 2, s->stream), "alloc total");
  CK(launch_sample(s->d, s->prec, s->n, 0, 0, d_scratch, nullptr, d_total, s->stream), "sample sums");
  const uint64_t* d_q = (const uint64_t*)d_scratch;
  CK(cudaMemcpyAsync(h_csum, d_q, sizeof(uint64_t) * nch, cudaMemcpyDeviceToHost, s->stream), "D2H chunk sums");
  CK(cudaMemcpyAsync(h_total, d_q + nch + nb + nb, sizeof(uint64_t), cudaMemcpyDeviceToHost, s->stream),
     "D2H total");
  CK(cudaStreamSynchronize(s->stream), "sync");
  cudaFreeAsync(d_scratch, s->stream);
  cudaFreeAsync(d_total, s->stream);
  return QG_OK;
}

int qg_diag_sample_sums(void* state, uint64_t* chunk_sums, uint64_t count, uint64_t* total) {
  if (!state || !chunk_sums || !total) return QG_ERR_INVALID_ARG;
  State* s = (State*)state;
  cudaSetDevice(s->ctx->device);
  std::string err;
  return state_err(s, st_sample_sums(s, chunk_sums, count, total, &err), err);
}

int qg_pass_kernels_info(int32_t* available, uint64_t* cache_hits, uint64_t* cache_misses) {
  if (available) *available = pass_kernels_unavailable() ? 0 : 1;
  size_t h = 0, m = 0;
  pass_kernel_cache_stats(&h, &m);
  if (cache_hits) *cache_hits = h;
  if (cache_misses) *cache_misses = m;
  return QG_OK;
}

// ---------------------------------------------------------------------------
// Autotuner: the specialised pass kernels' tile size and launch shape per
// (qubits, precision), chosen from measured device time on a calibration circuit.
// ---------------------------------------------------------------------------
int32_t qg_tuning_pick(const double* ms, const int32_t* valid, int32_t count, int32_t default_index,
                       double tie_frac) {
  if (!ms || !valid || count < 1) return -1;
  int best = -1;
  for (int i = 0; i < count; ++i)
    if (valid[i] && ms[i] > 0 && (best < 0 || ms[i] < ms[best])) best = i;
  if (best < 0) return -1;
  // the default shape stays unless another one is faster by more than tie_frac
  if (default_index >= 0 && default_index < count && valid[default_index] && ms[default_index] > 0 &&
      ms[default_index] <= ms[best] * (1.0 + (tie_frac > 0 ? tie_frac : 0)))
    return default_index;
  return best;
}

static bool tuning_valid(const qg_tuning& t, int n, int prec) {
  const int E = prec == QG_C128 ? 16 : 8;
  if (t.tile_bits < 10 || t.tile_bits > kMaxTileBits || t.tile_bits > n) return false;
  if (t.reg_bits < 3 || t.reg_bits > 4 || t.tile_bits - t.reg_bits < 5 || t.tile_bits - t.reg_bits > 10) return false;
  if (t.buffers < 1 || t.buffers > 3 || t.ctas_per_sm < 1 || t.ctas_per_sm > 8) return false;
  const long smem = (long)t.buffers * (1L << t.tile_bits) * E;
  return smem <= 227L * 1024 && smem * t.ctas_per_sm <= 228L * 1024;
}

int qg_tuning_set(void* ctx, int32_t n, int32_t precision, const qg_tuning* t) {
  if (!ctx || !t || n < 1 || n > QG_MAX_QUBITS || (precision != QG_C128 && precision != QG_C64))
    return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  std::lock_guard<std::mutex> lk(c->tune_mu);
  if (t->tile_bits == 0) {  // back to the default shape
    c->tunings.erase({n, precision});
    return QG_OK;
  }
  if (!tuning_valid(*t, n, precision)) return QG_ERR_INVALID_ARG;
  c->tunings[{n, precision}] = *t;
  return QG_OK;
}

int qg_tuning_get(void* ctx, int32_t n, int32_t precision, qg_tuning* out) {
  if (!ctx || !out) return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  std::lock_guard<std::mutex> lk(c->tune_mu);
  auto it = c->tunings.find({n, precision});
  if (it != c->tunings.end()) {
    *out = it->second;
    return QG_OK;
  }
  std::memset(out, 0, sizeof(*out));
  out->tile_bits = std::min(12, (int)n);
  out->reg_bits = precision == QG_C128 ? 3 : 4;
  out->buffers = 2;
  out->ctas_per_sm = precision == QG_C128 ? 1 : 2;
  return QG_OK;
}

// The calibration circuit: `depth` layers of the layered recipe (one gate from
// {H,X,Y,Z,S,T,RX,RY,RZ} per qubit, CNOTs on a random matching) and the first four
// columns of a QFT (H and controlled phases pi/2^k), from a fixed seed.
static std::vector<qg_op> calibration_ops(int n, int depth) {
  std::vector<qg_op> ops;
  uint64_t x = 0x9E3779B97F4A7C15ull;
  auto rnd = [&]() {
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    return x;
  };
  const int gates[9] = {QG_OP_H, QG_OP_X, QG_OP_Y, QG_OP_Z, QG_OP_S, QG_OP_T, QG_OP_RX, QG_OP_RY, QG_OP_RZ};
  auto op1 = [&](int code, int q, double a) {
    qg_op o;
    std::memset(&o, 0, sizeof(o));
    o.opcode = (uint16_t)code;
    o.nq = 1;
    o.q[0] = (uint32_t)q;
    o.angle = a;
    ops.push_back(o);
  };
  auto op2 = [&](int code, int a, int b, double ang) {
    qg_op o;
    std::memset(&o, 0, sizeof(o));
    o.opcode = (uint16_t)code;
    o.nq = 2;
    o.q[0] = (uint32_t)a;
    o.q[1] = (uint32_t)b;
    o.angle = ang;
    ops.push_back(o);
  };
  std::vector<int> perm(n);
  for (int d = 0; d < depth; ++d) {
    for (int q = 0; q < n; ++q) op1(gates[rnd() % 9], q, (double)(rnd() % 100000) * 6.283185307179586e-5);
    for (int q = 0; q < n; ++q) perm[q] = q;
    for (int q = n - 1; q > 0; --q) std::swap(perm[q], perm[rnd() % (q + 1)]);
    for (int q = 0; q + 1 < n; q += 2) op2(QG_OP_CNOT, perm[q], perm[q + 1], 0.0);
  }
  for (int j = 0; j < std::min(4, n); ++j) {
    op1(QG_OP_H, j, 0.0);
    for (int k = j + 1; k < n; ++k) op2(QG_OP_RYDBERG_CPHASE, k, j, 3.141592653589793 / (double)(1ull << (k - j)));
  }
  return ops;
}

int qg_autotune(void* ctx, int32_t n, int32_t precision, const qg_circuit* calibration, qg_tuning* chosen,
                qg_tuning* tried, int32_t cap, int32_t* count_out) {
  if (!ctx || !chosen || n < 11 || n > QG_MAX_QUBITS || (precision != QG_C128 && precision != QG_C64))
    return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  NvtxRange nvtx("qg autotune");
  if (const char* why = pass_kernels_unavailable()) {
    set_ctx_error(c, std::string("autotune: ") + why);
    return QG_ERR_UNSUPPORTED;
  }
  const int arith = c->cfg.arithmetic;
  if (precision == QG_C128 && arith != QG_ARITH_DOUBLE_FLOAT) {
    set_ctx_error(c, "autotune: complex128 exact arithmetic runs interpreted (nothing to tune)");
    return QG_ERR_UNSUPPORTED;
  }
  if (!will_specialise(c, n, precision, arith, QG_FUSE_TILED)) {
    set_ctx_error(c, "autotune: states of " + std::to_string(n) +
                         " qubits run interpreted under this context's pass-kernel policy (nothing to tune)");
    return QG_ERR_UNSUPPORTED;
  }
  // candidates: the default first (tile bits, register bits, buffers, CTAs per SM)
  std::vector<qg_tuning> cand;
  auto add = [&](int k, int r, int b, int ct) {
    qg_tuning t;
    std::memset(&t, 0, sizeof(t));
    t.tile_bits = k;
    t.reg_bits = r;
    t.buffers = b;
    t.ctas_per_sm = ct;
    if (tuning_valid(t, n, precision)) cand.push_back(t);
  };
  if (precision == QG_C128) {
    add(12, 3, 2, 1);
    add(11, 3, 2, 2);
    add(12, 3, 1, 1);
    add(11, 3, 1, 2);
    add(10, 3, 2, 4);
  } else {
    add(12, 4, 2, 2);
    add(11, 4, 2, 4);
    add(13, 4, 2, 1);
    add(12, 4, 1, 2);
    add(10, 4, 2, 8);
  }
  if (calibration && calibration->num_qubits != n) {
    set_ctx_error(c, "autotune: the calibration circuit has a different number of qubits");
    return QG_ERR_INVALID_ARG;
  }
  cudaSetDevice(c->device);
  std::vector<qg_op> ops = calibration_ops(n, 6);
  qg_circuit circ = calibration ? *calibration : qg_circuit{n, (int32_t)ops.size(), ops.data()};
  void* sh = nullptr;
  int rc = qg_state_create(ctx, n, precision, &sh);
  if (rc != QG_OK) return rc;
  State* s = (State*)sh;
  std::vector<double> ms(cand.size(), 0.0);
  std::vector<int32_t> ok(cand.size(), 0);
  std::string err;
  for (size_t i = 0; i < cand.size(); ++i) {
    Program prog;
    rc = compile_program(&circ, precision, QG_FUSE_TILED, c->cfg.fuse_k, arith, &prog, &err, true, &cand[i]);
    if (rc != QG_OK) break;
    std::string why;
    auto pk = pass_kernels_for(prog, precision, c->device, &why);
    if (!pk) continue;  // this shape did not compile: not a candidate
    // one warm-up run, then the median of three
    std::vector<double> runs;
    for (int r = 0; r < 4 && rc == QG_OK; ++r) {
      ExecStats st;
      rc = exec_program(s, prog, 0, nullptr, &st, &err);
      if (r > 0) runs.push_back(st.device_ms);
    }
    if (rc != QG_OK) break;
    std::sort(runs.begin(), runs.end());
    ms[i] = runs[runs.size() / 2];
    ok[i] = 1;
    cand[i].ms = ms[i];
  }
  qg_state_destroy(sh);
  if (rc != QG_OK) {
    set_ctx_error(c, "autotune: " + err);
    return rc;
  }
  const int pick = qg_tuning_pick(ms.data(), ok.data(), (int32_t)cand.size(), 0, 0.01);
  if (pick < 0) {
    set_ctx_error(c, "autotune: no candidate shape compiled");
    return QG_ERR_UNSUPPORTED;
  }
  *chosen = cand[pick];
  {
    std::lock_guard<std::mutex> lk(c->tune_mu);
    c->tunings[{n, precision}] = cand[pick];
  }
  if (count_out) *count_out = (int32_t)cand.size();
  if (tried)
    for (int i = 0; i < (int)cand.size() && i < cap; ++i) tried[i] = cand[i];
  return QG_OK;
}

// The specialisation crossover for one-off circuits: for each state size, a fresh
// calibration job of `layers` layers (never seen before, so its kernels compile cold)
// runs interpreted and specialised; the crossover is the smallest size from which
// compile wall time + specialised run beats the interpreted run at every larger size
// measured. Under QG_PASS_KERNELS_AUTO the context then specialises from there on.
int qg_autotune_crossover(void* ctx, int32_t precision, int32_t layers, int32_t* min_qubits_out, double* table,
                          int32_t cap, int32_t* count_out) {
  if (!ctx || !min_qubits_out || layers < 1 || (precision != QG_C128 && precision != QG_C64))
    return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  NvtxRange nvtx("qg autotune crossover");
  if (const char* why = pass_kernels_unavailable()) {
    set_ctx_error(c, std::string("autotune crossover: ") + why);
    return QG_ERR_UNSUPPORTED;
  }
  const int arith = c->cfg.arithmetic;
  if (precision == QG_C128 && arith != QG_ARITH_DOUBLE_FLOAT) {
    set_ctx_error(c, "autotune crossover: complex128 exact arithmetic runs interpreted");
    return QG_ERR_UNSUPPORTED;
  }
  static std::atomic<int> salt{0};
  cudaSetDevice(c->device);
  const int sizes[] = {20, 22, 24, 26, 28, 30};
  std::vector<std::array<double, 4>> rows;
  std::string err;
  int rc = QG_OK;
  for (int n : sizes) {
    if (n > QG_MAX_QUBITS) break;
    std::vector<qg_op> ops = calibration_ops(n, layers);
    // a distinct angle per call: the program is new to the kernel cache
    const int sl = salt.fetch_add(1);
    for (qg_op& o : ops)
      if (o.opcode == QG_OP_RX || o.opcode == QG_OP_RY || o.opcode == QG_OP_RZ) {
        o.angle += 1e-9 * (double)(sl + 1);
        break;
      }
    qg_circuit circ{n, (int32_t)ops.size(), ops.data()};
    void* sh = nullptr;
    rc = qg_state_create(ctx, n, precision, &sh);
    if (rc != QG_OK) break;
    State* s = (State*)sh;
    Program prog;
    rc = compile_program(&circ, precision, QG_FUSE_TILED, c->cfg.fuse_k, arith, &prog, &err);
    double interp = 0, spec = 0, comp = 0;
    if (rc == QG_OK) {
      // interpreted, then a cold compile, then specialised (the kernels just compiled)
      ExecStats st;
      rc = exec_program(s, prog, 0, nullptr, &st, &err, 0);
      interp = st.device_ms;
      if (rc == QG_OK) {
        std::string why;
        const auto t0 = Clock::now();
        auto pk = pass_kernels_for(prog, precision, c->device, &why);
        comp = ms_since(t0);
        if (!pk) {
          err = "pass kernels: " + why;
          rc = QG_ERR_UNSUPPORTED;
        } else {
          ExecStats st2;
          rc = exec_program(s, prog, 0, nullptr, &st2, &err, 1);
          spec = st2.device_ms;
        }
      }
    }
    qg_state_destroy(sh);
    if (rc != QG_OK) break;
    rows.push_back({(double)n, interp, comp, spec});
  }
  if (rc != QG_OK) {
    set_ctx_error(c, "autotune crossover: " + err);
    return rc;
  }
  // from the largest size down, as long as compiling and running specialised wins
  int cross = rows.empty() ? kPassKernelMinQubits : (int)rows.back()[0] + 1;
  for (int i = (int)rows.size() - 1; i >= 0; --i) {
    if (rows[i][2] + rows[i][3] < rows[i][1]) cross = (int)rows[i][0];
    else break;
  }
  c->spec_min_qubits[precision == QG_C64 ? 1 : 0].store(cross);
  *min_qubits_out = cross;
  if (count_out) *count_out = (int32_t)rows.size();
  if (table)
    for (int i = 0; i < (int)rows.size() && i < cap; ++i)
      for (int q = 0; q < 4; ++q) table[4 * i + q] = rows[i][q];
  return QG_OK;
}

int qg_kernel_launches(uint64_t* count) {
  if (!count) return QG_ERR_INVALID_ARG;
  *count = kernel_launch_count();
  return QG_OK;
}

}  // extern "C"

// ===========================================================================
// Parameter sweeps (batched states of one structure, CUDA-graph replays)
// ===========================================================================
namespace qg {

struct SweepGroup {
  int n = 0;
  std::vector<int> members;              // circuit indices
  std::vector<Program> progs;            // one per member; equal pass structure
  std::vector<int> pass_steps;           // TILE_PASS step indices
  std::vector<int64_t> pass_off;         // first op record of each pass in d_kops
  std::vector<int> pass_nops;
  bool batched = true;                   // false: members run one by one (small or measured circuits)
  void* slab = nullptr;
  void** d_states = nullptr;
  void* d_kops = nullptr;
  std::vector<unsigned char> kops_host;
  std::vector<std::unique_ptr<State>> views;
  cudaGraphExec_t exec = nullptr;
  int launches = 0;
  // table-form specialised kernels (one per pass, shared by the members), or null
  std::shared_ptr<const PassKernels> pk;
  float* d_coefs = nullptr;               // per pass: [member][16 x ops] matrix entries
  std::vector<float> coefs_host;
  std::vector<int64_t> coef_off;          // first float of each pass's rows
  // energy tables of the diagonal path (kept between runs with equal terms)
  bool diag = false;
  void* d_diag = nullptr;
  uint64_t* d_z = nullptr;                // nz z-masks, then nz 16-bit q-patterns (uint32)
  size_t nz = 0;
  double* d_gcoef = nullptr;
  double* d_epart = nullptr;
  double* d_en = nullptr;
};

struct Sweep {
  Ctx* ctx = nullptr;
  int prec = QG_C128, arith = QG_ARITH_EXACT;
  cudaStream_t stream = nullptr;
  int count = 0;
  std::vector<SweepGroup> groups;
  // level kernels: one launch per pass level over every group in lk_groups (sizes
  // side by side), after one launch that sets all their states to |0...0>
  std::shared_ptr<const PassKernels> lk;
  std::vector<int> lk_groups;              // sweep groups run by the level kernels
  std::vector<char> in_level;              // per group: run by the level kernels
  GroupLevelDesc* d_levels = nullptr;      // descriptors of every level, level after level
  cudaGraphExec_t lk_exec = nullptr;
  int lk_launches = 0;
  float level_ms = 0, group_ms = 0;        // measured at creation: level graph, per-size graphs
  std::vector<std::pair<int, int>> where;  // circuit -> (group, member)
  uint64_t bytes = 0;
  // the term arrays the energy tables were built from
  bool e_valid = false;
  std::vector<int32_t> e_offsets;
  std::vector<double> e_coefs;
  std::string e_strings;
};

static std::vector<int64_t> pass_signature(const Program& p) {
  std::vector<int64_t> sig{p.n};
  for (const Step& s : p.steps) {
    if (s.kind != Step::TILE_PASS) {
      sig.push_back(-1 - (int)s.kind);
      continue;
    }
    sig.push_back(s.pass.k);
    sig.push_back(s.pass.klow);
    for (int j = 0; j < s.pass.k; ++j) sig.push_back(s.pass.lbits[j]);
    sig.push_back(s.pass.op_end - s.pass.op_begin);
  }
  return sig;
}

static int view_init(State* v, Ctx* c, void* d, int n, int prec, cudaStream_t st, std::string* err) {
  v->ctx = c;
  v->n = n;
  v->prec = prec;
  v->d = d;
  v->bytes = amp_bytes(prec) << n;
  v->stream = st;
  v->nblocks = reduce_blocks_for(n);
  CK(cudaMallocAsync((void**)&v->d_part, sizeof(double) * 4 * v->nblocks, st), "alloc partials");
  CK(cudaMallocAsync((void**)&v->d_self, sizeof(void*), st), "alloc self");
  CK(cudaMemcpyAsync(v->d_self, &v->d, sizeof(void*), cudaMemcpyHostToDevice, st), "H2D self");
  return QG_OK;
}

static void encode_group_kops(Sweep* sw, SweepGroup& g) {
  const size_t rec = kop_record_bytes();
  for (size_t p = 0; p < g.pass_steps.size(); ++p)
    for (size_t m = 0; m < g.members.size(); ++m) {
      const Program& pr = g.progs[m];
      const PassDesc& pd = pr.steps[g.pass_steps[p]].pass;
      encode_kops(sw->prec, pr.arith, pr.tops.data() + pd.op_begin, pd.op_end - pd.op_begin,
                  g.kops_host.data() + rec * (size_t)(g.pass_off[p] + (int64_t)m * g.pass_nops[p]));
    }
}

static void encode_group_coefs(Sweep* sw, SweepGroup& g) {
  for (size_t p = 0; p < g.pass_steps.size(); ++p) {
    const size_t row = 16 * (size_t)g.pass_nops[p];
    for (size_t m = 0; m < g.members.size(); ++m)
      pass_coefficients(g.progs[m], (size_t)g.pass_steps[p], sw->prec,
                        g.coefs_host.data() + g.coef_off[p] + row * m);
  }
}

// Table-form kernels for a batched group whose members share one structure:
// compiled once (cached by structure), coefficients uploaded per member.
static void setup_group_pass_kernels(Sweep* sw, SweepGroup& g) {
  const Ctx* c = sw->ctx;
  if (c->cfg.pass_kernels == QG_PASS_KERNELS_OFF) return;
  if (sw->prec == QG_C128 && sw->arith != QG_ARITH_DOUBLE_FLOAT) return;
  const std::string k0 = pass_structure_key(g.progs[0], true);
  for (size_t m = 1; m < g.progs.size(); ++m)
    if (pass_structure_key(g.progs[m], true) != k0) return;
  std::string why;
  auto pk = pass_kernels_for(g.progs[0], sw->prec, c->device, &why, true);
  if (!pk) return;
  for (int ps : g.pass_steps)
    if (!pass_kernel_ready(*pk, (size_t)ps)) return;
  int64_t off = 0;
  g.coef_off.clear();
  for (size_t p = 0; p < g.pass_steps.size(); ++p) {
    g.coef_off.push_back(off);
    off += 16 * (int64_t)g.pass_nops[p] * (int64_t)g.members.size();
  }
  g.coefs_host.assign((size_t)std::max<int64_t>(off, 1), 0.0f);
  encode_group_coefs(sw, g);
  if (cudaMallocAsync((void**)&g.d_coefs, sizeof(float) * g.coefs_host.size(), sw->stream) != cudaSuccess) {
    g.d_coefs = nullptr;
    cudaGetLastError();
    return;
  }
  if (cudaMemcpyAsync(g.d_coefs, g.coefs_host.data(), sizeof(float) * g.coefs_host.size(), cudaMemcpyHostToDevice,
                      sw->stream) != cudaSuccess) {
    cudaFreeAsync(g.d_coefs, sw->stream);
    g.d_coefs = nullptr;
    return;
  }
  g.pk = pk;
}

static cudaError_t launch_group_passes(Sweep* sw, SweepGroup& g) {
  const size_t rec = kop_record_bytes();
  cudaError_t e = launch_batch_zero(g.slab, sw->prec, g.n, (int)g.members.size(), sw->stream);
  for (size_t p = 0; p < g.pass_steps.size() && e == cudaSuccess; ++p) {
    if (g.pk) {
      e = launch_pass_kernel_batch(*g.pk, (size_t)g.pass_steps[p], g.n, g.progs[0].steps[g.pass_steps[p]].pass,
                                   g.d_states, (int)g.members.size(), g.d_coefs + g.coef_off[p], sw->prec,
                                   sw->stream);
      continue;
    }
    PassDesc pd = g.progs[0].steps[g.pass_steps[p]].pass;
    pd.op_begin = 0;
    pd.op_end = g.pass_nops[p];
    e = launch_tile_pass(sw->prec, g.progs[0].arith, tile_pass_io(g.progs[0], g.pass_steps[p]), g.n, pd,
                         g.d_states, (int)g.members.size(),
                         (const unsigned char*)g.d_kops + rec * (size_t)g.pass_off[p], g.pass_nops[p], nullptr,
                         sw->stream);
  }
  return e;
}

// Level kernels over the batched groups that have table-form kernels: their states are
// set to |0...0> in one launch and pass level l of all of them runs in one launch
// (qgl_<l>), the whole captured in one graph. A sweep of one group keeps its own graph.
constexpr float kLevelGraphMargin = 1.02f;  // level graph kept up to 2 % slower than the per-size graphs

static void setup_level_kernels(Sweep* sw) {
  std::vector<int> cand;
  for (size_t gi = 0; gi < sw->groups.size(); ++gi) {
    const SweepGroup& g = sw->groups[gi];
    if (g.batched && g.pk && g.d_coefs && !g.pass_steps.empty()) cand.push_back((int)gi);
  }
  sw->in_level.assign(sw->groups.size(), 0);
  if (cand.size() < 2 || cand.size() > (size_t)kMaxZeroGroups) return;
  std::vector<const Program*> progs;
  std::vector<std::vector<int>> steps;
  for (int gi : cand) {
    progs.push_back(&sw->groups[gi].progs[0]);
    steps.push_back(sw->groups[gi].pass_steps);
  }
  std::string why;
  auto lk = level_kernels_for(progs, steps, sw->prec, sw->ctx->device, &why);
  if (!lk) return;
  const int L = level_count(*lk);
  std::vector<GroupLevelDesc> desc;
  std::vector<size_t> off(L);
  std::vector<uint64_t> total(L, 0);
  for (int l = 0; l < L; ++l) {
    off[l] = desc.size();
    for (int q : level_groups(*lk, l)) {
      const SweepGroup& g = sw->groups[cand[q]];
      const PassDesc& pd = g.progs[0].steps[g.pass_steps[l]].pass;
      GroupLevelDesc d;
      d.states = g.d_states;
      d.coefs = g.d_coefs + g.coef_off[l];
      d.ncoef = 16 * g.pass_nops[l];
      d.nstates = (int32_t)g.members.size();
      d.ntiles = 1ULL << (g.n - pd.k);
      d.item0 = total[l];
      d.items = d.ntiles * (uint64_t)d.nstates;
      total[l] += d.items;
      desc.push_back(d);
    }
  }
  if (cudaMallocAsync((void**)&sw->d_levels, sizeof(GroupLevelDesc) * desc.size(), sw->stream) != cudaSuccess ||
      cudaMemcpyAsync(sw->d_levels, desc.data(), sizeof(GroupLevelDesc) * desc.size(), cudaMemcpyHostToDevice,
                      sw->stream) != cudaSuccess ||
      cudaStreamSynchronize(sw->stream) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  MultiZero z;
  std::memset(&z, 0, sizeof(z));
  for (int gi : cand) {
    const SweepGroup& g = sw->groups[gi];
    z.slab[z.ngroups] = g.slab;
    z.per[z.ngroups] = 1ULL << g.n;
    z.nstates[z.ngroups] = (int32_t)g.members.size();
    ++z.ngroups;
  }
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  if (cudaStreamBeginCapture(sw->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  cudaError_t le = launch_multi_zero(z, sw->prec, sw->stream);
  for (int l = 0; l < L && le == cudaSuccess; ++l) le = launch_level_kernel(*lk, l, sw->d_levels + off[l], total[l], sw->stream);
  cudaError_t ce = cudaStreamEndCapture(sw->stream, &graph);
  count_launch(-(1 + L));  // captured launches do not run here; replays count them
  if (le == cudaSuccess && ce == cudaSuccess && graph && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess) {
    // keep whichever form runs these groups faster: time both (second replay of each)
    auto time_ms = [&](auto&& run) {
      cudaEvent_t a, b;
      cudaEventCreate(&a);
      cudaEventCreate(&b);
      float best = -1.0f;
      for (int rep = 0; rep < 2; ++rep) {
        cudaEventRecord(a, sw->stream);
        const cudaError_t re = run();
        cudaEventRecord(b, sw->stream);
        if (re != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess) {
          best = -1.0f;
          break;
        }
        cudaEventElapsedTime(&best, a, b);
      }
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      return best;
    };
    const float t_level = time_ms([&]() { return cudaGraphLaunch(exec, sw->stream); });
    const float t_groups = time_ms([&]() {
      cudaError_t e = cudaSuccess;
      for (int gi : cand) {
        SweepGroup& g = sw->groups[gi];
        e = g.exec ? cudaGraphLaunch(g.exec, sw->stream) : launch_group_passes(sw, g);
        if (e != cudaSuccess) break;
      }
      return e;
    });
    sw->level_ms = t_level;
    sw->group_ms = t_groups;
    // The level graph is kept unless it is measurably slower: at equal speed one
    // launch per layer over every size beats a graph per size (fewer launches, and
    // the small sizes fill the SMs the large ones leave idle at their tails); one
    // replay's timing varies by about a percent, hence the margin.
    if (t_level > 0 && (t_groups <= 0 || t_level <= kLevelGraphMargin * t_groups)) {
      sw->lk = lk;
      sw->lk_exec = exec;
      sw->lk_launches = 1 + L;
      sw->lk_groups = cand;
      for (int gi : cand) sw->in_level[gi] = 1;
      exec = nullptr;
    }
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  cudaGetLastError();
}

static void sweep_free(Sweep* sw) {
  if (sw->lk_exec) cudaGraphExecDestroy(sw->lk_exec);
  if (sw->d_levels) cudaFreeAsync(sw->d_levels, sw->stream);
  for (auto& g : sw->groups) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    for (auto& v : g.views) {
      if (v->d_part) cudaFreeAsync(v->d_part, sw->stream);
      if (v->d_self) cudaFreeAsync(v->d_self, sw->stream);
    }
    if (g.slab) cudaFreeAsync(g.slab, sw->stream);
    if (g.d_states) cudaFreeAsync(g.d_states, sw->stream);
    if (g.d_kops) cudaFreeAsync(g.d_kops, sw->stream);
    if (g.d_coefs) cudaFreeAsync(g.d_coefs, sw->stream);
    for (void* p : {(void*)g.d_diag, (void*)g.d_z, (void*)g.d_gcoef, (void*)g.d_epart, (void*)g.d_en})
      if (p) cudaFreeAsync(p, sw->stream);
  }
  if (sw->stream) {
    cudaStreamSynchronize(sw->stream);
    cudaStreamDestroy(sw->stream);
  }
  delete sw;
}

// Energies of every member: per group, the diagonal path (I/Z strings with at
// most diag_max_groups() distinct coefficients, 12 qubits and more) runs one
// k_diag_expect + k_diag_reduce over all members; other groups evaluate each
// Pauli term on each member. The diagonal path's device tables (z masks, group
// counts, coefficients) are kept between runs and rebuilt only when the term
// arrays differ from the previous run's, and all groups share one sync.
static int sweep_energies(Sweep* sw, const int32_t* term_offsets, const double* coefficients,
                          const char* pauli_strings, double* energies, int* launches, std::string* err) {
  const int count = sw->count;
  std::vector<int64_t> char_off(count + 1, 0);
  for (int i = 0; i < count; ++i) {
    const int n = sw->groups[sw->where[i].first].n;
    char_off[i + 1] = char_off[i] + (int64_t)(term_offsets[i + 1] - term_offsets[i]) * n;
  }
  const int64_t nterms = term_offsets[count];
  const bool same = sw->e_valid && sw->e_offsets.size() == (size_t)count + 1 &&
                    std::memcmp(sw->e_offsets.data(), term_offsets, sizeof(int32_t) * (count + 1)) == 0 &&
                    std::memcmp(sw->e_coefs.data(), coefficients, sizeof(double) * (size_t)nterms) == 0 &&
                    sw->e_strings.compare(0, std::string::npos, pauli_strings, (size_t)char_off[count]) == 0;
  const int G = diag_max_groups();
  if (!same) {
    sw->e_valid = false;
    for (auto& g : sw->groups) {
      for (void* p : {(void*)g.d_diag, (void*)g.d_z, (void*)g.d_gcoef, (void*)g.d_epart, (void*)g.d_en})
        if (p) cudaFreeAsync(p, sw->stream);
      g.d_diag = nullptr, g.d_z = nullptr, g.d_gcoef = nullptr, g.d_epart = nullptr, g.d_en = nullptr;
      const size_t S = g.members.size();
      // diagonal path: every member's terms are I/Z strings with at most G distinct coefficients
      bool diag = g.n >= 12;
      std::vector<unsigned char> dstate(diag_state_bytes() * S);
      std::vector<uint64_t> zs;
      std::vector<double> gcoef(S * G, 0.0);
      for (size_t m = 0; m < S && diag; ++m) {
        const int ci = g.members[m];
        std::vector<double> vals;
        std::vector<std::vector<uint64_t>> per(G);
        std::vector<int> nid(G, 0);
        for (int t = term_offsets[ci]; t < term_offsets[ci + 1] && diag; ++t) {
          const char* ps = pauli_strings + char_off[ci] + (int64_t)(t - term_offsets[ci]) * g.n;
          uint64_t z = 0;
          for (int q = 0; q < g.n; ++q) {
            if (ps[q] == 'Z') z |= 1ULL << (g.n - 1 - q);
            else if (ps[q] != 'I') diag = false;
          }
          int gi = -1;
          for (size_t k = 0; k < vals.size(); ++k)
            if (vals[k] == coefficients[t]) gi = (int)k;
          if (gi < 0) {
            if ((int)vals.size() == G) {
              diag = false;
              break;
            }
            gi = (int)vals.size();
            vals.push_back(coefficients[t]);
          }
          if (z) per[gi].push_back(z);
          else ++nid[gi];
        }
        if (!diag) break;
        int gcount[8] = {0};
        const uint64_t zoff = zs.size();
        for (int k = 0; k < (int)vals.size(); ++k) {
          gcount[k] = (int)per[k].size();
          if (gcount[k] > diag_max_terms_per_group()) diag = false;
          zs.insert(zs.end(), per[k].begin(), per[k].end());
          gcoef[m * G + k] = vals[k];
        }
        if (!diag) break;
        fill_diag_state(dstate.data() + diag_state_bytes() * m, zoff, (int)vals.size(), gcount, nid.data());
      }
      g.diag = diag;
      if (!diag) continue;
      const uint64_t chunks = 1ULL << (g.n - 12);
      std::vector<uint32_t> qm(zs.size());
      for (size_t q = 0; q < zs.size(); ++q) qm[q] = diag_qmask(zs[q]);
      cudaError_t e = cudaMallocAsync(&g.d_diag, dstate.size(), sw->stream);
      if (e == cudaSuccess)
        e = cudaMallocAsync((void**)&g.d_z, (sizeof(uint64_t) + sizeof(uint32_t)) * std::max<size_t>(zs.size(), 1),
                            sw->stream);
      if (e == cudaSuccess) e = cudaMallocAsync((void**)&g.d_gcoef, sizeof(double) * gcoef.size(), sw->stream);
      if (e == cudaSuccess) e = cudaMallocAsync((void**)&g.d_epart, sizeof(double) * G * chunks * S, sw->stream);
      if (e == cudaSuccess) e = cudaMallocAsync((void**)&g.d_en, sizeof(double) * S, sw->stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(g.d_diag, dstate.data(), dstate.size(), cudaMemcpyHostToDevice, sw->stream);
      if (e == cudaSuccess && !zs.empty())
        e = cudaMemcpyAsync(g.d_z, zs.data(), sizeof(uint64_t) * zs.size(), cudaMemcpyHostToDevice, sw->stream);
      if (e == cudaSuccess && !zs.empty())
        e = cudaMemcpyAsync(g.d_z + zs.size(), qm.data(), sizeof(uint32_t) * qm.size(), cudaMemcpyHostToDevice,
                            sw->stream);
      g.nz = zs.size();
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(g.d_gcoef, gcoef.data(), sizeof(double) * gcoef.size(), cudaMemcpyHostToDevice,
                            sw->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(sw->stream);  // host tables die at scope end
      if (e != cudaSuccess) return cuda_fail(err, e, "sweep energy tables");
    }
    sw->e_offsets.assign(term_offsets, term_offsets + count + 1);
    sw->e_coefs.assign(coefficients, coefficients + nterms);
    sw->e_strings.assign(pauli_strings, (size_t)char_off[count]);
    sw->e_valid = true;
  }
  std::vector<std::vector<double>> en(sw->groups.size());
  for (size_t gi = 0; gi < sw->groups.size(); ++gi) {
    SweepGroup& g = sw->groups[gi];
    if (!g.diag) continue;
    const size_t S = g.members.size();
    en[gi].resize(S);
    cudaError_t e = launch_diag_expect(g.d_states, sw->prec, g.n, g.d_diag, g.d_z,
                                       reinterpret_cast<const uint32_t*>(g.d_z + g.nz), (int)S, g.d_epart,
                                       g.d_gcoef, g.d_en, sw->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(en[gi].data(), g.d_en, sizeof(double) * S, cudaMemcpyDeviceToHost, sw->stream);
    if (e != cudaSuccess) return cuda_fail(err, e, "sweep energies");
    *launches += 2;
  }
  cudaError_t se = cudaStreamSynchronize(sw->stream);
  if (se != cudaSuccess) return cuda_fail(err, se, "sweep energies");
  for (size_t gi = 0; gi < sw->groups.size(); ++gi) {
    SweepGroup& g = sw->groups[gi];
    if (g.diag) {
      for (size_t m = 0; m < g.members.size(); ++m) energies[g.members[m]] = en[gi][m];
      continue;
    }
    for (size_t m = 0; m < g.members.size(); ++m) {
      const int ci = g.members[m];
      double energy = 0;
      for (int t = term_offsets[ci]; t < term_offsets[ci + 1]; ++t) {
        double v;
        const int rc = st_pauli(g.views[m].get(), pauli_strings + char_off[ci] + (int64_t)(t - term_offsets[ci]) * g.n,
                                &v, err);
        if (rc != QG_OK) return rc;
        const double term = coefficients[t] * v;
        energy = (t == term_offsets[ci]) ? term : energy + term;
        ++*launches;
      }
      energies[ci] = energy;
    }
  }
  return QG_OK;
}

}  // namespace qg

extern "C" {

int qg_sweep_create(void* ctx, const qg_circuit* circuits, int32_t count, int32_t precision, int32_t arithmetic,
                    void** sweep_out) {
  if (!ctx || !circuits || count < 1 || !sweep_out) return QG_ERR_INVALID_ARG;
  if (precision != QG_C128 && precision != QG_C64) return QG_ERR_INVALID_ARG;
  Ctx* c = (Ctx*)ctx;
  cudaSetDevice(c->device);
  auto* sw = new Sweep();
  sw->ctx = c;
  sw->prec = precision;
  sw->arith = arithmetic == QG_ARITH_DOUBLE_FLOAT ? QG_ARITH_DOUBLE_FLOAT : QG_ARITH_EXACT;
  sw->count = count;
  sw->where.resize(count);
  std::string err;
  if (cudaStreamCreateWithFlags(&sw->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete sw;
    return QG_ERR_DEVICE;
  }
  std::map<std::vector<int64_t>, int> by_sig;
  for (int i = 0; i < count; ++i) {
    Program prog;
    int rc = compile_program(&circuits[i], precision, QG_FUSE_TILED, c->cfg.fuse_k, sw->arith, &prog, &err, false);
    if (rc != QG_OK) {
      set_ctx_error(c, "circuit " + std::to_string(i) + ": " + err);
      sweep_free(sw);
      return rc;
    }
    std::vector<int64_t> sig = pass_signature(prog);
    auto it = by_sig.find(sig);
    int gi;
    if (it == by_sig.end()) {
      gi = (int)sw->groups.size();
      by_sig[sig] = gi;
      sw->groups.emplace_back();
      sw->groups.back().n = prog.n;
    } else {
      gi = it->second;
    }
    SweepGroup& g = sw->groups[gi];
    sw->where[i] = {gi, (int)g.members.size()};
    g.members.push_back(i);
    g.progs.push_back(std::move(prog));
  }
  const size_t rec = kop_record_bytes();
  for (auto& g : sw->groups) {
    const Program& p0 = g.progs[0];
    for (size_t s = 0; s < p0.steps.size(); ++s) {
      if (p0.steps[s].kind != Step::TILE_PASS) g.batched = false;
      else g.pass_steps.push_back((int)s);
    }
    if (!p0.dense.empty()) g.batched = false;
    const size_t S = g.members.size();
    const size_t per = amp_bytes(precision) << g.n;
    cudaError_t e = cudaMallocAsync(&g.slab, per * S, sw->stream);
    if (e != cudaSuccess) {
      set_ctx_error(c, "sweep states do not fit in HBM");
      sweep_free(sw);
      return QG_ERR_OOM;
    }
    sw->bytes += per * S;
    std::vector<void*> ptrs(S);
    for (size_t m = 0; m < S; ++m) {
      ptrs[m] = (unsigned char*)g.slab + per * m;
      g.views.push_back(std::make_unique<State>());
      int rc = view_init(g.views.back().get(), c, ptrs[m], g.n, precision, sw->stream, &err);
      if (rc != QG_OK) {
        set_ctx_error(c, err);
        sweep_free(sw);
        return rc;
      }
    }
    if (cudaMallocAsync((void**)&g.d_states, sizeof(void*) * S, sw->stream) != cudaSuccess ||
        cudaMemcpyAsync(g.d_states, ptrs.data(), sizeof(void*) * S, cudaMemcpyHostToDevice, sw->stream) !=
            cudaSuccess) {
      sweep_free(sw);
      return QG_ERR_DEVICE;
    }
    if (!g.batched) continue;
    int64_t off = 0;
    for (int ps : g.pass_steps) {
      const PassDesc& pd = p0.steps[ps].pass;
      g.pass_off.push_back(off);
      g.pass_nops.push_back((int)(pd.op_end - pd.op_begin));
      off += (int64_t)(pd.op_end - pd.op_begin) * (int64_t)S;
    }
    g.kops_host.assign(rec * (size_t)std::max<int64_t>(off, 1), 0);
    encode_group_kops(sw, g);
    if (cudaMallocAsync(&g.d_kops, g.kops_host.size(), sw->stream) != cudaSuccess ||
        cudaMemcpyAsync(g.d_kops, g.kops_host.data(), g.kops_host.size(), cudaMemcpyHostToDevice, sw->stream) !=
            cudaSuccess) {
      sweep_free(sw);
      return QG_ERR_DEVICE;
    }
    setup_group_pass_kernels(sw, g);
    cudaStreamSynchronize(sw->stream);
    g.launches = 1 + (int)g.pass_steps.size();
    // capture the group's passes once; runs replay the graph
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(sw->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      cudaError_t le = launch_group_passes(sw, g);
      cudaError_t ce = cudaStreamEndCapture(sw->stream, &graph);
      if (le == cudaSuccess && ce == cudaSuccess && graph) {
        if (cudaGraphInstantiate(&g.exec, graph, 0) != cudaSuccess) g.exec = nullptr;
      }
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      count_launch(-g.launches);  // captured launches do not run here; replays count them
    }
  }
  setup_level_kernels(sw);
  if (cudaStreamSynchronize(sw->stream) != cudaSuccess) {
    sweep_free(sw);
    return QG_ERR_DEVICE;
  }
  *sweep_out = sw;
  return QG_OK;
}

int qg_sweep_update(void* sweep, const qg_circuit* circuits, int32_t count) {
  if (!sweep || !circuits) return QG_ERR_INVALID_ARG;
  Sweep* sw = (Sweep*)sweep;
  if (count != sw->count) return QG_ERR_INVALID_ARG;
  cudaSetDevice(sw->ctx->device);
  std::string err;
  for (int i = 0; i < count; ++i) {
    Program prog;
    int rc = compile_program(&circuits[i], sw->prec, QG_FUSE_TILED, sw->ctx->cfg.fuse_k, sw->arith, &prog, &err,
                             false);
    if (rc != QG_OK) {
      set_ctx_error(sw->ctx, err);
      return rc;
    }
    SweepGroup& g = sw->groups[sw->where[i].first];
    Program& old = g.progs[sw->where[i].second];
    if (pass_signature(prog) != pass_signature(old) ||
        (g.pk && pass_structure_key(prog, true) != pass_structure_key(old, true))) {
      set_ctx_error(sw->ctx, "circuit " + std::to_string(i) + " changed its structure; create a new sweep");
      return QG_ERR_INVALID_ARG;
    }
    old = std::move(prog);
  }
  for (auto& g : sw->groups) {
    if (!g.batched) continue;
    encode_group_kops(sw, g);
    if (cudaMemcpyAsync(g.d_kops, g.kops_host.data(), g.kops_host.size(), cudaMemcpyHostToDevice, sw->stream) !=
        cudaSuccess)
      return QG_ERR_DEVICE;
    if (g.pk) {
      encode_group_coefs(sw, g);
      if (cudaMemcpyAsync(g.d_coefs, g.coefs_host.data(), sizeof(float) * g.coefs_host.size(),
                          cudaMemcpyHostToDevice, sw->stream) != cudaSuccess)
        return QG_ERR_DEVICE;
    }
  }
  return cudaStreamSynchronize(sw->stream) == cudaSuccess ? QG_OK : QG_ERR_DEVICE;
}

int qg_sweep_run(void* sweep, const int32_t* term_offsets, const double* coefficients, const char* pauli_strings,
                 double* energies, qg_sweep_stats* stats) {
  if (!sweep) return QG_ERR_INVALID_ARG;
  NvtxRange nvtx("qg sweep run");
  Sweep* sw = (Sweep*)sweep;
  cudaSetDevice(sw->ctx->device);
  std::string err;
  cudaEvent_t e0, e1, e2;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreate(&e2);
  cudaEventRecord(e0, sw->stream);
  int launches = 0, graphs = 0;
  int rc = QG_OK;
  if (sw->lk_exec) {
    cudaError_t e = cudaGraphLaunch(sw->lk_exec, sw->stream);
    if (e != cudaSuccess) rc = cuda_fail(&err, e, "sweep level kernels");
    launches += sw->lk_launches;
    graphs += 1;
    count_launch(sw->lk_launches);
  }
  for (size_t gi = 0; gi < sw->groups.size() && rc == QG_OK; ++gi) {
    SweepGroup& g = sw->groups[gi];
    if (!sw->in_level.empty() && sw->in_level[gi]) continue;
    if (g.batched) {
      cudaError_t e = g.exec ? cudaGraphLaunch(g.exec, sw->stream) : launch_group_passes(sw, g);
      if (e != cudaSuccess) {
        rc = cuda_fail(&err, e, "sweep passes");
        break;
      }
      launches += g.launches;
      graphs += g.exec ? 1 : 0;
      if (g.exec) count_launch(g.launches);
    } else {
      for (size_t m = 0; m < g.members.size() && rc == QG_OK; ++m) {
        State* v = g.views[m].get();
        cudaError_t e = launch_set_basis(v->d, v->prec, v->n, 0, sw->stream);
        if (e != cudaSuccess) rc = cuda_fail(&err, e, "zero-state");
        ExecStats st;
        if (rc == QG_OK) rc = exec_program(v, g.progs[m], 0, nullptr, &st, &err);
        launches += st.passes + 1;
      }
    }
  }
  cudaEventRecord(e1, sw->stream);
  // energies
  if (rc == QG_OK && term_offsets && energies) rc = sweep_energies(sw, term_offsets, coefficients, pauli_strings,
                                                                   energies, &launches, &err);
  cudaEventRecord(e2, sw->stream);
  cudaError_t se = cudaEventSynchronize(e2);
  if (se != cudaSuccess && rc == QG_OK) rc = cuda_fail(&err, se, "sweep");
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, e0, e1);
    cudaEventElapsedTime(&b, e1, e2);
    stats->device_ms = a;
    stats->expect_ms = b;
    stats->groups = (int32_t)sw->groups.size();
    stats->launches = launches;
    stats->graphs = graphs;
    int spec = 0;
    for (auto& g : sw->groups) spec += g.pk ? 1 : 0;
    stats->specialised = spec;
    stats->state_bytes = sw->bytes;
    uint64_t pb = 0;
    for (auto& g : sw->groups) {
      const uint64_t per = (uint64_t)amp_bytes(sw->prec) << g.n;
      uint64_t passes = 0;
      for (size_t m = 0; m < g.progs.size(); ++m)
        passes += g.batched ? g.pass_steps.size() : (uint64_t)g.progs[m].hbm_passes;
      pb += per * (2 * passes + g.progs.size());  // passes read and write; the zeroing writes
    }
    stats->pass_bytes = pb;
    stats->level_graph_ms = sw->level_ms;
    stats->size_graphs_ms = sw->group_ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  if (rc != QG_OK) set_ctx_error(sw->ctx, err);
  return rc;
}

int qg_sweep_state(void* sweep, int32_t c, double* host) {
  if (!sweep || !host) return QG_ERR_INVALID_ARG;
  Sweep* sw = (Sweep*)sweep;
  if (c < 0 || c >= sw->count) return QG_ERR_INVALID_ARG;
  cudaSetDevice(sw->ctx->device);
  std::string err;
  State* v = sw->groups[sw->where[c].first].views[sw->where[c].second].get();
  int rc = download_c128(v, host, &err);
  if (rc != QG_OK) set_ctx_error(sw->ctx, err);
  return rc;
}

int qg_sweep_destroy(void* sweep) {
  if (!sweep) return QG_ERR_INVALID_ARG;
  Sweep* sw = (Sweep*)sweep;
  cudaSetDevice(sw->ctx->device);
  sweep_free(sw);
  return QG_OK;
}

}  // extern "C"
