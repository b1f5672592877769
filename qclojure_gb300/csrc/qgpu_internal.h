// Internal types shared by the circuit compiler (compile.cpp), the kernels
// (kernels.cu) and the runtime (runtime.cpp) of libqgpu.so.
#pragma once

#include <atomic>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/qgpu.h"

#if !defined(__CUDACC_RTC__)
#include <nvtx3/nvToolsExt.h>
#endif

namespace qg {

// A named NVTX range for the lifetime of the object (host code): admission, compile,
// device launch and result extraction show up as ranges in a timeline profiler. The
// header-only NVTX library does nothing unless a tool is attached.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// ---------------------------------------------------------------------------
// Device operation ("gate op") in amplitude-index space. Bit b of the basis
// index is qubit (n-1-b). All controlled forms are already transposed the way
// the reference's apply-controlled-gate applies them.
// ---------------------------------------------------------------------------
enum OpKind : int32_t {
  OK_U2 = 0,        // 2x2 on bit t where (idx & cmask) == cmask; class in cls
  OK_PHASE = 1,     // amp *= ph where (idx & mask) == mask; class in cls
  OK_SWAP = 2,      // exchange bits t,t2 where (idx & cmask) == cmask; flags&1: iSWAP phase i
  OK_BLOCKADE = 3,  // amp *= ph where popcount(idx & mask) == 1
  OK_PARITY = 4,    // amp *= (parity(idx & mask) ? ph1 : ph0)
  OK_COLLAPSE = 5,  // amp = ((idx & mask) == val) ? amp * scale : 0
  OK_DENSE = 6,     // dense 2^dk x 2^dk block on bits dbits[0..dk) (dbits[0] = least significant)
  OK_LAYOUT = 7     // tiled executor only: registers hold the local bits dbits[0..3) from here on
};

// Matrix classes of OK_U2 (picked on the host from exact zero / unit entries).
enum U2Class : int32_t {
  U2_GENERAL = 0,   // y0 = m0 x0 + m1 x1, y1 = m2 x0 + m3 x1
  U2_REAL = 1,      // all four entries real
  U2_RXLIKE = 2,    // real diagonal, imaginary off-diagonal
  U2_DIAG = 3,      // off-diagonal exactly zero
  U2_ANTIDIAG = 4,  // diagonal exactly zero
  U2_X = 5,         // [[0,1],[1,0]] exactly: a pure swap
  U2_IMAG_ANTI = 6  // diagonal zero, off-diagonal = +-i exactly: swap with (re,im) rotation
};

// Phase classes of OK_PHASE.
enum PhaseClass : int32_t {
  PH_GENERAL = 0,   // multiply by (m[0], m[1])
  PH_NEG = 1,       // multiply by -1 (exact)
  PH_I = 2,         // multiply by +i (exact)
  PH_MINUS_I = 3    // multiply by -i (exact)
};

struct GOp {
  int32_t kind;
  int32_t cls;
  int32_t t, t2;
  int32_t flags;
  int32_t dk;
  uint64_t cmask;
  uint64_t mask;
  uint64_t val;
  double m[8];
  int32_t dbits[5];
  int32_t tag;      // 1 + ordinal of the QG_OP_KRAUS operation it came from, 0 otherwise
  int64_t doff;     // offset (in complex entries) of a dense block in the pass's matrix buffer
};

// ---------------------------------------------------------------------------
// Tile-local operation: a GOp rewritten for one pass of the tiled executor.
// l* fields are masks / bit positions in tile-local index space (0..k-1),
// g* fields are the parts of the masks on non-local bits, tested once per tile.
// ---------------------------------------------------------------------------
struct TOp {
  int32_t kind;
  int32_t cls;
  int32_t t, t2;     // local bit positions; for OK_U2 in the tiled executor t2 = register position
  int32_t flags;
  int32_t dk;
  uint32_t lcmask;   // local control mask
  uint32_t lmask;    // local part of mask
  uint32_t lval;     // local part of val
  uint32_t tag;      // GOp::tag
  uint64_t gcmask;   // non-local control bits (absolute)
  uint64_t gmask;    // non-local part of mask (absolute)
  uint64_t gval;     // non-local part of val (absolute)
  double m[8];
  int32_t dbits[5];  // local bit positions of a dense block; register bits of OK_LAYOUT;
                     // register positions (a < b) of OK_SWAP
  int32_t pad1;
  int64_t doff;
  float mf[16];      // m split into float pairs: hi in mf[0..8), lo in mf[8..16)
  // Tiled executor: the local mask of the op (controls of U2/SWAP, mask of the
  // diagonal kinds) split into its register positions (3-bit rmask/rval) and its
  // thread bits (tmask/tval), so each thread tests one word per op.
  uint32_t rmask, rval, tmask, tval;
  uint32_t lj[8];    // OK_LAYOUT: local offset of register slot j
};

constexpr int kMaxTileBits = 13;     // 2^13 amplitudes per tile at most
constexpr int kMaxLocal = kMaxTileBits;

// One HBM pass of the tiled executor.
struct PassDesc {
  int32_t k;                 // local bits per tile
  int32_t klow;              // bits 0..klow-1 are always local (contiguous runs)
  int32_t lbits[kMaxLocal];  // absolute bit position of local bit j (ascending)
  int32_t nruns;             // runs of non-local bits for the tile-index deposit
  int32_t run_src[kMaxLocal + 1];
  int32_t run_dst[kMaxLocal + 1];
  int32_t run_len[kMaxLocal + 1];
  int64_t op_begin, op_end;  // range in the TOp array
};

// A compiled step sequence.
struct Step {
  enum Kind { PLAIN_OP, TILE_PASS, MEASURE } kind;
  GOp op;                  // PLAIN_OP
  PassDesc pass;           // TILE_PASS
  std::vector<int> mqubits;// MEASURE (qubit indices, outcome bit i <-> mqubits[i])
};

struct Program {
  int n = 0;
  std::vector<Step> steps;
  std::vector<TOp> tops;             // all tile ops, referenced by PassDesc ranges
  std::vector<double> dense;         // dense block matrices (re, im interleaved)
  std::vector<float> dense_tc;       // tensor-core blocks: TF32 hi / lo operands (dense_tc_prepare)
  int hbm_passes = 0;
  int arith = QG_ARITH_EXACT;        // complex128 arithmetic of the tiled passes
  // shape of the specialised pass kernels (qg_tuning); 0: the precision's default
  int32_t rbits = 0, bufs = 0, ctas = 0;
};

// Compile a reference-level circuit into GOps (returns QG_OK or an error code;
// err receives a message in the reference's words).
int lower_circuit(const qg_circuit* c, std::vector<GOp>* gops, std::vector<std::vector<int>>* measures,
                  std::vector<int>* measure_at, std::string* err);
// Tolerance-held policies only: uncontrolled diagonal gates to half-state phases
// and Hadamards to sum / difference, their factors applied as one global op
// before each measurement and at the end; measure_at is rewritten.
constexpr int kFactorNone = 0, kFactorRotations = 1;
void factor_global_phases(std::vector<GOp>* gops, std::vector<int>* measure_at, int rotations);
// Schedule GOps into passes for the given fusion mode; reorder lets commuting ops
// overtake each other to fill passes (tolerance-held policies only).
// tile_bits: local qubits per tile (0: tile_bits_for(n, precision)).
int schedule(int n, int precision, int fusion, int fuse_k, const std::vector<GOp>& gops,
             const std::vector<std::vector<int>>& measures, const std::vector<int>& measure_at,
             Program* prog, std::string* err, bool reorder, int tile_bits = 0);

// ---------------------------------------------------------------------------
// Kernel launchers (kernels.cu). All return cudaError_t from the launch.
// ---------------------------------------------------------------------------
int tile_bits_for(int n, int precision);

cudaError_t launch_set_basis(void* s, int precision, int n, uint64_t idx, cudaStream_t st);
cudaError_t launch_plain_op(void* s, int precision, int n, const GOp& op, cudaStream_t st);
// One tiled pass over nstates states of n qubits sharing the pass structure pd.
// d_states: device array of amplitude pointers; d_kops: compact op records on the
// device (encode_kops) for state 0, indexed by pd's op range; state s uses the
// records ops_stride further on (0: all states share one list).
// io (double-float arithmetic only): bit 0 = the state arrives as float pairs
// (re.hi, re.lo, im.hi, im.lo) written by the previous pass, bit 1 = leave it as
// float pairs for the next pass; without the bit the state is IEEE doubles.
constexpr int kTileInPairs = 1, kTileOutPairs = 2;
cudaError_t launch_tile_pass(int precision, int arithmetic, int io, int n, const PassDesc& pd,
                             void* const* d_states, int nstates, const void* d_kops, int64_t ops_stride,
                             const double* d_dense, cudaStream_t st);
// io bits for step i of a program: consecutive double-float tiled passes hand the
// state over as float pairs; the first converts from doubles, the last back.
int tile_pass_io(const Program& prog, size_t step);
int max_ops_per_tile_pass();
// Small jobs (tiled programs of 5..kMaxSmallJobQubits qubits: one tile per state)
// run whole in one CTA each; one launch per qubit count (k_tile_jobs).
constexpr int kMaxSmallJobQubits = 12;
struct TileJobRec {
  void* state;          // device amplitudes (IEEE layout of the job's precision)
  int64_t op_begin;     // first op record of the job in the launch's record array
  int32_t npasses;      // passes of the job's program
  int32_t pass_begin;   // index of its first pass in the launch's op-count array
};
// Device-resident loop for small jobs (k_job_loop): the host publishes jobs of one qubit
// count into a ring of slots in mapped host memory and raises *tail; the loop's CTAs
// claim slots in order (*head, device memory), run each job whole (as k_tile_jobs does)
// and set the slot's done flag. A CTA that finds no work for idle_ns nanoseconds
// returns (the bounded wait); the host relaunches the loop when work arrives again.
struct JobLoopSlot {
  TileJobRec rec;        // state; op_begin and pass_begin index the two arrays below
  const void* kops;      // the job's op records (device)
  const int32_t* pass_nops;
  int32_t done;          // set to 1 by the device when the job's state is final
  int32_t pad;
};
constexpr int kJobLoopCtas = 8;
cudaError_t launch_job_loop(int precision, int arithmetic, int n, JobLoopSlot* d_slots, uint32_t cap,
                            const uint32_t* d_tail, uint32_t* d_head, uint32_t* d_served, uint64_t idle_ns,
                            cudaStream_t st);
cudaError_t launch_tile_jobs(int precision, int arithmetic, int n, const TileJobRec* d_jobs, int njobs,
                             const void* d_kops, const int32_t* d_pass_nops, cudaStream_t st);
size_t kop_record_bytes();
// Context services (runtime.cpp) for the noisy-trajectory runner (noisy.cpp).
int ctx_device_of(void* ctx);
int ctx_arithmetic_of(void* ctx);
void ctx_report_error(void* ctx, const std::string& msg);
int ctx_compile_tiled(void* ctx, const qg_circuit* c, int precision, Program* prog, std::string* err);
// Set the 2x2 matrix of a tiled op (and its float-pair split for the float policies).
void set_op_matrix(TOp* t, const double m[8]);
// ---------------------------------------------------------------------------
// Specialised pass kernels (pass_kernels.cpp): every tiled pass of a program
// (complex64, or complex128 double-float) compiled by NVRTC into its own
// straight-line kernel; cached per device by generated source.
// ---------------------------------------------------------------------------
constexpr int kSMCount = 152;
struct PassKernels {
  virtual ~PassKernels() = default;
};
// nullptr (with the reason in why) when the program has nothing to specialise,
// NVRTC is missing or a compile or load failed: the caller runs it interpreted.
// table = true: one kernel per pass for every program of the same structure (a
// sweep group); matrix entries come from per-state coefficient rows.
std::shared_ptr<const PassKernels> pass_kernels_for(const Program& prog, int prec, int device, std::string* why,
                                                    bool table = false);
// The program's kernels if an earlier call compiled them (no compile here).
std::shared_ptr<const PassKernels> pass_kernels_cached(const Program& prog, int prec, int device);
// Programs with equal keys share table-form kernels (coefficients left out).
std::string pass_structure_key(const Program& prog, bool table);
// Launch the table form over nstates states; d_coefs holds nstates rows of
// 16 * (ops of the pass) floats (pass_coefficients of each state's program).
cudaError_t launch_pass_kernel_batch(const PassKernels& pk, size_t step, int n, const PassDesc& pd,
                                     void* const* d_states, int nstates, const float* d_coefs, int prec,
                                     cudaStream_t st);
void pass_coefficients(const Program& prog, size_t step, int prec, float* out);
// Sweep level kernels (pass_kernels.cpp): level l runs pass pass_steps[g][l] of every
// group g that has one, in one launch over all those groups' (state, tile) items. The
// descriptor array of a level lists its groups in level_groups order; each group's
// items are [item0, item0 + items) with items = ntiles * nstates. Layout shared with
// the device (qgp::GroupLevel).
struct GroupLevelDesc {
  void* const* states;
  const float* coefs;
  int32_t ncoef, nstates;
  uint64_t ntiles, item0, items;
};
std::shared_ptr<const PassKernels> level_kernels_for(const std::vector<const Program*>& progs,
                                                     const std::vector<std::vector<int>>& pass_steps, int prec,
                                                     int device, std::string* why);
int level_count(const PassKernels& lk);
const std::vector<int>& level_groups(const PassKernels& lk, int level);
double level_kernels_compile_ms(const PassKernels& lk);
cudaError_t launch_level_kernel(const PassKernels& lk, int level, const GroupLevelDesc* d_desc, uint64_t total,
                                cudaStream_t st);
bool pass_kernel_ready(const PassKernels& pk, size_t step);
double pass_kernels_compile_ms(const PassKernels& pk);
cudaError_t launch_pass_kernel(const PassKernels& pk, size_t step, int n, const PassDesc& pd, void* state, int prec,
                               cudaStream_t st);
// NVRTC availability (nullptr when usable, else the reason).
const char* pass_kernels_unavailable();
// Generate and compile without loading (no device needed): 1 compiled, 0 nothing
// to specialise, -1 a compile error (in why).
int pass_kernels_build_only(const Program& prog, int prec, int* kernels, double* compile_ms, std::string* why,
                            bool table = false);
std::string pass_kernels_source(const Program& prog, int prec);
void pass_kernel_cache_stats(size_t* hits, size_t* misses);
// batched sweep kernels (sweep.cu)
int diag_max_groups();
size_t diag_state_bytes();
void fill_diag_state(void* out, uint64_t zoff, int ngroups, const int* gcount, const int* nid);
cudaError_t launch_batch_zero(void* slab, int precision, int n, int nstates, cudaStream_t st);
// every state of up to kMaxZeroGroups slabs to |0...0> in one launch
constexpr int kMaxZeroGroups = 16;
struct MultiZero {
  void* slab[kMaxZeroGroups];
  uint64_t per[kMaxZeroGroups];  // amplitudes per state
  int32_t nstates[kMaxZeroGroups];
  int32_t ngroups;
};
cudaError_t launch_multi_zero(const MultiZero& z, int precision, cudaStream_t st);
// Noisy trajectories: one CTA per state renormalises it in place and records its
// squared norm before renormalisation; one CTA per shot draws an outcome of state
// d_state_of[shot] (draw64(seed, traj0 + shot, stream)), shifted right by `shift`
// (states padded with idle low qubits).
cudaError_t launch_traj_normalise(int precision, void* const* d_states, int nstates, int n, double* d_norm2,
                                  cudaStream_t st);
cudaError_t launch_traj_sample(int precision, void* const* d_states, const int32_t* d_state_of, int nshots, int n,
                               int shift, uint64_t seed, uint64_t traj0, uint32_t stream, uint64_t* d_out,
                               cudaStream_t st);
int diag_max_terms_per_group();
uint32_t diag_qmask(uint64_t z);  // bit q: parity of q & bits 8..11 of z
cudaError_t launch_diag_expect(void* const* d_states, int precision, int n, const void* d_diag, const uint64_t* d_z,
                               const uint32_t* d_qm, int nstates, double* d_partial, const double* d_gcoef,
                               double* d_energies, cudaStream_t st);
void encode_kops(int precision, int arithmetic, const TOp* tops, int64_t count, void* out);
void count_launch(int k);
cudaError_t launch_c128_to_c64(const double* src, float* dst, uint64_t count, cudaStream_t st);
cudaError_t launch_c64_to_c128(const float* src, double* dst, uint64_t count, cudaStream_t st);

// Reductions (results written to device scratch, copied by the caller).
// partial sums per block are (sum, compensation) pairs of doubles.
struct ReduceScratch {
  double* d_part = nullptr;     // 2 * nblocks doubles
  int nblocks = 0;
};
cudaError_t launch_probabilities(const void* s, int precision, int n, double* d_p, cudaStream_t st);
cudaError_t launch_norm2(const void* s, int precision, int n, double* d_part, int nblocks, cudaStream_t st);
cudaError_t launch_pauli_expect(const void* s, int precision, int n, uint64_t xmask, uint64_t zmask, int ny,
                                double* d_part, int nblocks, cudaStream_t st);
cudaError_t launch_expect_1q(const void* s, int precision, int n, int bit, const double* o8, double* d_part,
                             int nblocks, cudaStream_t st);
cudaError_t launch_inner(const void* a, const void* b, int precision, int n, double* d_part, int nblocks,
                         cudaStream_t st);
// a: complex64 or complex128, b: complex128; partials 6 x nblocks double-doubles, maxima nblocks
cudaError_t launch_compare(const void* a, int precision, const void* b, int n, double* d_part, double* d_max,
                           int nblocks, cudaStream_t st);
// Marginal probabilities over measured bits: per outcome FP64 (sum, comp) and u64 quantised totals.
cudaError_t launch_marginal_host(const void* s, int precision, int n, const int* h_bits, const int* d_bits, int m,
                                 int nbx, double* d_pm, unsigned long long* d_qm, cudaStream_t st);
cudaError_t launch_gather(const void* s, int precision, const uint64_t* d_idx, int64_t count, double* d_out,
                          cudaStream_t st);
cudaError_t launch_density(const void* s, int precision, int n, double* d_rho, cudaStream_t st);

// Hierarchical shot sampler. Scratch sized by sampler_scratch_bytes(); its layout:
// chunks of min(2^n, 32) amplitudes, blocks of min(chunks, 256) chunks, then one u64
// sum per chunk, one u64 sum per block, the blocks' exclusive prefixes plus a total,
// and FP64 per-block sums plus two (compensated total), with 256 bytes of slack.
constexpr size_t sampler_scratch_bytes_at(int n) {
  const uint64_t N = 1ULL << n;
  const uint64_t ch = N < 32 ? N : 32;
  const uint64_t nch = N / ch;
  const uint64_t cpb = nch < 256 ? nch : 256;
  const uint64_t nb = nch / cpb;
  return sizeof(unsigned long long) * (nch + nb + (nb + 1)) + sizeof(double) * (nb + 2) + 256;
}
size_t sampler_scratch_bytes(int n, uint64_t shots);
cudaError_t launch_sample(const void* s, int precision, int n, uint64_t shots, uint64_t seed, void* d_scratch,
                          uint64_t* d_outcomes, double* d_total, cudaStream_t st);

// File-scope sampler scratch of qg_state_sample_noalloc (noalloc.cu): its device
// address for `device` (which must be current), resolved once per device, and its size.
constexpr int kNoAllocSampleMaxQubits = 24;
cudaError_t noalloc_sample_scratch(int device, void** ptr, size_t* bytes);

// Dense blocks on the tensor cores (dense_tc.cu, complex64). A block of dk <= 5 qubits
// of an n >= 12 qubit state qualifies; dense_tc_prepare widens it to ke = max(dk, 4)
// target bits (tbits_out, ascending), lays out its TF32 operands (w_out) and returns
// ke; launch_dense_tc applies it in one HBM pass and sets *d_err when a bounded wait
// inside the kernel gives up.
constexpr int kDenseTcFlag = 1;  // GOp::flags of an OK_DENSE op run by launch_dense_tc
bool dense_tc_eligible(int n, int dk);
extern std::atomic<int> g_dense_tc_stall;  // qg_diag_dense_tc_stall
int dense_tc_prepare(int n, int dk, const int* pos, const double* mat, std::vector<float>* w_out, int* tbits_out);
cudaError_t launch_dense_tc(void* state, int n, int ke, const int* tbits, const float* d_w, int* d_err,
                            cudaStream_t st);

int reduce_blocks_for(int n);
unsigned long long kernel_launch_count();

// Philox4x32-10 (Salmon et al., SC'11), shared by host and device code.
#if defined(__CUDACC__)
#define QG_HD __host__ __device__ __forceinline__
#else
#define QG_HD inline
#endif
QG_HD void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                         uint32_t out[4]) {
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}
// 64 uniform bits for (seed, index, stream): stream 0 = shots, 1 = mid-circuit measurements.
QG_HD uint64_t draw64(uint64_t seed, uint64_t index, uint32_t stream) {
  uint32_t o[4];
  philox4x32_10((uint32_t)index, (uint32_t)(index >> 32), stream, 0u, (uint32_t)seed, (uint32_t)(seed >> 32), o);
  return ((uint64_t)o[1] << 32) | o[0];
}

}  // namespace qg
