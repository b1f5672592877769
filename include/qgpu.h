/*
 * qgpu.h - C ABI of libqgpu.so, a GB300 (sm_103a) state-vector simulator backend.
 *
 * The library is a drop-in for QClojure's ideal simulator
 * (src/org/soulspace/qclojure/adapter/backend/ideal_simulator.clj). The
 * QuantumBackend protocol methods (src/org/soulspace/qclojure/application/backend.clj:72-115)
 * map onto the job functions below; a JVM shim calls them through the Foreign
 * Function & Memory API, a Python host calls them through ctypes. Every entry
 * point:
 *   - takes plain pointers and sizes (no C++ or torch types cross the boundary),
 *   - returns an int status (QG_OK = 0) and never throws, aborts or traps,
 *   - writes results into caller-owned host buffers; device memory stays owned
 *     by the library (the amplitude array lives in HBM from the first gate to
 *     result extraction),
 *   - is thread-safe on one context.
 *
 * Conventions shared with the reference:
 *   - qubit q of an n-qubit register is bit (n-1-q) of the basis index
 *     (big-endian, src/org/soulspace/qclojure/domain/state.clj:114-136);
 *   - SWAP and iSWAP operands are bit positions counted from the least
 *     significant bit (src/org/soulspace/qclojure/domain/gate.clj:768-778);
 *   - controlled single-qubit gates apply the transpose of their 2x2 matrix
 *     (src/org/soulspace/qclojure/domain/gate.clj:473-483);
 *   - amplitudes cross the boundary as interleaved complex128 (re, im) pairs.
 */
#ifndef QGPU_H
#define QGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QG_ABI_VERSION 1
#define QG_MAX_QUBITS 40
#define QG_MAX_OP_QUBITS 40

/* ---- status codes (returned by every entry point) ---------------------- */
enum {
  QG_OK = 0,
  QG_ERR_INVALID_ARG = 1,      /* null pointer, bad size, bad enum value          */
  QG_ERR_UNKNOWN_GATE = 2,     /* opcode the reference dispatch rejects           */
  QG_ERR_QUBIT_RANGE = 3,      /* operand >= num_qubits or repeated operand        */
  QG_ERR_OOM = 4,              /* state does not fit the HBM budget                */
  QG_ERR_DEVICE = 5,           /* CUDA error (message via qg_last_error)           */
  QG_ERR_TIMEOUT = 6,          /* qg_wait ran out of time                          */
  QG_ERR_CANCELLED = 7,        /* job was cancelled                                */
  QG_ERR_NOT_FOUND = 8,        /* unknown job / batch id                           */
  QG_ERR_NOT_COMPLETED = 9,    /* result requested before completion               */
  QG_ERR_NOT_NORMALIZED = 10,  /* |sum p - 1| > 1e-8 before sampling (state.clj:901) */
  QG_ERR_BUFFER_TOO_SMALL = 11,/* caller buffer shorter than the result            */
  QG_ERR_UNSUPPORTED = 12,     /* request the reference also refuses               */
  QG_ERR_NO_RESULT = 13,       /* result type was not requested in the spec         */
  QG_ERR_NO_DEVICE = 14        /* no CUDA device visible                           */
};

/* ---- job status (ideal_simulator.clj:138-141 keywords) ------------------ */
enum {
  QG_JOB_QUEUED = 0,
  QG_JOB_RUNNING = 1,
  QG_JOB_COMPLETED = 2,
  QG_JOB_FAILED = 3,
  QG_JOB_CANCELLED = 4,
  QG_JOB_NOT_FOUND = 5
};

/* ---- qg_cancel outcomes (ideal_simulator.clj:154-163) ------------------- */
enum { QG_CANCEL_CANCELLED = 0, QG_CANCEL_CANNOT = 1, QG_CANCEL_NOT_FOUND = 2 };

/* ---- precision --------------------------------------------------------- */
enum { QG_C128 = 0, QG_C64 = 1 };

/* ---- complex128 arithmetic in tiled passes ---------------------------- */
enum {
  QG_ARITH_EXACT = 0,        /* FP64, same rounded products and sums as the reference (bit-identical) */
  QG_ARITH_DOUBLE_FLOAT = 1  /* float pairs on the FP32 pipes (about 48 bits), doubles in HBM          */
};

/* ---- specialised pass kernels ------------------------------------------ */
/* A tiled pass of a complex64 or double-float complex128 program can run as its own
   kernel, generated from the pass's gates and compiled at run time (NVRTC, cached per
   device by generated source), instead of the interpreting tiled kernel. AUTO uses
   them for states of 29 qubits and more; without NVRTC every pass runs interpreted. */
enum {
  QG_PASS_KERNELS_AUTO = 0,
  QG_PASS_KERNELS_OFF = 1,
  QG_PASS_KERNELS_ALWAYS = 2
};

/* ---- fusion modes ------------------------------------------------------ */
enum {
  QG_FUSE_PLAIN = 0,   /* one HBM pass per gate (the plain method)                    */
  QG_FUSE_TILED = 1,   /* gate runs applied in shared-memory tiles, one pass per run  */
  QG_FUSE_DENSE = 2    /* gate runs merged into dense 2^k x 2^k blocks (k = fuse_k)   */
};

/* ---- opcodes: the gate set of circuit.clj:933-1072 ---------------------- */
enum {
  QG_OP_X = 1, QG_OP_Y = 2, QG_OP_Z = 3, QG_OP_H = 4,
  QG_OP_S = 5, QG_OP_SDAG = 6, QG_OP_T = 7, QG_OP_TDAG = 8,
  QG_OP_RX = 9, QG_OP_RY = 10, QG_OP_RZ = 11, QG_OP_PHASE = 12,
  QG_OP_CNOT = 20, QG_OP_CZ = 21, QG_OP_CRX = 22, QG_OP_CRY = 23, QG_OP_CRZ = 24,
  QG_OP_CY = 25,              /* reached through :controlled with :target-gate :y   */
  QG_OP_SWAP = 26, QG_OP_ISWAP = 27, QG_OP_TOFFOLI = 28, QG_OP_FREDKIN = 29,
  QG_OP_RYDBERG_CZ = 40, QG_OP_RYDBERG_CPHASE = 41, QG_OP_RYDBERG_BLOCKADE = 42,
  QG_OP_GLOBAL_RX = 50, QG_OP_GLOBAL_RY = 51, QG_OP_GLOBAL_RZ = 52, QG_OP_GLOBAL_H = 53,
  QG_OP_GLOBAL_X = 54, QG_OP_GLOBAL_Y = 55, QG_OP_GLOBAL_Z = 56,
  QG_OP_MEASURE = 60,         /* mid-circuit measurement with collapse (circuit.clj:1074) */
  QG_OP_U = 70,               /* explicit 2x2 matrix m on q[0], applied like a 1-qubit gate */
  QG_OP_CU = 71,              /* explicit 2x2 matrix m on q[1], control q[0] (transposed, as the reference) */
  QG_OP_RZZ = 72,             /* exp(-i angle/2 Z(q0) Z(q1)); a diagonal extension for QAOA cost layers */
  QG_OP_KRAUS = 73,           /* explicit 2x2 operator m on q[0], applied as a general matrix whatever its
                                 entries and without renormalisation (noisy trajectories renormalise once,
                                 after the last operation) */
  QG_OP_I = 80                /* identity: the reference dispatch has no case for it and fails */
};

/* One operation. Operand meaning per opcode, in the reference's parameter order:
 *   1-qubit gates:   q[0] = :target
 *   CNOT/CZ/CRx/CY:  q[0] = :control, q[1] = :target
 *   SWAP/iSWAP:      q[0] = :qubit1,  q[1] = :qubit2  (LSB bit positions)
 *   TOFFOLI:         q[0] = :control1, q[1] = :control2, q[2] = :target
 *   FREDKIN:         q[0] = :control, q[1] = :target1, q[2] = :target2
 *   RYDBERG_CZ/CPHASE: q[0] = :control, q[1] = :target
 *   RYDBERG_BLOCKADE:  q[0..nq) = :qubit-indices
 *   MEASURE:           q[0..nq) = :measurement-qubits (outcome bit i <-> q[i])
 *   GLOBAL_*:          no operands
 *   RZZ:               q[0], q[1]
 * angle is :angle (radians); m holds a row-major 2x2 complex matrix (re, im) for U/CU. */
typedef struct qg_op {
  int32_t opcode;
  int32_t nq;
  uint8_t q[QG_MAX_OP_QUBITS];
  double angle;
  double m[8];
} qg_op;

typedef struct qg_circuit {
  int32_t num_qubits;
  int32_t num_ops;
  const qg_op* ops;
} qg_circuit;

/* Result specification: the keys of result.clj:535-639. A zero flag omits the result. */
enum {
  QG_RES_MEASUREMENTS = 1 << 0,   /* :measurements  {:shots}                       */
  QG_RES_EXPECTATION = 1 << 1,    /* :expectation   {:observables :targets}        */
  QG_RES_VARIANCE = 1 << 2,       /* :variance      {:observables :targets}        */
  QG_RES_HAMILTONIAN = 1 << 3,    /* :hamiltonian   [pauli terms]                  */
  QG_RES_PROBABILITIES = 1 << 4,  /* :probabilities {:targets}                      */
  QG_RES_AMPLITUDES = 1 << 5,     /* :amplitudes    {:basis-states}                 */
  QG_RES_STATE_VECTOR = 1 << 6,   /* :state-vector  true                            */
  QG_RES_DENSITY_MATRIX = 1 << 7, /* :density-matrix true (n <= 14)                 */
  QG_RES_FIDELITY = 1 << 8,       /* :fidelity      {:references}                   */
  QG_RES_ACCURACY = 1 << 9        /* no reference counterpart: distance of the result from
                                     the exact FP64 run of the same circuit             */
};

typedef struct qg_result_spec {
  uint32_t flags;
  int32_t reserved;
  uint64_t shots;                 /* :measurements :shots (default 1)                   */
  /* :hamiltonian: n_terms coefficients and n_terms strings of num_qubits chars over IXYZ,
     concatenated; char i of a string acts on qubit i (observables.clj:216-232). */
  int32_t n_terms;
  int32_t n_observables;
  const double* coefficients;
  const char* pauli_strings;
  /* :expectation / :variance: n_observables 2x2 Hermitian matrices (8 doubles each,
     row-major re/im) and one target qubit per observable. */
  const double* observables;
  const int32_t* observable_targets;
  /* :amplitudes :basis-states and :probabilities :targets (basis indices). */
  int32_t n_basis_states;
  int32_t n_probability_targets;
  const uint64_t* basis_states;
  const uint64_t* probability_targets;
  /* :fidelity :references: n_references host states of 2^num_qubits complex128 each. */
  int32_t n_references;
  int32_t reserved2;
  const double* references;
} qg_result_spec;

typedef struct qg_options {
  const qg_result_spec* spec;     /* may be NULL: no results beyond the final state      */
  const double* initial_state;    /* host complex128, 2^n amplitudes, or NULL for |0..0> */
  uint64_t seed;                  /* drives shot sampling and mid-circuit collapse       */
  int32_t precision;              /* QG_C128 / QG_C64, -1 = context default              */
  int32_t fusion;                 /* QG_FUSE_*, -1 = context default                     */
  int32_t arithmetic;             /* QG_ARITH_*, -1 = context default                    */
  int32_t reserved;
} qg_options;

typedef struct qg_config {
  int32_t device;                 /* CUDA ordinal                                        */
  int32_t precision;              /* default precision                                   */
  int32_t fusion;                 /* default fusion mode                                 */
  int32_t fuse_k;                 /* dense block width for QG_FUSE_DENSE (1..5)          */
  int32_t max_qubits;             /* admission limit (0 = derived from HBM)              */
  int32_t workers;                /* device streams serving jobs concurrently (>=1)      */
  uint64_t hbm_budget_bytes;      /* 0 = free HBM minus a reserve                        */
  uint64_t seed;                  /* default seed                                        */
  int32_t arithmetic;             /* QG_ARITH_* for complex128 tiled passes              */
  int32_t pass_kernels;           /* QG_PASS_KERNELS_*                                   */
  int32_t small_job_loop;         /* QG_JOB_LOOP_*: how jobs of 5..12 qubits run         */
  int32_t reserved0;
} qg_config;

/* Jobs of 5..12 qubits (the whole state is one tile) run one CTA per job. AUTO / ON:
   a device-resident loop per qubit count claims them as they are published (no launch
   per job or batch); OFF: a host batcher groups ready jobs into one launch. */
enum { QG_JOB_LOOP_AUTO = 0, QG_JOB_LOOP_ON = 1, QG_JOB_LOOP_OFF = 2 };

typedef struct qg_queue_info {    /* queue-status (ideal_simulator.clj:165-176) + device fields */
  int64_t total_jobs, queued, running, completed, failed, cancelled;
  uint64_t hbm_free_bytes, hbm_budget_bytes, hbm_in_use_bytes;
  int32_t workers;
  int32_t precompiled_jobs;       /* queued large jobs whose pass kernels a background
                                     compile prepared before they ran (no counterpart)  */
} qg_queue_info;

typedef struct qg_job_info {
  int32_t status;
  int32_t num_qubits;
  int32_t precision;
  int32_t num_passes;             /* HBM passes the compiled circuit took                */
  double execution_time_ms;       /* wall time submit-to-completion on the worker         */
  double device_time_ms;          /* CUDA-event time of the gate passes                   */
  double queue_time_ms;
  uint64_t shots;
  int64_t num_distinct_outcomes;
  int32_t has_results;            /* QG_RES_* flags that are available                    */
  int32_t error_code;
  int32_t batched_with;           /* jobs that shared its small-job launch (0: ran alone) */
  int32_t specialised_passes;     /* tiled passes that ran as specialised kernels         */
} qg_job_info;

/* ---- context ------------------------------------------------------------ */
int qg_abi_version(void);
int qg_device_count(int32_t* count);
int qg_ctx_create(const qg_config* cfg, void** ctx_out);
int qg_ctx_destroy(void* ctx);
/* backend-info / device: capability numbers for the device map (ideal_simulator.clj:34-51). */
int qg_ctx_capabilities(void* ctx, int32_t* max_qubits_c128, int32_t* max_qubits_c64,
                        uint64_t* hbm_total_bytes, int32_t* sm_count);

/* ---- jobs: QuantumBackend (backend.clj:72-115) -------------------------- */
/* submit-circuit (ideal_simulator.clj:120-136): validates, copies the circuit and
   returns at once; a device worker runs the job. */
int qg_submit(void* ctx, const qg_circuit* circuit, const qg_options* options, uint64_t* job_out);
/* job-status (ideal_simulator.clj:138-141). */
int qg_job_status(void* ctx, uint64_t job, int32_t* status_out);
/* Blocking wait; replaces the 100 ms poll loop of backend.clj:239-256. */
int qg_wait(void* ctx, uint64_t job, int64_t timeout_ms, int32_t* status_out);
/* cancel-job (ideal_simulator.clj:154-163): QG_CANCEL_* in *outcome. */
int qg_cancel(void* ctx, uint64_t job, int32_t* outcome);
/* queue-status (ideal_simulator.clj:165-176). */
int qg_queue_status(void* ctx, qg_queue_info* out);
/* qg_job_loop_info has no counterpart in the reference: the device-resident small-job
   loops of the context. loops: qubit counts that have one; running: loop kernels still
   resident; launches: loop kernels started (a loop leaves after a few milliseconds
   without work and starts again when a job arrives); jobs: jobs served by the loops. */
typedef struct qg_loop_info {
  int32_t loops, running;
  uint64_t launches, jobs;
} qg_loop_info;
int qg_job_loop_info(void* ctx, qg_loop_info* out);
int qg_job_details(void* ctx, uint64_t job, qg_job_info* out);
/* job-result pieces (result.clj:179-497). Buffers are caller-owned. */
int qg_result_counts(void* ctx, uint64_t job, uint64_t* outcomes, uint64_t* counts, int64_t cap, int64_t* n_out);
int qg_result_shots(void* ctx, uint64_t job, uint64_t* outcomes, int64_t cap);
int qg_result_probabilities(void* ctx, uint64_t job, double* out, int64_t cap);
int qg_result_target_probabilities(void* ctx, uint64_t job, double* out, int64_t cap);
int qg_result_state(void* ctx, uint64_t job, double* out_c128, int64_t cap_amplitudes);
int qg_result_amplitudes(void* ctx, uint64_t job, double* out_c128, int64_t cap_amplitudes);
int qg_result_expectations(void* ctx, uint64_t job, double* expectation, double* variance, int64_t cap);
int qg_result_hamiltonian(void* ctx, uint64_t job, double* energy, double* term_values, int64_t cap);
int qg_result_fidelities(void* ctx, uint64_t job, double* out, int64_t cap);
int qg_result_density_matrix(void* ctx, uint64_t job, double* out_c128, int64_t cap_entries);
/* QG_RES_ACCURACY (no counterpart in the reference): the job's final state against the
   same circuit run again in complex128 with exact FP64 arithmetic in the reference's gate
   order (the path that equals the reference's simulator bit for bit): out3 = largest
   amplitude difference, 1 - fidelity, total variation distance of the outcome
   probabilities. Costs one more run and a complex128 state of the job's size. */
int qg_result_accuracy(void* ctx, uint64_t job, double* out3);
int qg_last_error(void* ctx, uint64_t job, char* buf, int64_t len);
/* Releases a job and its device state (cleanup-completed-jobs!, ideal_simulator.clj:243-264). */
int qg_job_free(void* ctx, uint64_t job);
int qg_cleanup_completed(void* ctx, int64_t max_age_ms, int64_t* removed);

/* ---- batches: BatchJobBackend (backend.clj:136-168) --------------------- */
/* batch-submit: all circuits share the options; jobs_out receives one job id per circuit.
   Queued jobs of equal qubit count are run together by the batched pass kernel. */
int qg_batch_submit(void* ctx, const qg_circuit* circuits, int32_t count, const qg_options* options,
                    uint64_t* batch_out, uint64_t* jobs_out);
/* batch-status: one QG_JOB_* per job, in submission order. */
int qg_batch_status(void* ctx, uint64_t batch, int32_t* statuses, int32_t cap, int32_t* n_out);
int qg_batch_jobs(void* ctx, uint64_t batch, uint64_t* jobs, int32_t cap, int32_t* n_out);

/* ---- device-resident state (state.clj, gate.clj, result.clj on one state) ----
   These bypass the job queue: the state stays in HBM between calls, which is
   how the QAOA/VQE loop and the benchmarks drive the kernels. */
int qg_state_create(void* ctx, int32_t num_qubits, int32_t precision, void** state_out);
int qg_state_destroy(void* state);
int qg_state_num_qubits(void* state, int32_t* n, int32_t* precision);
/* zero-state (state.clj:251-284) or basis state |index>. */
int qg_state_set_basis(void* state, uint64_t index);
int qg_state_upload(void* state, const double* host_c128);
int qg_state_download(void* state, double* host_c128);
/* Apply a circuit in place with the given fusion mode; mid-circuit measurements draw
   from seed. passes_out (may be NULL) receives the number of HBM passes. */
int qg_state_apply(void* state, const qg_circuit* circuit, int32_t fusion, uint64_t seed, int32_t* passes_out);
/* No counterpart in the reference: compile (and cache) the specialised pass kernels
   that qg_state_apply would use for this circuit on this state, without running it,
   so a later apply starts at once. specialised_out receives how many passes have a
   kernel (0 when the context's pass-kernel setting or the circuit uses none). */
int qg_state_prepare(void* state, const qg_circuit* circuit, int32_t fusion, double* compile_ms_out,
                     int32_t* specialised_out);
/* probabilities (state.clj:658-682) into a host buffer of 2^n doubles. */
int qg_state_probabilities(void* state, double* host_out);
/* Shot sampling (state.clj:869-913 rule: first outcome whose cumulative probability
   reaches the uniform draw) with Philox uniforms from seed; outcomes in shot order. */
int qg_state_sample(void* state, uint64_t shots, uint64_t seed, uint64_t* host_outcomes);
/* qg_state_sample_noalloc has no counterpart in the reference. It draws the same
   outcomes as qg_state_sample (same seed, same shots) but allocates no device memory:
   for callers that cannot allocate while sampling, such as a host runtime that has
   handed every free byte of HBM to its own pool, or a loop that must not take the
   allocator's locks and possible synchronisation on each call. Its scratch is one fixed
   array per device inside this library (about 4.3 MB), which limits the state to
   24 qubits; larger states return QG_ERR_INVALID_ARG. device_outcomes is caller-owned
   device memory of the state's device holding at least `shots` values; the call
   returns after the outcomes are written (it synchronises the state's stream).
   The first call on a device looks up the array's device address once (with that
   device current); make that first call before any stream capture begins. After a
   device reset (cudaDeviceReset, or another library destroying the primary context)
   the next call sees a new context and looks the address up again. Calls that
   overlap on one device (from several host threads) share the array and race:
   serialise them. */
int qg_state_sample_noalloc(void* state, uint64_t shots, uint64_t seed, uint64_t* device_outcomes);
/* <psi|P|psi> for a Pauli string of num_qubits chars (hamiltonian.clj:82-94). */
int qg_state_pauli_expectation(void* state, const char* pauli, double* out);
/* sum_j c_j <P_j> (hamiltonian.clj:96-114), strings concatenated. */
int qg_state_hamiltonian(void* state, int32_t n_terms, const double* coeffs, const char* paulis, double* out);
/* <psi|O_t|psi> for a 2x2 observable on one target qubit (result.clj:254-288). */
int qg_state_expectation_1q(void* state, const double* obs8, int32_t target, double* out);
/* Sum of |a|^2 and <a|b> (complex_linear_algebra.clj:318,435), FP64 compensated. */
int qg_state_norm2(void* state, double* out);
int qg_state_inner(void* a, void* b, double* re, double* im);
/* Accuracy of a state against a complex128 state of the same size (for instance an exact
 * FP64 run of the same circuit); no reference counterpart. out3[0] = max_i |a_i - r_i|,
 * out3[1] = 1 - |<r|a>|^2 / (<a|a><r|r>), out3[2] = 1/2 sum_i | |a_i|^2 - |r_i|^2 |
 * (total variation distance of the outcome distributions). */
int qg_state_compare(void* state, void* reference, double* out3);
/* Partial measurement with collapse (state.clj:915-1014); outcome bit i <-> qubits[i]. */
int qg_state_measure(void* state, const int32_t* qubits, int32_t count, uint64_t seed,
                     uint64_t* outcome_out, double* probability_out);
/* Device pointer of the amplitude array (interleaved re/im, fp64 for c128, fp32 for c64)
   and its CUDA stream, for callers that hand the state to other CUDA code. */
int qg_state_device_ptr(void* state, void** dptr, void** stream);
int qg_state_synchronize(void* state);

/* ---- parameter sweeps: many circuits of one structure, replayed -------------
   The variational loop of the reference (application/algorithm/variational_algorithm.clj:310-363,
   qaoa.clj:1087-1115) executes the same circuit structure with new angles, one
   execute-circuit per parameter vector. A sweep holds one device state per circuit;
   circuits of equal qubit count and equal pass structure run together, one kernel
   launch per HBM pass over all of their states, captured once into a CUDA graph and
   replayed. Every run starts from |0...0>. */
typedef struct qg_sweep_stats {
  double device_ms;       /* CUDA-event time of the gate passes (graph replays)   */
  double expect_ms;       /* CUDA-event time of the energy kernels                */
  int32_t groups;         /* batches of equal structure                           */
  int32_t launches;       /* kernel launches per run (inside the graphs)          */
  int32_t graphs;         /* groups replayed from a CUDA graph                    */
  int32_t specialised;    /* groups whose passes run as specialised kernels       */
  uint64_t state_bytes;   /* HBM held by the sweep's states                       */
  uint64_t pass_bytes;    /* algorithmic HBM bytes of one run's gate passes: one read
                             and one write of every amplitude per pass, plus the write
                             that zeroes each state                                  */
  double level_graph_ms;  /* measured when the sweep was created: all sizes through
                             one launch per pass level (0: not built)                */
  double size_graphs_ms;  /* the same passes as one graph per size; the sweep runs
                             the faster of the two                                   */
} qg_sweep_stats;

/* Compile circuits (no mid-circuit measurement), allocate their states, capture graphs. */
int qg_sweep_create(void* ctx, const qg_circuit* circuits, int32_t count, int32_t precision, int32_t arithmetic,
                    void** sweep_out);
/* New parameters for the same circuits: op records are rewritten in place; a circuit
   whose pass structure changed makes this return QG_ERR_INVALID_ARG. */
int qg_sweep_update(void* sweep, const qg_circuit* circuits, int32_t count);
/* Run every circuit and evaluate one Hamiltonian per circuit: circuit c owns terms
   [term_offsets[c], term_offsets[c+1]) of coefficients / pauli_strings (strings of
   that circuit's num_qubits chars, concatenated in term order). energies[c] =
   sum_j c_j <P_j> (hamiltonian.clj:96-114). term_offsets may be NULL (no energies). */
int qg_sweep_run(void* sweep, const int32_t* term_offsets, const double* coefficients, const char* pauli_strings,
                 double* energies, qg_sweep_stats* stats);
/* Copy circuit c's final state (complex128) to the host. */
int qg_sweep_state(void* sweep, int32_t c, double* host_c128);
int qg_sweep_destroy(void* sweep);

/* ---- noisy trajectories ----------------------------------------------------------
   The hardware simulator's shot loop (adapter/backend/hardware_simulator.clj:84-193):
   every shot runs the circuit from |0...0>, applying after each operation that has a
   gate-noise entry one Kraus operator of that entry's channel on the operation's
   :target (noise.clj:53-102); the operator is drawn with the probabilities
   max_ij |K_ij|^2 of the channel's operators (channel.clj:194-232) and the state is
   renormalised (channel.clj:127-171). The shot then samples one outcome from its final
   state and applies readout noise with correlations (noise.clj:107-202). Shots run as
   batched trajectories: the noise draws depend only on (seed, shot, site), so every
   trajectory shares one compiled program and differs only in its Kraus matrices. */
enum {
  QG_NOISE_NONE = 0,               /* noise type the reference ignores (noise.clj:101)    */
  QG_NOISE_DEPOLARIZING = 1,       /* {sqrt(1-p) I, sqrt(p/3) X, Y, Z}, channel.clj:40-63 */
  QG_NOISE_AMPLITUDE_DAMPING = 2,  /* {[[1,0],[0,sqrt(1-g)]], [[0,sqrt g],[0,0]]}, :65-84 */
  QG_NOISE_PHASE_DAMPING = 3,      /* {[[1,0],[0,sqrt(1-g)]], [[0,0],[0,sqrt g]]}, :86-104 */
  QG_NOISE_COHERENT = 4            /* one rotation operator, channel.clj:106-125           */
};
enum { QG_NOISE_HAS_T1 = 1, QG_NOISE_HAS_T2 = 2, QG_NOISE_HAS_GATE_TIME = 4 };
typedef struct qg_gate_noise {
  int32_t noise_type;      /* QG_NOISE_*                                                  */
  int32_t present;         /* QG_NOISE_HAS_* bits for t1_us, t2_us, gate_time_ns          */
  double strength;         /* :noise-strength (the reference's default is 0.01)           */
  double t1_us, t2_us;     /* :t1-time, :t2-time (microseconds)                           */
  double gate_time_ns;     /* :gate-time (nanoseconds)                                    */
  double coherent_angle;   /* :coherent-error :rotation-angle                             */
  int32_t coherent_axis;   /* :rotation-axis 0 = :x, 1 = :y, 2 = :z                       */
  int32_t pad;
} qg_gate_noise;
typedef struct qg_noise_model {
  int32_t num_entries;            /* gate-noise entries                                    */
  int32_t has_readout;            /* :readout-error present                                */
  const qg_gate_noise* entries;
  const int32_t* op_entry;        /* per circuit operation: its entry (looked up by the
                                     operation's :operation-type), or -1 for none          */
  const int32_t* op_target;       /* per circuit operation: (get-in op [:operation-params
                                     :target] 0), the qubit the noise acts on              */
  double prob_0_to_1, prob_1_to_0;
  int32_t num_correlations;       /* :correlated-errors {source {target factor}} as triples */
  int32_t pad;
  const int32_t* corr_source;
  const int32_t* corr_target;
  const double* corr_factor;
} qg_noise_model;
typedef struct qg_noisy_stats {
  double device_ms;        /* device time: state set-up, passes, renormalisation, sampling */
  double total_ms;         /* wall time of the call                                       */
  int32_t batches;         /* device batches of trajectories                              */
  int32_t batch_size;      /* trajectories per batch                                      */
  int64_t noise_sites;     /* Kraus operators per trajectory                              */
  int64_t passes;          /* tiled HBM passes per batch                                  */
  int64_t distinct_states; /* states simulated: shots with equal Kraus choices share one  */
} qg_noisy_stats;
/* Run `shots` trajectories of `circuit` (no mid-circuit measurements) in `precision`
   (complex128 with the context's arithmetic, or complex64). outcomes[s] is the basis
   index read in shot s after readout noise (qubit q <-> bit n-1-q). trajectories, if not
   NULL, receives the first min(shots, max_trajectories) final states, renormalised, as
   complex128 (2 * 2^n doubles each); final_state, if not NULL, the last shot's. */
int qg_noisy_run(void* ctx, const qg_circuit* circuit, const qg_noise_model* noise, uint64_t shots, uint64_t seed,
                 int32_t precision, int32_t max_trajectories, uint64_t* outcomes, double* trajectories,
                 double* final_state, qg_noisy_stats* stats);

/* ---- measurement (no counterpart in the reference) ----------------------------
   qg_state_profile applies a circuit like qg_state_apply and records a CUDA event
   pair around every HBM pass on the state's stream: pass_ms[i] is the duration of
   pass i and pass_kind[i] its kind (0 plain gate, 1 tiled pass, 2 measurement,
   3 tiled pass run by its specialised kernel, 4 dense block on the tensor cores).
   qg_kernel_launches reports how many kernels this library has launched in the
   process so far. */
int qg_state_profile(void* state, const qg_circuit* circuit, int32_t fusion, uint64_t seed, float* pass_ms,
                     int32_t* pass_kind, int32_t cap, int32_t* n_passes);
int qg_kernel_launches(uint64_t* count);
/* Specialised pass kernels (no counterpart in the reference). qg_pass_kernels_build
   generates and compiles the kernels of a circuit's tiled passes for sm_103a without
   loading them (no device needed): QG_OK with the kernel count and compile time,
   QG_ERR_DEVICE with the compiler's message in err_buf when a compile fails,
   QG_ERR_UNSUPPORTED when NVRTC is not available. With QG_PASS_BUILD_TABLE OR'ed into
   `arithmetic` it builds the table-form kernels a parameter sweep compiles for the
   circuit's structure instead (gates in circuit order, matrix entries and parity masks
   read from a per-state table). qg_pass_kernels_info reports whether NVRTC is available
   and the compiled-program cache's hits and misses. */
#define QG_PASS_BUILD_TABLE 0x100
int qg_pass_kernels_build(const qg_circuit* circuit, int32_t precision, int32_t arithmetic, int32_t* kernels_out,
                          double* compile_ms_out, char* err_buf, int64_t err_len);
int qg_pass_kernels_info(int32_t* available, uint64_t* cache_hits, uint64_t* cache_misses);
/* Failure-path diagnostic (no counterpart in the reference): while on != 0, the
   tensor-core dense-block kernel's MMA thread issues nothing, so the kernel's bounded
   waits (about a second) run out, it frees its tensor memory and returns, and the run
   fails with QG_ERR_DEVICE ("a bounded wait gave up"); the context stays usable.
   Process-wide; for tests of the failure path only. */
int qg_diag_dense_tc_stall(int32_t on);
/* Sampler diagnostic (no counterpart in the reference): the quantised probability sums
   measure-state's draws use (state.clj:869-913 with floor(p 2^62) integer prefix sums),
   one per chunk of min(2^n, 32) amplitudes in chunk_sums[0 .. count) (count must be
   2^n / min(2^n, 32)), and their total in *total. Runs the sampler's first two kernels
   only; for parity tests of the quantisation. */
int qg_diag_sample_sums(void* state, uint64_t* chunk_sums, uint64_t count, uint64_t* total);

/* ---- autotuner (no counterpart in the reference; the reference's hook for gate
   optimisation is gate_optimization.clj:776-860, which this tiled executor replaces) --
   The specialised pass kernels apply a pass's gates to tiles of 2^tile_bits amplitudes,
   each thread holding 2^reg_bits of them, with `buffers` tile buffers in shared memory
   and the kernels built for ctas_per_sm CTAs per SM. qg_autotune times candidate shapes
   on a calibration circuit (the caller's workload, or when null six layers of the
   layered recipe and four QFT columns) on a state of num_qubits qubits, keeps the fastest (the default unless another is faster
   by more than 1 %), records it in the context for programs of that size and precision
   that run specialised, and reports every candidate with its median device time (ms).
   It allocates one state of that size while it runs. qg_tuning_set records a shape
   directly (tile_bits 0: back to the default); qg_tuning_get reports the shape in use.
   qg_tuning_pick is the choice rule on its own: the index of the fastest valid entry,
   or default_index when that one is within tie_frac of it (-1: none valid). */
typedef struct qg_tuning {
  int32_t tile_bits;    /* local qubits per tile: 10 to 13 */
  int32_t reg_bits;     /* amplitudes per thread = 2^reg_bits (3 or 4) */
  int32_t buffers;      /* tile buffers in shared memory (1 to 3: tiles in flight + 1) */
  int32_t ctas_per_sm;  /* CTAs per SM the kernels are built for */
  double ms;            /* measured device time of the calibration circuit (qg_autotune) */
} qg_tuning;
int qg_autotune(void* ctx, int32_t num_qubits, int32_t precision, const qg_circuit* calibration, qg_tuning* chosen,
                qg_tuning* tried, int32_t cap, int32_t* count_out);
int qg_tuning_set(void* ctx, int32_t num_qubits, int32_t precision, const qg_tuning* tuning);
int qg_tuning_get(void* ctx, int32_t num_qubits, int32_t precision, qg_tuning* out);
int32_t qg_tuning_pick(const double* ms, const int32_t* valid, int32_t count, int32_t default_index, double tie_frac);
/* qg_autotune_crossover (no counterpart in the reference) measures from which state size
   a circuit that runs once gains from its specialised kernels: for 20, 22, ..., 30 qubits
   it runs a calibration circuit of `layers` layers interpreted, compiles its kernels cold
   and runs it specialised. The crossover is the smallest size from which compile wall
   time plus the specialised run beats the interpreted run at every larger size; the
   context then specialises states of at least that many qubits under
   QG_PASS_KERNELS_AUTO (29 until measured). table receives up to cap rows of
   (qubits, interpreted ms, compile ms, specialised ms). Call it before submitting work:
   it allocates one state of each size in turn. */
int qg_autotune_crossover(void* ctx, int32_t precision, int32_t layers, int32_t* min_qubits_out, double* table,
                          int32_t cap, int32_t* count_out);

#ifdef __cplusplus
}
#endif
#endif /* QGPU_H */
