"""ctypes view of include/qgpu.h and the loader of libqgpu.so.

The structures mirror the C header field for field. load_library() fails
loudly when the shared library is missing or lacks a declared symbol: there is
no CPU fallback anywhere in the package.
"""
from __future__ import annotations

import ctypes as C
import re
import threading
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_lib" / "libqgpu.so"
HEADER = PKG.parent / "include" / "qgpu.h"

QG_MAX_QUBITS = 40
QG_MAX_OP_QUBITS = 40

# status codes
QG_OK = 0
QG_ERR_INVALID_ARG = 1
QG_ERR_UNKNOWN_GATE = 2
QG_ERR_QUBIT_RANGE = 3
QG_ERR_OOM = 4
QG_ERR_DEVICE = 5
QG_ERR_TIMEOUT = 6
QG_ERR_CANCELLED = 7
QG_ERR_NOT_FOUND = 8
QG_ERR_NOT_COMPLETED = 9
QG_ERR_NOT_NORMALIZED = 10
QG_ERR_BUFFER_TOO_SMALL = 11
QG_ERR_UNSUPPORTED = 12
QG_ERR_NO_RESULT = 13
QG_ERR_NO_DEVICE = 14

ERROR_NAMES = {
    0: "ok", 1: "invalid-argument", 2: "unknown-gate", 3: "qubit-range", 4: "out-of-memory",
    5: "device-error", 6: "timeout", 7: "cancelled", 8: "not-found", 9: "not-completed",
    10: "not-normalized", 11: "buffer-too-small", 12: "unsupported", 13: "no-result", 14: "no-device",
}

# job status
QG_JOB_QUEUED, QG_JOB_RUNNING, QG_JOB_COMPLETED, QG_JOB_FAILED, QG_JOB_CANCELLED, QG_JOB_NOT_FOUND = range(6)
JOB_STATUS = {0: "queued", 1: "running", 2: "completed", 3: "failed", 4: "cancelled", 5: "not-found"}
QG_CANCEL_CANCELLED, QG_CANCEL_CANNOT, QG_CANCEL_NOT_FOUND = range(3)
CANCEL_OUTCOME = {0: "cancelled", 1: "cannot-cancel", 2: "not-found"}

QG_C128, QG_C64 = 0, 1
QG_FUSE_PLAIN, QG_FUSE_TILED, QG_FUSE_DENSE = 0, 1, 2
QG_ARITH_EXACT, QG_ARITH_DOUBLE_FLOAT = 0, 1
QG_PASS_BUILD_TABLE = 0x100
QG_PASS_KERNELS_AUTO, QG_PASS_KERNELS_OFF, QG_PASS_KERNELS_ALWAYS = 0, 1, 2
PASS_KERNELS = {"auto": 0, "off": 1, "always": 2}

# opcodes
OP = dict(
    x=1, y=2, z=3, h=4, s=5, s_dag=6, t=7, t_dag=8, rx=9, ry=10, rz=11, phase=12,
    cnot=20, cz=21, crx=22, cry=23, crz=24, cy=25, swap=26, iswap=27, toffoli=28, fredkin=29,
    rydberg_cz=40, rydberg_cphase=41, rydberg_blockade=42,
    global_rx=50, global_ry=51, global_rz=52, global_h=53, global_x=54, global_y=55, global_z=56,
    measure=60, u=70, cu=71, rzz=72, kraus=73, i=80,
)

# noise channels of qg_noisy_run
QG_NOISE_NONE, QG_NOISE_DEPOLARIZING, QG_NOISE_AMPLITUDE_DAMPING, QG_NOISE_PHASE_DAMPING, QG_NOISE_COHERENT = range(5)
NOISE_TYPES = {"depolarizing": 1, "amplitude-damping": 2, "phase-damping": 3, "coherent": 4}
QG_NOISE_HAS_T1, QG_NOISE_HAS_T2, QG_NOISE_HAS_GATE_TIME = 1, 2, 4

# result flags
QG_RES_MEASUREMENTS = 1 << 0
QG_RES_EXPECTATION = 1 << 1
QG_RES_VARIANCE = 1 << 2
QG_RES_HAMILTONIAN = 1 << 3
QG_RES_PROBABILITIES = 1 << 4
QG_RES_AMPLITUDES = 1 << 5
QG_RES_STATE_VECTOR = 1 << 6
QG_RES_DENSITY_MATRIX = 1 << 7
QG_RES_FIDELITY = 1 << 8
QG_RES_ACCURACY = 1 << 9


class QgOp(C.Structure):
    _fields_ = [("opcode", C.c_int32), ("nq", C.c_int32), ("q", C.c_uint8 * QG_MAX_OP_QUBITS),
                ("angle", C.c_double), ("m", C.c_double * 8)]


class QgCircuit(C.Structure):
    _fields_ = [("num_qubits", C.c_int32), ("num_ops", C.c_int32), ("ops", C.POINTER(QgOp))]


class QgResultSpec(C.Structure):
    _fields_ = [
        ("flags", C.c_uint32), ("reserved", C.c_int32), ("shots", C.c_uint64),
        ("n_terms", C.c_int32), ("n_observables", C.c_int32),
        ("coefficients", C.POINTER(C.c_double)), ("pauli_strings", C.c_char_p),
        ("observables", C.POINTER(C.c_double)), ("observable_targets", C.POINTER(C.c_int32)),
        ("n_basis_states", C.c_int32), ("n_probability_targets", C.c_int32),
        ("basis_states", C.POINTER(C.c_uint64)), ("probability_targets", C.POINTER(C.c_uint64)),
        ("n_references", C.c_int32), ("reserved2", C.c_int32), ("references", C.POINTER(C.c_double)),
    ]


class QgOptions(C.Structure):
    _fields_ = [("spec", C.POINTER(QgResultSpec)), ("initial_state", C.POINTER(C.c_double)),
                ("seed", C.c_uint64), ("precision", C.c_int32), ("fusion", C.c_int32),
                ("arithmetic", C.c_int32), ("reserved", C.c_int32)]


class QgConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("precision", C.c_int32), ("fusion", C.c_int32), ("fuse_k", C.c_int32),
                ("max_qubits", C.c_int32), ("workers", C.c_int32), ("hbm_budget_bytes", C.c_uint64),
                ("seed", C.c_uint64), ("arithmetic", C.c_int32), ("pass_kernels", C.c_int32),
                ("small_job_loop", C.c_int32), ("reserved0", C.c_int32)]


JOB_LOOP = {"auto": 0, "on": 1, "off": 2}


class QgLoopInfo(C.Structure):
    _fields_ = [("loops", C.c_int32), ("running", C.c_int32), ("launches", C.c_uint64), ("jobs", C.c_uint64)]


class QgQueueInfo(C.Structure):
    _fields_ = [("total_jobs", C.c_int64), ("queued", C.c_int64), ("running", C.c_int64),
                ("completed", C.c_int64), ("failed", C.c_int64), ("cancelled", C.c_int64),
                ("hbm_free_bytes", C.c_uint64), ("hbm_budget_bytes", C.c_uint64), ("hbm_in_use_bytes", C.c_uint64),
                ("workers", C.c_int32), ("precompiled_jobs", C.c_int32)]


class QgJobInfo(C.Structure):
    _fields_ = [("status", C.c_int32), ("num_qubits", C.c_int32), ("precision", C.c_int32),
                ("num_passes", C.c_int32), ("execution_time_ms", C.c_double), ("device_time_ms", C.c_double),
                ("queue_time_ms", C.c_double), ("shots", C.c_uint64), ("num_distinct_outcomes", C.c_int64),
                ("has_results", C.c_int32), ("error_code", C.c_int32), ("batched_with", C.c_int32),
                ("specialised_passes", C.c_int32)]


class QgSweepStats(C.Structure):
    _fields_ = [("device_ms", C.c_double), ("expect_ms", C.c_double), ("groups", C.c_int32),
                ("launches", C.c_int32), ("graphs", C.c_int32), ("specialised", C.c_int32),
                ("state_bytes", C.c_uint64), ("pass_bytes", C.c_uint64), ("level_graph_ms", C.c_double),
                ("size_graphs_ms", C.c_double)]


class QgTuning(C.Structure):
    _fields_ = [("tile_bits", C.c_int32), ("reg_bits", C.c_int32), ("buffers", C.c_int32),
                ("ctas_per_sm", C.c_int32), ("ms", C.c_double)]

    def as_dict(self) -> dict:
        return {"tile_bits": self.tile_bits, "reg_bits": self.reg_bits, "buffers": self.buffers,
                "ctas_per_sm": self.ctas_per_sm, "ms": self.ms}


class QgGateNoise(C.Structure):
    _fields_ = [("noise_type", C.c_int32), ("present", C.c_int32), ("strength", C.c_double),
                ("t1_us", C.c_double), ("t2_us", C.c_double), ("gate_time_ns", C.c_double),
                ("coherent_angle", C.c_double), ("coherent_axis", C.c_int32), ("pad", C.c_int32)]


class QgNoiseModel(C.Structure):
    _fields_ = [("num_entries", C.c_int32), ("has_readout", C.c_int32), ("entries", C.POINTER(QgGateNoise)),
                ("op_entry", C.POINTER(C.c_int32)), ("op_target", C.POINTER(C.c_int32)),
                ("prob_0_to_1", C.c_double), ("prob_1_to_0", C.c_double),
                ("num_correlations", C.c_int32), ("pad", C.c_int32),
                ("corr_source", C.POINTER(C.c_int32)), ("corr_target", C.POINTER(C.c_int32)),
                ("corr_factor", C.POINTER(C.c_double))]


class QgNoisyStats(C.Structure):
    _fields_ = [("device_ms", C.c_double), ("total_ms", C.c_double), ("batches", C.c_int32),
                ("batch_size", C.c_int32), ("noise_sites", C.c_int64), ("passes", C.c_int64),
                ("distinct_states", C.c_int64)]


P = C.c_void_p
U64 = C.c_uint64
I32 = C.c_int32
I64 = C.c_int64
DP = C.POINTER(C.c_double)
U64P = C.POINTER(C.c_uint64)
I32P = C.POINTER(C.c_int32)

SIGNATURES = {
    "qg_abi_version": ([], C.c_int),
    "qg_device_count": ([I32P], C.c_int),
    "qg_ctx_create": ([C.POINTER(QgConfig), C.POINTER(P)], C.c_int),
    "qg_ctx_destroy": ([P], C.c_int),
    "qg_ctx_capabilities": ([P, I32P, I32P, U64P, I32P], C.c_int),
    "qg_submit": ([P, C.POINTER(QgCircuit), C.POINTER(QgOptions), U64P], C.c_int),
    "qg_job_status": ([P, U64, I32P], C.c_int),
    "qg_wait": ([P, U64, I64, I32P], C.c_int),
    "qg_cancel": ([P, U64, I32P], C.c_int),
    "qg_queue_status": ([P, C.POINTER(QgQueueInfo)], C.c_int),
    "qg_job_details": ([P, U64, C.POINTER(QgJobInfo)], C.c_int),
    "qg_result_counts": ([P, U64, U64P, U64P, I64, C.POINTER(I64)], C.c_int),
    "qg_result_shots": ([P, U64, U64P, I64], C.c_int),
    "qg_result_probabilities": ([P, U64, DP, I64], C.c_int),
    "qg_result_target_probabilities": ([P, U64, DP, I64], C.c_int),
    "qg_result_state": ([P, U64, DP, I64], C.c_int),
    "qg_result_amplitudes": ([P, U64, DP, I64], C.c_int),
    "qg_result_expectations": ([P, U64, DP, DP, I64], C.c_int),
    "qg_result_hamiltonian": ([P, U64, DP, DP, I64], C.c_int),
    "qg_result_fidelities": ([P, U64, DP, I64], C.c_int),
    "qg_result_density_matrix": ([P, U64, DP, I64], C.c_int),
    "qg_result_accuracy": ([P, C.c_uint64, DP], C.c_int),
    "qg_last_error": ([P, U64, C.c_char_p, I64], C.c_int),
    "qg_job_free": ([P, U64], C.c_int),
    "qg_cleanup_completed": ([P, I64, C.POINTER(I64)], C.c_int),
    "qg_batch_submit": ([P, C.POINTER(QgCircuit), I32, C.POINTER(QgOptions), U64P, U64P], C.c_int),
    "qg_batch_status": ([P, U64, I32P, I32, I32P], C.c_int),
    "qg_batch_jobs": ([P, U64, U64P, I32, I32P], C.c_int),
    "qg_state_create": ([P, I32, I32, C.POINTER(P)], C.c_int),
    "qg_state_destroy": ([P], C.c_int),
    "qg_state_num_qubits": ([P, I32P, I32P], C.c_int),
    "qg_state_set_basis": ([P, U64], C.c_int),
    "qg_state_upload": ([P, DP], C.c_int),
    "qg_state_download": ([P, DP], C.c_int),
    "qg_state_apply": ([P, C.POINTER(QgCircuit), I32, U64, I32P], C.c_int),
    "qg_state_prepare": ([P, C.POINTER(QgCircuit), I32, DP, I32P], C.c_int),
    "qg_state_probabilities": ([P, DP], C.c_int),
    "qg_state_sample": ([P, U64, U64, U64P], C.c_int),
    "qg_state_sample_noalloc": ([P, U64, U64, P], C.c_int),
    "qg_state_pauli_expectation": ([P, C.c_char_p, DP], C.c_int),
    "qg_state_hamiltonian": ([P, I32, DP, C.c_char_p, DP], C.c_int),
    "qg_state_expectation_1q": ([P, DP, I32, DP], C.c_int),
    "qg_state_norm2": ([P, DP], C.c_int),
    "qg_state_inner": ([P, P, DP, DP], C.c_int),
    "qg_state_compare": ([P, P, DP], C.c_int),
    "qg_noisy_run": ([P, C.POINTER(QgCircuit), C.POINTER(QgNoiseModel), U64, U64, I32, I32, U64P, DP, DP,
                      C.POINTER(QgNoisyStats)], C.c_int),
    "qg_state_measure": ([P, I32P, I32, U64, U64P, DP], C.c_int),
    "qg_state_device_ptr": ([P, C.POINTER(P), C.POINTER(P)], C.c_int),
    "qg_state_synchronize": ([P], C.c_int),
    "qg_state_profile": ([P, C.POINTER(QgCircuit), I32, U64, C.POINTER(C.c_float), I32P, I32, I32P], C.c_int),
    "qg_kernel_launches": ([U64P], C.c_int),
    "qg_pass_kernels_build": ([C.POINTER(QgCircuit), I32, I32, I32P, DP, C.c_char_p, I64], C.c_int),
    "qg_pass_kernels_info": ([I32P, U64P, U64P], C.c_int),
    "qg_diag_dense_tc_stall": ([I32], C.c_int),
    "qg_diag_sample_sums": ([P, U64P, U64, U64P], C.c_int),
    "qg_job_loop_info": ([P, C.POINTER(QgLoopInfo)], C.c_int),
    "qg_autotune": ([P, I32, I32, C.POINTER(QgCircuit), C.POINTER(QgTuning), C.POINTER(QgTuning), I32, I32P],
                    C.c_int),
    "qg_tuning_set": ([P, I32, I32, C.POINTER(QgTuning)], C.c_int),
    "qg_tuning_get": ([P, I32, I32, C.POINTER(QgTuning)], C.c_int),
    "qg_tuning_pick": ([DP, I32P, I32, I32, C.c_double], I32),
    "qg_autotune_crossover": ([P, I32, I32, I32P, DP, I32, I32P], C.c_int),
    "qg_sweep_create": ([P, C.POINTER(QgCircuit), I32, I32, I32, C.POINTER(P)], C.c_int),
    "qg_sweep_update": ([P, C.POINTER(QgCircuit), I32], C.c_int),
    "qg_sweep_run": ([P, I32P, DP, C.c_char_p, DP, C.POINTER(QgSweepStats)], C.c_int),
    "qg_sweep_state": ([P, I32, DP], C.c_int),
    "qg_sweep_destroy": ([P], C.c_int),
}


def declared_symbols() -> list[str]:
    """Every function the header declares (used by the export test)."""
    text = HEADER.read_text()
    return re.findall(r"^(?:int|int32_t)\s+(qg_\w+)\s*\(", text, flags=re.M)


class QgError(RuntimeError):
    def __init__(self, code: int, message: str = ""):
        self.code = code
        name = ERROR_NAMES.get(code, str(code))
        super().__init__(f"{name}: {message}" if message else name)


_lib = None
_lock = threading.Lock()


def load_library(path: Path | None = None):
    """Load libqgpu.so (built by qclojure_gb300.build) and bind every signature."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise RuntimeError(
                f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "(the GPU backend has no CPU fallback)")
        lib = C.CDLL(str(p))
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(lib, name)  # AttributeError here means the library lacks a declared entry point
            fn.argtypes = args
            fn.restype = res
        if lib.qg_abi_version() != 1:
            raise RuntimeError("libqgpu.so ABI version mismatch")
        if path is None:
            _lib = lib
        return lib
