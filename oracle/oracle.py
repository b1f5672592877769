"""ctypes wrapper of the CPU oracle (oracle/qgo.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference arm of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))

from oracle.build import build_oracle  # noqa: E402
from qclojure_gb300 import _abi as A  # noqa: E402  (struct layouts only)
from qclojure_gb300.circuit import encode  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle()
        L = C.CDLL(str(path))
        DP = C.POINTER(C.c_double)
        L.or_run_circuit.argtypes = [DP, C.c_int, C.POINTER(A.QgOp), C.c_int, C.c_uint64]
        L.or_run_circuit.restype = C.c_int
        L.or_zero_state.argtypes = [DP, C.c_int]
        L.or_probabilities.argtypes = [DP, C.c_int, DP]
        L.or_sample.argtypes = [DP, C.c_int, C.c_uint64, C.c_uint64, C.POINTER(C.c_uint64)]
        L.or_sample.restype = C.c_int
        L.or_pauli_expectation.argtypes = [DP, C.c_int, C.c_char_p]
        L.or_pauli_expectation.restype = C.c_double
        L.or_expectation_1q.argtypes = [DP, C.c_int, DP, C.c_int]
        L.or_expectation_1q.restype = C.c_double
        L.or_inner.argtypes = [DP, DP, C.c_int, DP, DP]
        L.or_measure.argtypes = [DP, C.c_int, C.POINTER(C.c_int), C.c_int, C.c_uint64, C.c_uint64,
                                 C.POINTER(C.c_uint64), DP]
        L.or_measure.restype = C.c_int
        L.or_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.or_draw64.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32]
        L.or_draw64.restype = C.c_uint64
        L.or_refalgo_rows.argtypes = [DP, C.c_int, DP, C.c_int, C.c_uint64, C.c_uint64, DP]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def zero_state(n: int) -> np.ndarray:
    s = np.zeros(1 << n, np.complex128)
    s[0] = 1
    return s


def run(circuit: dict, initial: np.ndarray | None = None, seed: int = 0) -> np.ndarray:
    """Final state of a circuit (reference semantics, FP64 without FMA)."""
    n = circuit["num-qubits"]
    s = zero_state(n) if initial is None else np.ascontiguousarray(initial, np.complex128).copy()
    enc = encode(circuit)
    rc = lib().or_run_circuit(_dp(s), n, enc.array, enc.count, C.c_uint64(seed))
    if rc:
        raise ValueError(f"oracle rejected operation {rc - 1}")
    return s


def probabilities(s: np.ndarray) -> np.ndarray:
    n = int(np.log2(s.size))
    p = np.empty(s.size)
    lib().or_probabilities(_dp(np.ascontiguousarray(s)), n, _dp(p))
    return p


def sample(s: np.ndarray, shots: int, seed: int) -> np.ndarray:
    n = int(np.log2(s.size))
    out = np.empty(max(1, shots), np.uint64)
    rc = lib().or_sample(_dp(np.ascontiguousarray(s)), n, shots, C.c_uint64(seed),
                         out.ctypes.data_as(C.POINTER(C.c_uint64)))
    if rc:
        raise ValueError("State is not properly normalized")
    return out[:shots]


def pauli_expectation(s: np.ndarray, pauli: str) -> float:
    n = int(np.log2(s.size))
    return lib().or_pauli_expectation(_dp(np.ascontiguousarray(s)), n, pauli.encode())


def hamiltonian_expectation(s: np.ndarray, terms) -> float:
    total = None
    for t in terms:
        v = t["coefficient"] * pauli_expectation(s, t["pauli-string"])
        total = v if total is None else total + v
    return 0.0 if total is None else total


def expectation_1q(s: np.ndarray, obs, target: int) -> float:
    n = int(np.log2(s.size))
    flat = np.array([[complex(z).real, complex(z).imag] for row in obs for z in row]).ravel()
    return lib().or_expectation_1q(_dp(np.ascontiguousarray(s)), n, _dp(flat), target)


def inner(a: np.ndarray, b: np.ndarray) -> complex:
    n = int(np.log2(a.size))
    re, im = C.c_double(), C.c_double()
    lib().or_inner(_dp(np.ascontiguousarray(a)), _dp(np.ascontiguousarray(b)), n, C.byref(re), C.byref(im))
    return complex(re.value, im.value)


def measure(s: np.ndarray, qubits, seed: int, draw_index: int = 0):
    n = int(np.log2(s.size))
    s = np.ascontiguousarray(s, np.complex128).copy()
    arr = (C.c_int * len(qubits))(*qubits)
    o, p = C.c_uint64(), C.c_double()
    lib().or_measure(_dp(s), n, arr, len(qubits), C.c_uint64(seed), C.c_uint64(draw_index), C.byref(o), C.byref(p))
    return s, o.value, p.value


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().or_philox4x32_10(c, k, o)
    return list(o)


def refalgo_rows(x: np.ndarray, gate2x2, target: int, row0: int, nrows: int) -> np.ndarray:
    """Rows of the reference's dense Kronecker mat-vec (the algorithm, for timing)."""
    n = int(np.log2(x.size))
    g = np.array([[complex(z).real, complex(z).imag] for row in gate2x2 for z in row]).ravel()
    y = np.empty(nrows, np.complex128)
    lib().or_refalgo_rows(_dp(np.ascontiguousarray(x)), n, _dp(g), target, C.c_uint64(row0), C.c_uint64(nrows),
                          _dp(y))
    return y
