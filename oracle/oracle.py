"""ctypes wrapper of the CPU oracle (oracle/qgo.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference arm of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import math
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
        L.or_sample_one.argtypes = [DP, C.c_int, C.c_uint64, C.c_uint64, C.c_uint32]
        L.or_refalgo_circuit.argtypes = [DP, C.c_int, C.POINTER(A.QgOp), C.c_int, C.c_uint64, C.c_uint64,
                                         C.POINTER(C.c_uint64)]
        L.or_refalgo_circuit.restype = C.c_int
        L.or_sample_one.restype = C.c_uint64
        L.or_chunk_sums.argtypes = [DP, C.c_int, C.POINTER(C.c_uint64)]
        L.or_chunk_sums.restype = C.c_uint64
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


def chunk_sums(s: np.ndarray) -> tuple[np.ndarray, int]:
    """The sampler's quantised sums per chunk of min(2^n, 32) amplitudes, and their total."""
    n = int(np.log2(s.size))
    out = np.empty(max(1, s.size // 32), np.uint64)
    T = lib().or_chunk_sums(_dp(np.ascontiguousarray(s, dtype=np.complex128)), n,
                            out.ctypes.data_as(C.POINTER(C.c_uint64)))
    return out, int(T)


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


def refalgo_circuit(circuit: dict, shots: int, seed: int) -> tuple[np.ndarray, np.ndarray]:
    """A whole circuit and its shots run by the reference's algorithm (dense Kronecker
    mat-vec per single-qubit gate, a full probability scan per shot), single-threaded;
    for timing the reference at the sizes it reaches. Returns (final state, outcomes)."""
    n = circuit["num-qubits"]
    s = zero_state(n)
    enc = encode(circuit)
    out = np.zeros(max(1, shots), np.uint64)
    rc = lib().or_refalgo_circuit(_dp(s), n, enc.array, enc.count, C.c_uint64(shots), C.c_uint64(seed),
                                  out.ctypes.data_as(C.POINTER(C.c_uint64)))
    if rc:
        raise ValueError(f"reference algorithm failed ({rc})")
    return s, out[:shots]


# ---------------------------------------------------------------------------
# Noisy trajectories (adapter/backend/hardware_simulator.clj:84-193). Each shot
# restated as the reference runs it: the operation, then, if its :operation-type has
# a gate-noise entry, one Kraus operator of that channel on its :target chosen by the
# draw (seed, shot, 0x40000000 + site), applied and renormalised (QG_OP_KRAUS of
# qgo.c); one outcome drawn with (seed, shot, 2); readout noise with one draw per
# qubit (seed, shot, 0x20000000 + qubit).
# ---------------------------------------------------------------------------
_KRAUS_STREAM, _READOUT_STREAM, _MEASURE_STREAM = 0x40000000, 0x20000000, 2


def _key(k) -> str:
    s = str(k)
    return s[1:] if s.startswith(":") else s


def _uniform(seed: int, index: int, stream: int) -> float:
    return (lib().or_draw64(C.c_uint64(seed), C.c_uint64(index), C.c_uint32(stream)) >> 11) * 2.0 ** -53


def kraus_channel(cfg: dict) -> list[np.ndarray] | None:
    """The Kraus operators apply-gate-noise builds (noise.clj:73-99, channel.clj:40-125,
    :234-250); None for a noise type it ignores. Raises ValueError where the reference's
    preconditions fail."""
    t = _key(cfg.get("noise-type"))
    strength = cfg.get("noise-strength", 0.01)
    t1, t2, gt = cfg.get("t1-time"), cfg.get("t2-time"), cfg.get("gate-time")

    def deco(a, b, g):
        if not (a > 0 and b > 0 and g > 0):
            raise ValueError("decoherence parameters must be positive")
        us = g / 1000.0
        return 1.0 - math.exp(-(us / a)), 1.0 - math.exp(-(us / b))

    if t == "depolarizing":
        p = strength
        if not (0 <= p <= 1) or p > 0.75:
            raise ValueError("depolarizing probability out of range")
        a, b = math.sqrt(1.0 - p), math.sqrt(p / 3.0)
        return [np.array([[a, 0], [0, a]], complex), np.array([[0, b], [b, 0]], complex),
                np.array([[0, -1j * b], [1j * b, 0]], complex), np.array([[b, 0], [0, -b]], complex)]
    if t in ("amplitude-damping", "phase-damping"):
        g = strength
        if t == "amplitude-damping" and t1 is not None and gt is not None:
            g = deco(t1, t2 if t2 is not None else t1, gt)[0]
        if t == "phase-damping" and t2 is not None and gt is not None:
            g = deco(t1 if t1 is not None else t2, t2, gt)[1]
        if not (0 <= g <= 1):
            raise ValueError("damping parameter out of range")
        k0 = np.array([[1, 0], [0, math.sqrt(1.0 - g)]], complex)
        k1 = (np.array([[0, math.sqrt(g)], [0, 0]], complex) if t == "amplitude-damping"
              else np.array([[0, 0], [0, math.sqrt(g)]], complex))
        return [k0, k1]
    if t == "coherent":
        ce = cfg.get("coherent-error") or {"rotation-angle": 0.01, "rotation-axis": "z"}
        th, ax = ce["rotation-angle"], _key(ce["rotation-axis"])
        c, s_ = math.cos(th / 2.0), math.sin(th / 2.0)
        if ax == "x":
            return [np.array([[c, -s_], [s_, c]], complex)]
        if ax == "y":
            return [np.array([[c, s_], [-s_, c]], complex)]
        if ax == "z":
            return [np.array([[math.cos(th), 0], [0, math.cos(-th)]], complex)]
        raise ValueError("rotation axis")
    return None


def choose_kraus(ops: list[np.ndarray], u: float) -> int:
    """apply-quantum-channel (channel.clj:194-232): probabilities max_ij |K_ij|^2."""
    if len(ops) == 1:
        return 0
    probs = [max(z.real * z.real + z.imag * z.imag for z in m.ravel()) for m in ops]
    cum = 0.0
    for i, p in enumerate(probs):
        nc = cum + p
        if u < nc or i >= len(ops) - 1:
            return i
        cum = nc
    return len(ops) - 1


def readout_noise(outcome: int, n: int, readout: dict | None, seed: int, shot: int) -> int:
    """calculate-final-bitstring (noise.clj:107-160)."""
    if not readout:
        return outcome
    # a row that is not a map (a bare factor) adjusts nothing: `get` on a number is nil
    corr = {int(a): {int(b): f for b, f in row.items()}
            for a, row in (readout.get("correlated-errors") or {}).items() if isinstance(row, dict)}
    bits = outcome
    hist: list[int] = []
    for q in range(n):
        b = n - 1 - q
        bit = (bits >> b) & 1
        base = readout["prob-1-to-0"] if bit else readout["prob-0-to-1"]
        f = 1.0
        if corr and hist:
            for src in hist:
                if q in corr.get(src, {}):
                    f *= corr[src][q]
        eff = min(1.0, max(0.0, base * f))
        if _uniform(seed, shot, _READOUT_STREAM + q) < eff:
            bits ^= 1 << b
            hist.append(q)
    return bits


def noisy_shots(circuit: dict, noise_model: dict | None, shots: int, seed: int):
    """(outcomes after readout noise, final states) of `shots` noisy shots."""
    nm = noise_model or {}
    gate_noise = {_key(k): v for k, v in (nm.get("gate-noise") or {}).items()}
    n = circuit["num-qubits"]
    chans = {}
    outs, states = [], []
    for shot in range(shots):
        s = zero_state(n)
        site = 0
        for op in circuit["operations"]:
            enc = encode({"num-qubits": n, "operations": [op]})
            rc = lib().or_run_circuit(_dp(s), n, enc.array, enc.count, C.c_uint64(seed))
            if rc:
                raise ValueError("oracle rejected an operation")
            name = _key(op.get("operation-type"))
            cfg = gate_noise.get(name)
            if cfg is None:
                continue
            if name not in chans:
                chans[name] = kraus_channel(cfg)
            ops = chans[name]
            if ops is None:
                continue
            k = choose_kraus(ops, _uniform(seed, shot, _KRAUS_STREAM + site)) if len(ops) > 1 else 0
            site += 1
            kop = A.QgOp()
            kop.opcode = A.OP["kraus"]
            kop.nq = 1
            kop.q[0] = int((op.get("operation-params") or {}).get("target", 0) or 0)
            for j, z in enumerate(ops[k].ravel()):
                kop.m[2 * j], kop.m[2 * j + 1] = z.real, z.imag
            rc = lib().or_run_circuit(_dp(s), n, C.pointer(kop), 1, C.c_uint64(seed))
            if rc:
                raise ValueError("oracle rejected a Kraus operator")
        o = int(lib().or_sample_one(_dp(s), n, C.c_uint64(seed), C.c_uint64(shot), C.c_uint32(_MEASURE_STREAM)))
        outs.append(readout_noise(o, n, nm.get("readout-error"), seed, shot))
        states.append(s)
    return np.array(outs, np.uint64), np.array(states)


# ---------------------------------------------------------------------------
# The optimised CPU state-vector baseline (oracle/cpu_sv.c): NOT the reference's
# algorithm; it only gives the benchmark's "best CPU" figure beside the GPU's.
# ---------------------------------------------------------------------------
_sv = None


def cpu_sv_lib():
    """libcpusv.so, or None when it could not be built."""
    global _sv
    if _sv is None:
        from oracle.build import build_cpu_sv

        path = build_cpu_sv()
        if path is None:
            return None
        L = C.CDLL(str(path))
        L.sv_run_circuit.argtypes = [C.POINTER(C.c_double), C.c_int, C.POINTER(A.QgOp), C.c_int]
        L.sv_run_circuit.restype = C.c_int
        L.sv_threads.restype = C.c_int
        _sv = L
    return _sv


def cpu_sv_run(circuit: dict, state: np.ndarray | None = None) -> np.ndarray:
    """Run a circuit from |0...0> (or in place on `state`) with the CPU baseline."""
    L = cpu_sv_lib()
    if L is None:
        raise RuntimeError("the CPU state-vector baseline could not be built")
    n = circuit["num-qubits"]
    s = zero_state(n) if state is None else state
    enc = encode(circuit)
    rc = L.sv_run_circuit(_dp(s), n, enc.array, enc.count)
    if rc:
        raise ValueError(f"CPU baseline does not implement operation {rc - 1}")
    return s
