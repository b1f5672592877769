"""DeviceState: an amplitude array resident in HBM, driven through the C ABI.

This is the state-level surface of the backend (state.clj, gate.clj and the
result extractors on one state) for callers that keep a state on the GPU
across many circuits, such as variational loops and the benchmarks.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from .backend import ARITHMETIC, PRECISIONS, FUSIONS, _check
from .circuit import encode


class Context:
    """A library context on one GPU (no job workers are needed for direct state use)."""

    def __init__(self, device: int = 0, precision: str = "c128", fusion: str = "tiled", fusion_width: int = 4,
                 workers: int = 1, seed: int = 0, arithmetic: str = "double-float", pass_kernels: str = "auto"):
        self.lib = A.load_library()
        cfg = A.QgConfig()
        cfg.device = device
        cfg.precision = PRECISIONS[precision]
        cfg.fusion = FUSIONS[fusion]
        cfg.fuse_k = fusion_width
        cfg.workers = workers
        cfg.seed = seed
        cfg.arithmetic = ARITHMETIC[arithmetic]
        cfg.pass_kernels = A.PASS_KERNELS[pass_kernels]
        ctx = C.c_void_p()
        _check(self.lib.qg_ctx_create(C.byref(cfg), C.byref(ctx)))
        self.ctx = ctx

    def close(self):
        if self.ctx:
            self.lib.qg_ctx_destroy(self.ctx)
            self.ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def state(self, num_qubits: int, precision: str = "c128") -> "DeviceState":
        return DeviceState(self, num_qubits, precision)

    def autotune(self, num_qubits: int, precision: str = "c128", circuit: dict | None = None) -> dict:
        """Time candidate pass-kernel shapes on a calibration circuit of num_qubits (the given
        workload, or the library's own) and keep the fastest for this context (qg_autotune);
        returns the choice and every candidate."""
        chosen = A.QgTuning()
        tried = (A.QgTuning * 16)()
        count = C.c_int32()
        enc = encode(circuit) if circuit is not None else None
        _check(self.lib.qg_autotune(self.ctx, num_qubits, PRECISIONS[precision], enc.ref() if enc else None,
                                    C.byref(chosen), tried, 16, C.byref(count)), self.lib, self.ctx)
        return {"chosen": chosen.as_dict(), "candidates": [tried[i].as_dict() for i in range(count.value)]}

    def autotune_crossover(self, precision: str = "c64", layers: int = 100) -> dict:
        """Measure from which size a one-off circuit of `layers` layers gains from compiling its
        kernels (qg_autotune_crossover); the context specialises from there on."""
        mq, cnt = C.c_int32(), C.c_int32()
        tab = (C.c_double * 32)()
        _check(self.lib.qg_autotune_crossover(self.ctx, PRECISIONS[precision], layers, C.byref(mq), tab, 8,
                                              C.byref(cnt)), self.lib, self.ctx)
        rows = [{"qubits": int(tab[4 * i]), "interpreted_ms": tab[4 * i + 1], "compile_ms": tab[4 * i + 2],
                 "specialised_ms": tab[4 * i + 3]} for i in range(cnt.value)]
        return {"min_qubits": mq.value, "rows": rows}

    def tuning(self, num_qubits: int, precision: str = "c128") -> dict:
        t = A.QgTuning()
        _check(self.lib.qg_tuning_get(self.ctx, num_qubits, PRECISIONS[precision], C.byref(t)), self.lib, self.ctx)
        return t.as_dict()

    def set_tuning(self, num_qubits: int, precision: str, tile_bits: int, reg_bits: int = 0, buffers: int = 0,
                   ctas_per_sm: int = 0) -> None:
        t = A.QgTuning(tile_bits, reg_bits, buffers, ctas_per_sm, 0.0)
        _check(self.lib.qg_tuning_set(self.ctx, num_qubits, PRECISIONS[precision], C.byref(t)), self.lib, self.ctx)


class DeviceState:
    def __init__(self, ctx: Context, num_qubits: int, precision: str = "c128"):
        self.ctx, self.lib = ctx, ctx.lib
        self.n = num_qubits
        self.precision = precision
        h = C.c_void_p()
        _check(self.lib.qg_state_create(ctx.ctx, num_qubits, PRECISIONS[precision], C.byref(h)), self.lib, ctx.ctx)
        self.h = h

    def close(self):
        if self.h:
            self.lib.qg_state_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, rc):
        _check(rc, self.lib, self.ctx.ctx)

    def set_basis(self, index: int = 0):
        self._ck(self.lib.qg_state_set_basis(self.h, C.c_uint64(index)))

    def upload(self, sv: np.ndarray):
        sv = np.ascontiguousarray(sv, dtype=np.complex128)
        assert sv.size == 1 << self.n
        self._ck(self.lib.qg_state_upload(self.h, sv.ctypes.data_as(A.DP)))

    def download(self) -> np.ndarray:
        out = np.empty(1 << self.n, np.complex128)
        self._ck(self.lib.qg_state_download(self.h, out.ctypes.data_as(A.DP)))
        return out

    def apply(self, circuit: dict, fusion: str = "tiled", seed: int = 0) -> int:
        enc = encode(circuit)
        passes = C.c_int32()
        self._ck(self.lib.qg_state_apply(self.h, enc.ref(), FUSIONS[fusion], C.c_uint64(seed), C.byref(passes)))
        return passes.value

    def prepare(self, circuit: dict, fusion: str = "tiled") -> tuple[float, int]:
        """Compile the circuit's specialised pass kernels ahead of apply(); returns
        (compile milliseconds, passes that have a kernel)."""
        enc = encode(circuit)
        ms, cnt = C.c_double(), C.c_int32()
        self._ck(self.lib.qg_state_prepare(self.h, enc.ref(), FUSIONS[fusion], C.byref(ms), C.byref(cnt)))
        return ms.value, cnt.value

    def profile(self, circuit: dict, fusion: str = "tiled", seed: int = 0) -> tuple[np.ndarray, np.ndarray]:
        """Apply like apply() and return per-pass device times (ms) and kinds
        (0 plain gate, 1 tiled pass, 2 measurement, 3 tiled pass run by its
        specialised kernel, 4 dense block on the tensor cores)."""
        enc = encode(circuit)
        cap = 1 << 16
        ms = (C.c_float * cap)()
        kinds = (C.c_int32 * cap)()
        n = C.c_int32()
        self._ck(self.lib.qg_state_profile(self.h, enc.ref(), FUSIONS[fusion], C.c_uint64(seed), ms, kinds, cap,
                                           C.byref(n)))
        return np.array(ms[:n.value], np.float64), np.array(kinds[:n.value], np.int32)

    def probabilities(self) -> np.ndarray:
        out = np.empty(1 << self.n, np.float64)
        self._ck(self.lib.qg_state_probabilities(self.h, out.ctypes.data_as(A.DP)))
        return out

    def sample(self, shots: int, seed: int) -> np.ndarray:
        out = np.empty(max(1, shots), np.uint64)
        self._ck(self.lib.qg_state_sample(self.h, C.c_uint64(shots), C.c_uint64(seed), out.ctypes.data_as(A.U64P)))
        return out[:shots]

    def sample_sums(self) -> tuple[np.ndarray, int]:
        """The sampler's quantised probability sums (floor(p 2^62) per amplitude) per chunk
        of min(2^n, 32) amplitudes, and their total."""
        count = max(1, (1 << self.n) // 32)
        out = np.empty(count, np.uint64)
        total = C.c_uint64()
        self._ck(self.lib.qg_diag_sample_sums(self.h, out.ctypes.data_as(A.U64P), C.c_uint64(count),
                                              C.byref(total)))
        return out, int(total.value)

    def sample_noalloc(self, shots: int, seed: int, device_outcomes: int) -> None:
        """Write `shots` outcomes (uint64) to caller-owned device memory at address
        `device_outcomes`; no device allocation (states of at most 24 qubits)."""
        self._ck(self.lib.qg_state_sample_noalloc(self.h, C.c_uint64(shots), C.c_uint64(seed),
                                                  C.c_void_p(device_outcomes)))

    def pauli_expectation(self, pauli: str) -> float:
        out = C.c_double()
        self._ck(self.lib.qg_state_pauli_expectation(self.h, pauli.encode(), C.byref(out)))
        return out.value

    def hamiltonian(self, terms: list[tuple[float, str]]) -> float:
        coeffs = (C.c_double * max(1, len(terms)))(*[c for c, _ in terms])
        strs = "".join(s for _, s in terms).encode()
        out = C.c_double()
        self._ck(self.lib.qg_state_hamiltonian(self.h, len(terms), coeffs, strs, C.byref(out)))
        return out.value

    def expectation_1q(self, obs, target: int) -> float:
        flat = []
        for row in obs:
            for z in row:
                z = complex(z)
                flat += [z.real, z.imag]
        arr = (C.c_double * 8)(*flat)
        out = C.c_double()
        self._ck(self.lib.qg_state_expectation_1q(self.h, arr, target, C.byref(out)))
        return out.value

    def norm2(self) -> float:
        out = C.c_double()
        self._ck(self.lib.qg_state_norm2(self.h, C.byref(out)))
        return out.value

    def inner(self, other: "DeviceState") -> complex:
        re, im = C.c_double(), C.c_double()
        self._ck(self.lib.qg_state_inner(self.h, other.h, C.byref(re), C.byref(im)))
        return complex(re.value, im.value)

    def compare(self, reference: "DeviceState") -> dict:
        """Distance from a complex128 state of the same size: the largest amplitude
        difference, 1 - fidelity and the total variation distance of the outcome
        distributions."""
        out = (C.c_double * 3)()
        self._ck(self.lib.qg_state_compare(self.h, reference.h, out))
        return {"max_abs_diff": out[0], "one_minus_fidelity": out[1], "tvd": out[2]}

    def measure(self, qubits: list[int], seed: int) -> tuple[int, float]:
        arr = (C.c_int32 * len(qubits))(*qubits)
        o, p = C.c_uint64(), C.c_double()
        self._ck(self.lib.qg_state_measure(self.h, arr, len(qubits), C.c_uint64(seed), C.byref(o), C.byref(p)))
        return o.value, p.value

    def device_ptr(self):
        d, s = C.c_void_p(), C.c_void_p()
        self._ck(self.lib.qg_state_device_ptr(self.h, C.byref(d), C.byref(s)))
        return d.value, s.value

    def synchronize(self):
        self._ck(self.lib.qg_state_synchronize(self.h))
