"""Parameter sweeps: many circuits of one structure, one launch per pass, graph replays.

This is the batched form of the reference's variational loop
(src/org/soulspace/qclojure/application/algorithm/variational_algorithm.clj:310-363,
qaoa.clj:1087-1115): the same circuit structure is executed for many parameter
vectors and each run is reduced to an energy <H>. Circuits of equal qubit count
and equal pass structure share one kernel launch per HBM pass (over all of
their states); the pass sequence is captured once into a CUDA graph and
replayed by every run; new angles only rewrite the op records in HBM.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from .backend import ARITHMETIC, PRECISIONS, _check
from .circuit import encode


class Sweep:
    def __init__(self, ctx, circuits: list[dict], precision: str = "c64", arithmetic: str = "double-float"):
        """ctx: a qclojure_gb300.state.Context."""
        self.ctx, self.lib = ctx, ctx.lib
        self.n = [c["num-qubits"] for c in circuits]
        self.count = len(circuits)
        encs, arr = self._encode(circuits)
        h = C.c_void_p()
        _check(self.lib.qg_sweep_create(ctx.ctx, arr, self.count, PRECISIONS[precision], ARITHMETIC[arithmetic],
                                        C.byref(h)), self.lib, ctx.ctx)
        self.h = h

    @staticmethod
    def _encode(circuits):
        encs = [encode(c) for c in circuits]
        arr = (A.QgCircuit * len(encs))(*[e.c for e in encs])
        return encs, arr

    def update(self, circuits: list[dict]) -> None:
        encs, arr = self._encode(circuits)
        _check(self.lib.qg_sweep_update(self.h, arr, len(circuits)), self.lib, self.ctx.ctx)

    def run(self, hamiltonians: list[list[dict]] | None = None) -> tuple[np.ndarray | None, dict]:
        """Run all circuits from |0...0>; return (energies or None, stats)."""
        stats = A.QgSweepStats()
        if hamiltonians is None:
            _check(self.lib.qg_sweep_run(self.h, None, None, None, None, C.byref(stats)), self.lib, self.ctx.ctx)
            return None, self._stats(stats)
        offs = [0]
        coeffs: list[float] = []
        strs: list[str] = []
        for c, terms in enumerate(hamiltonians):
            for t in terms:
                if len(t["pauli-string"]) != self.n[c]:
                    raise ValueError("pauli strings must have num-qubits characters")
                coeffs.append(float(t["coefficient"]))
                strs.append(t["pauli-string"])
            offs.append(len(coeffs))
        o = (C.c_int32 * len(offs))(*offs)
        co = (C.c_double * max(1, len(coeffs)))(*coeffs)
        ps = "".join(strs).encode()
        en = np.zeros(self.count)
        _check(self.lib.qg_sweep_run(self.h, o, co, ps, en.ctypes.data_as(A.DP), C.byref(stats)),
               self.lib, self.ctx.ctx)
        return en, self._stats(stats)

    @staticmethod
    def _stats(s) -> dict:
        return {"device-ms": s.device_ms, "expect-ms": s.expect_ms, "groups": s.groups, "launches": s.launches,
                "graphs": s.graphs, "specialised": s.specialised, "state-bytes": s.state_bytes,
                "pass-bytes": s.pass_bytes, "level-graph-ms": s.level_graph_ms,
                "size-graphs-ms": s.size_graphs_ms}

    def state(self, c: int) -> np.ndarray:
        out = np.empty(1 << self.n[c], np.complex128)
        _check(self.lib.qg_sweep_state(self.h, c, out.ctypes.data_as(A.DP)), self.lib, self.ctx.ctx)
        return out

    def close(self):
        if self.h:
            self.lib.qg_sweep_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
