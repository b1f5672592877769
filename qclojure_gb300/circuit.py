"""Circuit data model, builders and the encoder into qg_op arrays.

A circuit is the reference's map written as a Python dict with the same keys
(src/org/soulspace/qclojure/domain/circuit.clj:15-45):

    {"num-qubits": 2, "operations": [
        {"operation-type": "h", "operation-params": {"target": 0}},
        {"operation-type": "cnot", "operation-params": {"control": 0, "target": 1}}]}

The builders mirror circuit.clj:47-888 (same names with '_' for '-', same
parameter keys). encode() resolves gate aliases (operation_registry.clj:387-422)
and the :controlled form (circuit.clj:889-931) on the host, exactly where the
reference's dispatch (circuit.clj:933-1072) does, and emits the C structs the
library consumes. circuit_depth() restates circuit.clj:1241-1449 so the result
metadata carries the same numbers.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import Any, Iterable

from . import _abi as A

Circuit = dict

# operation_registry.clj:387-407
GATE_ALIASES = {
    "not": "x", "bit-flip": "x", "phase-flip": "z", "id": "i", "cx": "cnot", "ccx": "toffoli",
    "ccnot": "toffoli", "cswap": "fredkin", "p": "phase", "u1": "phase", "sdg": "s-dag", "tdg": "t-dag",
    "phaseshift": "phase", "si": "s-dag", "ti": "t-dag",
}

# operation_registry.clj:380-383
NATIVE_SIMULATOR_GATE_SET = frozenset({
    "i", "x", "y", "z", "h", "s", "s-dag", "t", "t-dag", "rx", "ry", "rz", "phase",
    "cnot", "cz", "cy", "swap", "crx", "cry", "crz", "toffoli", "fredkin"})


def resolve_gate_alias(name: str) -> str:
    """operation_registry.clj:409-422"""
    return GATE_ALIASES.get(name, name)


class CircuitError(ValueError):
    """Raised where the reference's dispatch throws ex-info."""


# ---------------------------------------------------------------------------
# builders (circuit.clj:47-888)
# ---------------------------------------------------------------------------
def create_circuit(num_qubits: int, name: str | None = None, description: str | None = None) -> Circuit:
    if not isinstance(num_qubits, int) or num_qubits < 1:
        raise CircuitError("num-qubits must be a positive integer")
    c: Circuit = {"num-qubits": num_qubits, "operations": []}
    if name is not None:
        c["name"] = name
    if description is not None:
        c["description"] = description
    return c


def add_operation(circuit: Circuit, operation_type: str, params: dict | None = None) -> Circuit:
    op: dict[str, Any] = {"operation-type": operation_type}
    if params:
        op["operation-params"] = dict(params)
    return {**circuit, "operations": [*circuit["operations"], op]}


def add_gate(circuit: Circuit, gate_type: str, **params) -> Circuit:
    return add_operation(circuit, gate_type, {k.replace("_", "-"): v for k, v in params.items()})


def _one(name):
    def f(circuit: Circuit, target: int = 0) -> Circuit:
        return add_gate(circuit, name, target=target)
    f.__name__ = name.replace("-", "_") + "_gate"
    return f


def _rot(name):
    def f(circuit: Circuit, target: int, angle: float) -> Circuit:
        return add_gate(circuit, name, target=target, angle=angle)
    f.__name__ = name + "_gate"
    return f


x_gate, y_gate, z_gate, i_gate, h_gate = _one("x"), _one("y"), _one("z"), _one("i"), _one("h")
s_gate, s_dag_gate, t_gate, t_dag_gate = _one("s"), _one("s-dag"), _one("t"), _one("t-dag")
rx_gate, ry_gate, rz_gate, phase_gate = _rot("rx"), _rot("ry"), _rot("rz"), _rot("phase")


def cnot_gate(circuit, control, target):
    return add_gate(circuit, "cnot", control=control, target=target)


def cz_gate(circuit, control, target):
    return add_gate(circuit, "cz", control=control, target=target)


def cy_gate(circuit, control, target):
    return add_gate(circuit, "cy", control=control, target=target)


def crx_gate(circuit, control, target, angle):
    return add_gate(circuit, "crx", control=control, target=target, angle=angle)


def cry_gate(circuit, control, target, angle):
    return add_gate(circuit, "cry", control=control, target=target, angle=angle)


def crz_gate(circuit, control, target, angle):
    return add_gate(circuit, "crz", control=control, target=target, angle=angle)


def swap_gate(circuit, qubit1, qubit2):
    return add_gate(circuit, "swap", qubit1=qubit1, qubit2=qubit2)


def iswap_gate(circuit, qubit1, qubit2):
    return add_gate(circuit, "iswap", qubit1=qubit1, qubit2=qubit2)


def toffoli_gate(circuit, control1, control2, target):
    return add_gate(circuit, "toffoli", control1=control1, control2=control2, target=target)


def fredkin_gate(circuit, control, target1, target2):
    return add_gate(circuit, "fredkin", control=control, target1=target1, target2=target2)


def rydberg_cz_gate(circuit, control, target):
    return add_gate(circuit, "rydberg-cz", control=control, target=target)


def rydberg_cphase_gate(circuit, control, target, phi):
    return add_gate(circuit, "rydberg-cphase", control=control, target=target, angle=phi)


def rydberg_blockade_gate(circuit, qubit_indices, phi):
    return add_gate(circuit, "rydberg-blockade", qubit_indices=list(qubit_indices), angle=phi)


def global_x_gate(circuit):
    return add_gate(circuit, "global-x")


def global_y_gate(circuit):
    return add_gate(circuit, "global-y")


def global_z_gate(circuit):
    return add_gate(circuit, "global-z")


def global_hadamard_gate(circuit):
    return add_gate(circuit, "global-h")


def global_rx_gate(circuit, angle):
    return add_gate(circuit, "global-rx", angle=angle)


def global_ry_gate(circuit, angle):
    return add_gate(circuit, "global-ry", angle=angle)


def global_rz_gate(circuit, angle):
    return add_gate(circuit, "global-rz", angle=angle)


def measure_operation(circuit, qubits):
    return add_operation(circuit, "measure", {"measurement-qubits": list(qubits)})


def measure_all_operation(circuit):
    return measure_operation(circuit, range(circuit["num-qubits"]))


def bell_state_circuit():
    """circuit.clj:1651: H(0), CNOT(0,1)."""
    return cnot_gate(h_gate(create_circuit(2, "Bell State"), 0), 0, 1)


def ghz_state_circuit(n: int):
    """circuit.clj:1675: H(0) then a CNOT chain."""
    c = h_gate(create_circuit(n, "GHZ State"), 0)
    for i in range(1, n):
        c = cnot_gate(c, i - 1, i)
    return c


# an extension used for QAOA cost layers: exp(-i angle/2 Z Z)
def rzz_gate(circuit, qubit1, qubit2, angle):
    return add_gate(circuit, "rzz", qubit1=qubit1, qubit2=qubit2, angle=angle)


# ---------------------------------------------------------------------------
# encoder
# ---------------------------------------------------------------------------
_SINGLE = {"x", "y", "z", "h", "s", "s-dag", "t", "t-dag"}
_ROT = {"rx", "ry", "rz", "phase"}
_GLOBAL = {"global-rx", "global-ry", "global-rz", "global-h", "global-x", "global-y", "global-z"}


def _need(params, keys, msg, op):
    for k in keys:
        if params.get(k) is None:
            raise CircuitError(f"{msg}: {op}")
    return [params[k] for k in keys]


def _qubit(v) -> int:
    if not isinstance(v, int) or isinstance(v, bool) or v < 0 or v >= 256:
        raise CircuitError(f"qubit index must be a non-negative integer, got {v!r}")
    return v


def op_struct(opcode: int, qubits: Iterable[int] = (), angle: float = 0.0, matrix=None) -> A.QgOp:
    s = A.QgOp()
    s.opcode = opcode
    qs = [_qubit(q) for q in qubits]
    if len(qs) > A.QG_MAX_OP_QUBITS:
        raise CircuitError("too many operands")
    s.nq = len(qs)
    for i, q in enumerate(qs):
        s.q[i] = q
    s.angle = float(angle)
    if matrix is not None:
        flat = []
        for row in matrix:
            for z in row:
                z = complex(z)
                flat += [z.real, z.imag]
        if len(flat) != 8:
            raise CircuitError("matrix must be 2x2")
        for i, v in enumerate(flat):
            s.m[i] = v
    return s


def encode_operation(op: dict) -> list[A.QgOp]:
    """One reference operation -> qg_op structs (circuit.clj:933-1112)."""
    otype = op.get("operation-type")
    params = op.get("operation-params") or {}
    if otype == "measure":
        mq = params.get("measurement-qubits")
        if mq is None:
            raise CircuitError("Measure requires measurement-qubits parameter")
        return [op_struct(A.OP["measure"], list(mq))]
    gt = resolve_gate_alias(otype)
    target = params.get("target")
    angle = params.get("angle")
    if gt in _SINGLE:
        return [op_struct(A.OP[gt.replace("-", "_")], [target if target is not None else 0])]
    if gt in _ROT:
        return [op_struct(A.OP[gt], [target if target is not None else 0], angle if angle is not None else 0.0)]
    if gt in ("cnot", "cz"):
        c, t = _need(params, ["control", "target"], f"{gt.upper()} requires both control and target qubits", op)
        return [op_struct(A.OP[gt], [c, t])]
    if gt in ("crz", "crx", "cry"):
        c, t, a = _need(params, ["control", "target", "angle"],
                        f"{gt.upper()} requires control, target qubits and angle", op)
        return [op_struct(A.OP[gt], [c, t], a)]
    if gt in ("swap", "iswap"):
        q1, q2 = _need(params, ["qubit1", "qubit2"], f"{gt.upper()} requires both qubit1 and qubit2 parameters", op)
        return [op_struct(A.OP[gt], [q1, q2])]
    if gt == "toffoli":
        return [op_struct(A.OP["toffoli"], _need(params, ["control1", "control2", "target"],
                                                 "Toffoli requires control1, control2, and target parameters", op))]
    if gt == "fredkin":
        return [op_struct(A.OP["fredkin"], _need(params, ["control", "target1", "target2"],
                                                 "Fredkin requires control, target1, and target2 parameters", op))]
    if gt == "rydberg-cz":
        return [op_struct(A.OP["rydberg_cz"], _need(params, ["control", "target"],
                                                    "Rydberg CZ requires both control and target qubits", op))]
    if gt == "rydberg-cphase":
        c, t, a = _need(params, ["control", "target", "angle"],
                        "Rydberg CPhase requires control, target qubits and phase angle", op)
        return [op_struct(A.OP["rydberg_cphase"], [c, t], a)]
    if gt == "rydberg-blockade":
        qi, a = _need(params, ["qubit-indices", "angle"],
                      "Rydberg blockade requires qubit-indices vector and phase angle", op)
        return [op_struct(A.OP["rydberg_blockade"], list(qi), a)]
    if gt in _GLOBAL:
        if gt in ("global-rx", "global-ry", "global-rz") and angle is None:
            raise CircuitError(f"Global {gt[-2:].upper()} requires rotation angle")
        return [op_struct(A.OP[gt.replace("-", "_")], [], angle or 0.0)]
    if gt == "controlled":
        # circuit.clj:889-931: one control and one target only; :x/:z/:y controlled,
        # :h/:s/:t applied to the target uncontrolled, anything else leaves the state unchanged
        cq = params.get("control-qubits")
        tg = params.get("target-gate")
        if cq is None or tg is None:
            raise CircuitError("Controlled gate requires control-qubits and target-gate")
        tq = params.get("target-qubits") or [0]
        if len(cq) != 1 or len(tq) != 1:
            raise CircuitError("Multi-controlled gates with >1 control qubit not fully implemented")
        c, t = cq[0], tq[0]
        if tg == "x":
            return [op_struct(A.OP["cnot"], [c, t])]
        if tg == "z":
            return [op_struct(A.OP["cz"], [c, t])]
        if tg == "y":
            return [op_struct(A.OP["cy"], [c, t])]
        if tg in ("h", "s", "t"):
            return [op_struct(A.OP[tg], [t])]
        return []
    if gt == "rzz":
        q1, q2, a = _need(params, ["qubit1", "qubit2", "angle"], "RZZ requires qubit1, qubit2 and angle", op)
        return [op_struct(A.OP["rzz"], [q1, q2], a)]
    if gt == "u":
        return [op_struct(A.OP["u"], [target if target is not None else 0], 0.0, params["matrix"])]
    # :i, :cy and anything else: the reference dispatch throws (circuit.clj:1072)
    raise CircuitError(f"Unknown gate type: {gt}")


def validate_circuit(circuit: Circuit) -> None:
    """The ::circuit spec (circuit.clj:30-45) checked by backend.clj:228-230."""
    if not isinstance(circuit, dict):
        raise CircuitError("circuit must be a map")
    n = circuit.get("num-qubits")
    if not isinstance(n, int) or isinstance(n, bool) or n < 1:
        raise CircuitError("circuit :num-qubits must be a positive integer")
    ops = circuit.get("operations")
    if not isinstance(ops, list):
        raise CircuitError("circuit :operations must be a vector")
    for op in ops:
        if not isinstance(op, dict) or not isinstance(op.get("operation-type"), str):
            raise CircuitError("every operation needs an :operation-type")


class EncodedCircuit:
    """A qg_circuit plus the ctypes array that backs it."""

    def __init__(self, circuit: Circuit):
        validate_circuit(circuit)
        self.num_qubits = circuit["num-qubits"]
        structs: list[A.QgOp] = []
        for op in circuit["operations"]:
            structs += encode_operation(op)
        self.count = len(structs)
        self.array = (A.QgOp * max(1, self.count))(*structs)
        self.c = A.QgCircuit(self.num_qubits, self.count, C.cast(self.array, C.POINTER(A.QgOp)))

    def ref(self):
        return C.byref(self.c)


def encode(circuit: Circuit) -> EncodedCircuit:
    return EncodedCircuit(circuit)


# ---------------------------------------------------------------------------
# metadata (circuit.clj:1241-1470)
# ---------------------------------------------------------------------------
def _qubits_with_spans(op: dict, n: int):
    p = op.get("operation-params") or {}
    t = op.get("operation-type")
    if t == "measure":
        return list(p.get("measurement-qubits") or []), []
    if t in ("x", "y", "z", "h", "s", "s-dag", "t", "t-dag", "rx", "ry", "rz", "phase"):
        return [p.get("target")], []
    if t in ("cnot", "cx", "cz", "cy", "crx", "cry", "crz", "rydberg-cz", "rydberg-cphase"):
        c, tg = p.get("control"), p.get("target")
        return [c, tg], [(min(c, tg), max(c, tg))]
    if t == "rydberg-blockade":
        qi = list(p.get("qubit-indices"))
        return qi, [(min(qi), max(qi))]
    if t in _GLOBAL:
        return [], []  # the reference counts (:qubits operation), which is absent: no qubits
    if t in ("swap", "iswap"):
        a, b = p.get("qubit1"), p.get("qubit2")
        return [a, b], [(min(a, b), max(a, b))]
    if t == "toffoli":
        q = [p.get("control1"), p.get("control2"), p.get("target")]
        return q, [(min(q), max(q))]
    if t == "fredkin":
        q = [p.get("control"), p.get("target1"), p.get("target2")]
        return q, [(min(q), max(q))]
    q = [p.get(k) for k in ("target", "control", "qubit1", "qubit2", "control1", "control2", "target1", "target2")]
    return [x for x in q if x is not None], []


def circuit_depth(circuit: Circuit) -> int:
    """circuit.clj:1375-1449: an op's layer is one past the latest layer among its
    qubits, the spans (min..max qubit ranges of multi-qubit ops) that overlap its
    own span, and, for an op without a span, the spans covering its qubits. Two
    spans overlap exactly when some qubit lies in both, and a span's layer only
    grows, so the latest layer of any span covering qubit q is kept per qubit
    (cover[q]); each op then costs O(n) instead of a scan of every span seen."""
    ops = circuit["operations"]
    n = circuit["num-qubits"]
    if not ops:
        return 0
    qubit_layers = [0] * n
    cover = [0] * n
    max_layer = 0
    for op in ops:
        qubits, spans = _qubits_with_spans(op, n)
        qubits = [q for q in qubits if q is not None]
        mq = max([qubit_layers[q] for q in qubits], default=0)
        ms = max([cover[q] for a, b in spans for q in range(max(a, 0), min(b, n - 1) + 1)], default=0)
        mc = max([cover[q] for q in qubits if 0 <= q < n], default=0) if not spans else 0
        new = 1 + max(mq, ms, mc)
        for q in qubits:
            qubit_layers[q] = new
        for a, b in spans:
            for q in range(max(a, 0), min(b, n - 1) + 1):
                if cover[q] < new:
                    cover[q] = new
        max_layer = max(max_layer, new)
    return max_layer


def _circuit_depth_by_spans(circuit: Circuit) -> int:
    """The same layering by a scan of every span seen (the reference's form); kept
    to check circuit_depth against."""
    ops = circuit["operations"]
    n = circuit["num-qubits"]
    if not ops:
        return 0
    qubit_layers = [0] * n
    span_layers: dict[tuple, int] = {}
    max_layer = 0
    for op in ops:
        qubits, spans = _qubits_with_spans(op, n)
        qubits = [q for q in qubits if q is not None]
        mq = max([qubit_layers[q] for q in qubits], default=0)
        ms = max([layer for sp, layer in span_layers.items() for os in spans
                  if not (sp[1] < os[0] or os[1] < sp[0])], default=0)
        mc = max([layer for sp, layer in span_layers.items() for q in qubits if sp[0] <= q <= sp[1]],
                 default=0) if not spans else 0
        new = 1 + max(mq, ms, mc)
        for q in qubits:
            qubit_layers[q] = new
        for sp in spans:
            span_layers[sp] = new
        max_layer = max(max_layer, new)
    return max_layer


def circuit_operation_count(circuit: Circuit) -> int:
    return len(circuit["operations"])


def circuit_gate_count(circuit: Circuit) -> int:
    return sum(1 for op in circuit["operations"] if op["operation-type"] != "measure")


def circuit_metadata(circuit: Circuit) -> dict:
    return {"circuit-depth": circuit_depth(circuit),
            "circuit-operation-count": circuit_operation_count(circuit),
            "circuit-gate-count": circuit_gate_count(circuit)}


def gate_matrix(name: str, angle: float = 0.0):
    """2x2 matrices of gate.clj:38-283 as nested complex lists."""
    s2 = 1.0 / math.sqrt(2.0)
    if name == "x":
        return [[0, 1], [1, 0]]
    if name == "y":
        return [[0, -1j], [1j, 0]]
    if name == "z":
        return [[1, 0], [0, -1]]
    if name == "h":
        return [[s2, s2], [s2, -s2]]
    if name == "i":
        return [[1, 0], [0, 1]]
    raise CircuitError(f"no matrix for {name}")
