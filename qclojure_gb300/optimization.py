"""The first stages of the reference's hardware optimisation pipeline on the host.

application/hardware_optimization.clj:42-109 runs gate optimisation, qubit
optimisation, error correction, topology routing and gate decomposition. The first
two are restated here, as the reference defines them:

* `optimize_gates` (domain/gate_optimization.clj:776-860): repeat until nothing
  changes: cancel S/S†, T/T† and self-inverse pairs that meet with no gate between them
  on any of their qubits; fold consecutive rotations about one axis on one qubit
  (S, T, phase and RZ all count as Z rotations, and fold into an RZ of the summed angle
  modulo 2π); drop rotations of angle 0 (mod 2π); cancel equal self-inverse gates.
  A circuit optimised to nothing is an error ("Optimization resulted in an empty circuit").
* `optimize_qubit_usage` (domain/qubit_optimization.clj:104-150): renumber the qubits
  that operations use to 0..k-1 and shrink the register.

The hardware simulator calls the pipeline on submission and runs the original
circuit (hardware_simulator.clj:300-330): the pipeline only decides whether a job
fails. The ideal simulator's tiled passes do their own fusion on the device.
"""
from __future__ import annotations

import math

SELF_INVERSE = frozenset({"x", "y", "z", "h", "cnot", "cx", "cy", "cz", "swap", "toffoli", "ccx", "fredkin", "cswap",
                          "rydberg-cz", "global-x", "global-y", "global-z", "global-h"})
ROTATIONS = frozenset({"rx", "ry", "rz", "phase", "s", "s-dag", "t", "t-dag"})
INVERSE_PAIRS = {"s": "s-dag", "s-dag": "s", "t": "t-dag", "t-dag": "t"}
ANGLE_TOLERANCE = 1e-12
TWO_PI = 2 * math.pi
_QUBIT_KEYS = ("target", "control", "control1", "control2", "target1", "target2", "swap1", "swap2",
               "qubit1", "qubit2")


class OptimizationError(ValueError):
    """Raised where the reference throws ex-info from its optimisation pipeline."""


def normalize_angle(angle: float) -> float:
    """gate_optimization.clj:110-124: (rem (mod a 2π) 2π), near 0 or 2π -> 0."""
    n = math.fmod(angle % TWO_PI, TWO_PI)
    if n < ANGLE_TOLERANCE or TWO_PI - n < ANGLE_TOLERANCE:
        return 0.0
    return n


def rotation_angle(op: dict):
    g = op.get("operation-type")
    if g in ("rx", "ry", "rz", "phase"):
        return (op.get("operation-params") or {}).get("angle")
    return {"s": math.pi / 2, "s-dag": -(math.pi / 2), "t": math.pi / 4, "t-dag": -(math.pi / 4)}.get(g)


def rotation_axis(op: dict):
    g = op.get("operation-type")
    return "x" if g == "rx" else "y" if g == "ry" else "z" if g in ("rz", "phase", "s", "s-dag", "t", "t-dag") else None


def gate_qubits(op: dict) -> frozenset:
    """gate_optimization.clj:250-314."""
    p = op.get("operation-params") or {}
    g = op.get("operation-type")
    if g in ("x", "y", "z", "h", "s", "s-dag", "t", "t-dag", "rx", "ry", "rz", "phase"):
        return frozenset({p.get("target")})
    if g in ("cnot", "cx", "cz", "cy", "crx", "cry", "crz", "rydberg-cz", "rydberg-cphase"):
        return frozenset({p.get("control"), p.get("target")})
    if g == "rydberg-blockade":
        return frozenset(p.get("qubit-indices") or [])
    if g in ("swap", "iswap"):
        return frozenset({p.get("qubit1"), p.get("qubit2")})
    if g == "toffoli":
        return frozenset({p.get("control1"), p.get("control2"), p.get("target")})
    if g == "fredkin":
        return frozenset({p.get("control"), p.get("target1"), p.get("target2")})
    if g in ("global-x", "global-y", "global-z", "global-h", "global-rx", "global-ry", "global-rz"):
        cq = p.get("circuit-qubits")
        return frozenset(range(cq)) if cq else frozenset()
    return frozenset()


def rotations_combinable(a: dict, b: dict) -> bool:
    return (a.get("operation-type") in ROTATIONS and b.get("operation-type") in ROTATIONS
            and rotation_axis(a) == rotation_axis(b)
            and (a.get("operation-params") or {}).get("target") == (b.get("operation-params") or {}).get("target"))


def combine_rotations(a: dict, b: dict):
    """gate_optimization.clj:209-248: None when the sum is the identity."""
    ang = normalize_angle(rotation_angle(a) + rotation_angle(b))
    if ang < ANGLE_TOLERANCE:
        return None
    t = (a.get("operation-params") or {}).get("target")
    return {"operation-type": "r" + rotation_axis(a), "operation-params": {"target": t, "angle": ang}}


def gates_equivalent(a: dict, b: dict) -> bool:
    """gate_optimization.clj:365-419 (SWAP symmetric)."""
    g = a.get("operation-type")
    if g != b.get("operation-type") or g not in SELF_INVERSE:
        return False
    pa, pb = a.get("operation-params"), b.get("operation-params")
    if g == "swap":
        pa, pb = pa or {}, pb or {}
        return pa == pb or (pa.get("qubit1") == pb.get("qubit2") and pa.get("qubit2") == pb.get("qubit1"))
    return pa == pb


def gates_are_inverses(a: dict, b: dict) -> bool:
    """gate_optimization.clj:333-363."""
    if gate_qubits(a) != gate_qubits(b):
        return False
    ga, gb = a.get("operation-type"), b.get("operation-type")
    pa, pb = a.get("operation-params"), b.get("operation-params")
    return (ga == gb and ga in SELF_INVERSE and pa == pb) or (INVERSE_PAIRS.get(ga) == gb and pa == pb)


def next_gate_on_same_qubits(ops: list, start: int, qubits: frozenset):
    """gate_optimization.clj:421-452: the next op on exactly these qubits, unless an op
    sharing any of them comes first."""
    for i in range(start + 1, len(ops)):
        q = gate_qubits(ops[i])
        if q == qubits:
            return i
        if q & qubits:
            return None
    return None


def _pairs(ops: list, eligible, match) -> list:
    pairs, used = [], set()
    for i, op in enumerate(ops):
        if i in used or not eligible(op):
            continue
        j = next_gate_on_same_qubits(ops, i, gate_qubits(op))
        if j is not None and j not in used and match(op, ops[j]):
            pairs.append((i, j))
            used.update((i, j))
    return pairs


def find_cancellation_pairs(ops: list) -> list:
    return _pairs(ops, lambda o: o.get("operation-type") in SELF_INVERSE, gates_equivalent)


def find_inverse_cancellation_pairs(ops: list) -> list:
    return _pairs(ops, lambda o: True, gates_are_inverses)


def remove_pairs(ops: list, pairs) -> list:
    drop = {i for p in pairs for i in p}
    return [o for i, o in enumerate(ops) if i not in drop]


def find_rotation_folding_pairs(ops: list) -> list:
    """gate_optimization.clj:611-664: ((i, j), combined op or None)."""
    out, used = [], set()
    for i, op in enumerate(ops):
        if i in used or op.get("operation-type") not in ROTATIONS:
            continue
        j = next_gate_on_same_qubits(ops, i, gate_qubits(op))
        if j is not None and j not in used and rotations_combinable(op, ops[j]):
            out.append(((i, j), combine_rotations(op, ops[j])))
            used.update((i, j))
    return out


def apply_rotation_folding(ops: list, folds) -> list:
    drop = {i for (ij, _) in folds for i in ij}
    repl = {ij[0]: g for (ij, g) in folds if g is not None}
    out = []
    for i, o in enumerate(ops):
        if i in repl:
            out.append(repl[i])
        elif i not in drop:
            out.append(o)
    return out


def _until_stable(ops: list, step) -> list:
    while True:
        new = step(ops)
        if new is None:
            return ops
        ops = new


def optimize_rotations(ops: list) -> list:
    return _until_stable(ops, lambda o: (lambda f: apply_rotation_folding(o, f) if f else None)(
        find_rotation_folding_pairs(o)))


def optimize_inverse_cancellations(ops: list) -> list:
    return _until_stable(ops, lambda o: (lambda p: remove_pairs(o, p) if p else None)(
        find_inverse_cancellation_pairs(o)))


def is_identity_rotation(op: dict) -> bool:
    if op.get("operation-type") not in ROTATIONS:
        return False
    a = (op.get("operation-params") or {}).get("angle")
    return a is not None and abs(normalize_angle(a)) < ANGLE_TOLERANCE


def optimize_gates(circuit: dict, options: dict | None = None) -> dict:
    """optimize-gates (gate_optimization.clj:776-860) on a circuit; returns the circuit."""
    o = options or {}
    if not o.get("optimize-gates?", True):
        return circuit
    rot, inv = o.get("optimize-rotations?", True), o.get("optimize-inverse-pairs?", True)
    ops = list(circuit.get("operations") or [])
    while True:
        cur = optimize_inverse_cancellations(ops) if inv else ops
        if rot:
            cur = [x for x in optimize_rotations(cur) if not is_identity_rotation(x)]
        pairs = find_cancellation_pairs(cur)
        if not pairs:
            ops = cur
            break
        ops = remove_pairs(cur, pairs)
    if not ops:
        raise OptimizationError("Optimization resulted in an empty circuit")
    return {**circuit, "operations": ops}


def analyze_qubit_usage(circuit: dict) -> dict:
    """qubit_optimization.clj:35-70."""
    used = set()
    for op in circuit.get("operations") or []:
        for k, v in (op.get("operation-params") or {}).items():
            if k in _QUBIT_KEYS and isinstance(v, (int, float)) and not isinstance(v, bool):
                used.add(v)
    total = circuit["num-qubits"]
    return {"used-qubits": used, "total-qubits": total, "unused-qubits": set(range(total)) - used,
            "max-qubit-id": max(used) if used else -1,
            "qubit-usage-efficiency": len(used) / float(total) if total else 0.0}


def optimize_qubit_usage(circuit: dict, options: dict | None = None) -> tuple[dict, dict]:
    """optimize-qubit-usage (qubit_optimization.clj:104-150): (circuit, qubit mapping)."""
    o = options or {}
    if not o.get("optimize-qubits?", True):
        return circuit, {}
    used = analyze_qubit_usage(circuit)["used-qubits"]
    mapping = {old: new for new, old in enumerate(sorted(used))}
    ops = []
    for op in circuit.get("operations") or []:
        p = op.get("operation-params")
        if p is None:
            ops.append({**op, "operation-params": {}})
            continue
        ops.append({**op, "operation-params": {
            k: (mapping.get(v, v) if k in _QUBIT_KEYS and isinstance(v, (int, float)) and not isinstance(v, bool)
                else v) for k, v in p.items()}})
    out = {**circuit, "num-qubits": len(used), "operations": ops}
    if not ops:
        raise OptimizationError("Optimization resulted in an empty circuit")
    return out, mapping


def optimize(circuit: dict, options: dict | None = None) -> dict:
    """The pipeline's first stages (hardware_optimization.clj:42-109 steps 1-2)."""
    o = options or {}
    c = optimize_gates(circuit, o)
    c, mapping = optimize_qubit_usage(c, o)
    return {"circuit": c, "qubit-mapping": mapping, "pipeline-order": ["gate-cancellation", "qubit-optimization"]}
