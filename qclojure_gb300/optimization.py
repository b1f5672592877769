"""The reference's hardware optimisation pipeline on the host.

application/hardware_optimization.clj:42-109 runs gate optimisation, qubit
optimisation, error correction, topology routing and gate decomposition. Error
correction lives in `error_correction.py` and routing in `topology.py`; gate
optimisation, qubit optimisation and gate decomposition are restated here, as the
reference defines them:

* `optimize_gates` (domain/gate_optimization.clj:776-860): repeat until nothing
  changes: cancel S/S†, T/T† and self-inverse pairs that meet with no gate between them
  on any of their qubits; fold consecutive rotations about one axis on one qubit
  (S, T, phase and RZ all count as Z rotations, and fold into an RZ of the summed angle
  modulo 2π); drop rotations of angle 0 (mod 2π); cancel equal self-inverse gates.
  A circuit optimised to nothing is an error ("Optimization resulted in an empty circuit").
* `optimize_qubit_usage` (domain/qubit_optimization.clj:104-150): renumber the qubits
  that operations use to 0..k-1 and shrink the register.
* `transform_circuit` (domain/circuit_transformation.clj:21-74 with
  gate_decomposition.clj): decompose operations the device does not support through
  the operation catalog's decomposition entries, one at a time, at most
  :max-iterations (100) steps ("Maximum iterations reached during circuit transformation").

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


# ---------------------------------------------------------------------------
# Gate decomposition (domain/gate_decomposition.clj, with the decomposition entries of
# the operation catalog, domain/operation_registry.clj:53-370)
# ---------------------------------------------------------------------------
_PI = math.pi
# vector steps are tuples (gate, specs...), keyword steps plain strings
CATALOG_DECOMPOSITIONS = {
    "x": {"universal": ["ry"], "parametric-fn": lambda _: [("ry", _PI)], "rz-only": ["rz", "h", "rz", "h"]},
    "y": {"universal": ["s", "x", "s-dag"],
          "parametric-fn": lambda _: [("rz", _PI / 2), ("ry", _PI), ("rz", _PI / -2)],
          "t-basis": ["t", "t", "x", "t", "t", "t", "t"]},
    "z": {"universal": ["t", "t", "t", "t"], "parametric-fn": lambda _: [("rz", _PI)], "s-basis": ["s", "s"]},
    "i": {"universal": [], "parametric-fn": lambda _: [], "nop": True},
    "h": None,
    "s": {"universal": ["t", "t"], "parametric-fn": lambda _: [("rz", _PI / 2)]},
    "s-dag": {"universal": ["t-dag", "t-dag"], "parametric-fn": lambda _: [("rz", _PI / -2)]},
    "t": None,
    "t-dag": {"parametric-fn": lambda _: [("rz", _PI / -4)]},
    "rx": {"universal-fn": lambda th: [("h",), ("rz", th), ("h",)],
           "ry-rz-fn": lambda th: [("ry", _PI / 2), ("rz", th), ("ry", _PI / -2)]},
    "ry": {"universal-fn": lambda th: [("rx", _PI / 2), ("rz", th), ("rx", _PI / -2)]},
    "rz": None,
    "phase": ["rz"],
    "cnot": None,
    "cz": {"cnot-h": [("h", "target"), ("cnot", "control", "target"), ("h", "target")]},
    "cy": {"cnot-s": [("s-dag", "target"), ("cnot", "control", "target"), ("s", "target")]},
    "swap": {"cnot": [("cnot", "target1", "target2"), ("cnot", "target2", "target1"), ("cnot", "target1", "target2")]},
    "iswap": {"cnot-s": [("s", "target1"), ("s", "target2"), ("h", "target1"), ("cnot", "target1", "target2"),
                         ("cnot", "target2", "target1"), ("h", "target2")]},
    "crx": ["cnot", "rx"], "cry": ["cnot", "ry"], "crz": ["cnot", "rz"],
    "toffoli": {"cnot-t": [("h", "target"), ("cnot", "control2", "target"), ("t-dag", "target"),
                           ("cnot", "control1", "target"), ("t", "target"), ("cnot", "control2", "target"),
                           ("t-dag", "target"), ("cnot", "control1", "target"), ("t", "control2"), ("t", "target"),
                           ("cnot", "control1", "control2"), ("h", "target"), ("t", "control1"),
                           ("t-dag", "control2"), ("cnot", "control1", "control2")]},
    "fredkin": {"cnot-toffoli": [("cnot", "target2", "target1"), ("toffoli", "control", "target1", "target2"),
                                 ("cnot", "target2", "target1")]},
    "rydberg-cz": {"standard": ["cz"]},
    "rydberg-cphase": {"standard-fn": lambda phi: [("crz", phi)]},
    "rydberg-blockade": None,
    **{g: {"single-qubit-fn": None} for g in ("global-rx", "global-ry", "global-rz", "global-h", "global-x",
                                               "global-y", "global-z")},
    "measure": None,
}
_SELECT = ("target", "control", "control1", "control2", "target1", "target2")


def _select(params: dict) -> dict:
    return {k: params[k] for k in _SELECT if k in params}


def _step_op(step, params: dict) -> dict:
    if isinstance(step, tuple):
        g, specs = step[0], step[1:]
        if g in ("rz", "rx", "ry") and len(specs) == 1 and isinstance(specs[0], (int, float)):
            p = {"target": params.get("target"), "angle": specs[0]}
        elif g == "cnot":
            if len(specs) < 2:
                raise OptimizationError("decomposition step without operands")
            p = {"control": params.get(specs[0]), "target": params.get(specs[1])}
        elif g in ("h", "x", "y", "z", "s", "s-dag", "t", "t-dag"):
            p = {"target": params.get(specs[0])} if specs else {"target": params.get("target")}
        else:
            p = _select(params)
        return {"operation-type": g, "operation-params": p}
    return {"operation-type": step, "operation-params": _select(params)}


def decompose_operation(op: dict, supported) -> list:
    """decompose-operation (gate_decomposition.clj:50-234)."""
    g = op.get("operation-type")
    params = op.get("operation-params") or {}
    sup = supported if supported is not None else frozenset()
    if g in sup:
        return [op]
    decs = CATALOG_DECOMPOSITIONS.get(g)
    if decs is None:
        if g == "t" and "rz" in sup and "t" not in sup:
            return [{"operation-type": "rz", "operation-params": {**params, "angle": math.pi / 4}}]
        return [op]
    get = (lambda k: decs.get(k)) if isinstance(decs, dict) else (lambda k: None)
    angle = params.get("angle")  # Clojure truthiness: any number, 0.0 included, is true
    if angle is not None and get("parametric-fn"):
        steps = get("parametric-fn")(angle)
    elif get("parametric-fn") and angle is None and "rz" in sup:
        steps = get("parametric-fn")(None)
    elif angle is not None and get("universal-fn"):
        steps = get("universal-fn")(angle)
    elif supported is not None:
        steps = ((get("cnot") or get("cnot-h") or get("cnot-t") or get("cnot-s")) if "cnot" in sup else None) \
            or get("universal") or (decs if isinstance(decs, list) else None)
    else:
        steps = get("universal")
    if steps is None:
        return [op]
    return [_step_op(st, params) for st in steps]


def transform_operations(ops: list, supported, max_iterations: int = 100) -> list:
    """transform-operations (gate_decomposition.clj:236-289): replace the first
    operation needing decomposition until none is left; an operation type that does not
    decompose is left as it is."""
    sup = supported if supported is not None else frozenset()
    cur, processed = list(ops), set()
    for _ in range(max_iterations):
        idx = next((i for i, o in enumerate(cur)
                    if o.get("operation-type") not in processed and o.get("operation-type") not in sup), None)
        if idx is None:
            return cur
        op = cur[idx]
        idx = cur.index(op)
        dec = decompose_operation(op, supported)
        if dec == [op]:
            processed.add(op.get("operation-type"))
        cur = cur[:idx] + dec + cur[idx + 1:]
    raise OptimizationError("Maximum iterations reached during circuit transformation")


def transform_circuit(circuit: dict, device: dict | None = None, options: dict | None = None) -> dict:
    """transform-circuit (circuit_transformation.clj:21-74)."""
    o = options or {}
    if not o.get("transform-operations?", True):
        return {"circuit": circuit}
    d = device or {}
    supported = d.get("supported-operations")
    if supported is None:  # `or`: a nil set falls through to the native gates
        supported = d.get("native-gates")
    ops = list(circuit.get("operations") or [])
    new = transform_operations(ops, supported, o.get("max-iterations", 100)) \
        if o.get("transform-unsupported?", True) else ops
    sup = supported if supported is not None else frozenset()
    seen = []
    for x in new:
        t = x.get("operation-type")
        if t not in seen:
            seen.append(t)
    return {"circuit": {**circuit, "operations": new}, "transformed-operation-count": len(new) - len(ops),
            "unsupported-operations": [t for t in seen if t not in sup]}


# ---------------------------------------------------------------------------
# Reverse qubit mappings (domain/qubit_mapping.clj:19-200)
# ---------------------------------------------------------------------------
def compose_mappings(m1: dict | None, m2: dict | None) -> dict | None:
    """A -> B then B -> C gives A -> C; values missing from m2 pass through."""
    if m1 is None or m2 is None:
        return None
    return {k: m2.get(v, v) for k, v in m1.items()}


def invert_simple_mapping(m: dict | None) -> dict | None:
    return None if m is None else {v: k for k, v in m.items()}


def invert_vector_mapping(m: dict | None) -> dict | None:
    return None if m is None else {p: k for k, vec in m.items() for p in vec}


def create_all_reverse_mappings(ctx: dict) -> dict:
    """create-all-reverse-mappings (qubit_mapping.clj:83-147)."""
    out = dict(ctx)
    if ctx.get("qubit-mapping"):
        out["inverse-qubit-mapping"] = invert_simple_mapping(ctx["qubit-mapping"])
    l2p = ctx.get("logical-to-physical")
    if l2p:
        first = next(iter(l2p.values()))
        out["physical-to-logical"] = (invert_vector_mapping(l2p) if isinstance(first, (list, tuple))
                                      else invert_simple_mapping(l2p))
    if ctx.get("logical-to-ancillas"):
        out["ancilla-to-logical"] = invert_vector_mapping(ctx["logical-to-ancillas"])
    return out


def map_qubit_to_original(qubit: int, ctx: dict):
    """map-qubit-to-original (qubit_mapping.clj:149-182): through physical-to-logical
    (error correction or topology) and then the inverse qubit mapping; None when either
    is absent, as in the reference."""
    p2l = ctx.get("physical-to-logical")
    compacted = p2l.get(qubit) if p2l else None
    inv = ctx.get("inverse-qubit-mapping")
    if compacted is None or not inv:
        return None
    return inv.get(compacted, compacted)


def map_measurements_to_original(measurements: dict, ctx: dict) -> dict:
    """map-measurements-to-original (qubit_mapping.clj:184-202)."""
    out = {}
    for q, v in measurements.items():
        o = map_qubit_to_original(q, ctx)
        if o is not None:
            out[o] = v
    return out


def optimize(circuit: dict, device: dict | None = None, options: dict | None = None) -> dict:
    """The pipeline of hardware_optimization.clj:42-109: gate optimisation, qubit
    optimisation, error correction (`error_correction.py`, when "apply-error-correction?"),
    topology-aware routing (`topology.py`, when "optimize-topology?"), gate decomposition,
    reverse mappings and validation. The
    context threads through the stages as in the reference, including where a stage
    replaces it (routing on a device with native SWAP) and validation's lookup of the
    supported operations on the context itself (so every gate type is reported)."""
    from .error_correction import apply_error_correction
    from .topology import topology_aware_transform

    o = options or {}
    ctx: dict = {"circuit": optimize_gates(circuit, o), "device": device, "options": o}
    c, mapping = optimize_qubit_usage(ctx["circuit"], o)
    ctx.update({"circuit": c, "qubit-mapping": mapping})
    ctx = apply_error_correction(ctx)
    ctx = topology_aware_transform(ctx)
    tr = transform_circuit(ctx["circuit"], ctx.get("device"), ctx.get("options"))
    ctx = {**ctx, **tr}
    ctx = create_all_reverse_mappings(ctx)
    sup = ctx.get("supported-operations") or frozenset()
    seen = []
    for x in ctx["circuit"]["operations"]:
        if x.get("operation-type") not in seen:
            seen.append(x.get("operation-type"))
    unsupported = [t for t in seen if t not in sup]
    ctx.update({"all-gates-supported?": not unsupported, "final-unsupported-gates": unsupported,
                "pipeline-order": ["gate-cancellation", "qubit-optimization", "error-correction",
                                   "topology-optimization", "gate-decomposition", "reverse-mappings", "validation"]})
    return ctx
