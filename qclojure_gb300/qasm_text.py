"""The reference's line-based OpenQASM converters, restated.

Besides its grammar-based parser modules (restated in `qasm.py`), the reference has a
second pair of converters that read QASM line by line with regular expressions and
write it gate by gate (application/format/qasm2.clj, qasm3.clj). Their output differs
from the parser modules' (`cx q[0],q[1];` without a space in QASM 2, Braket names, a
`// Result extraction specifications` block in QASM 3), and so do their inputs:

* `qasm2_to_circuit_lines` (qasm2.clj:257-280): the register size is the first number
  of the first line that starts with `qreg`; a line adds a gate only when it starts with
  one (no leading blanks); angles are Java double literals (`pi` fails).
* `qasm3_to_circuit_lines` (qasm3.clj:466-490): lines are trimmed; the size comes from
  the first `qubit[` line; angles accept numbers, `pi`, `pi/n`, `n*pi`, `pi*n` and
  numeric fractions (parse-qasm-expression, qasm3.clj:288-340); `c[i] = measure q[j];`
  adds a measurement of qubit j; `#pragma qclojure result` lines become result specs.
"""
from __future__ import annotations

import math
import re

from .circuit import GATE_ALIASES
from .qasm import REGISTRY, clj_str

_TARGETS = {"qclojure": "qclojure", "braket": "braket"}


def _v(x) -> str:
    return "" if x is None else clj_str(x) if isinstance(x, (int, float)) else str(x)


def _name(o) -> str:
    s = str(o)
    return s[1:] if s.startswith(":") else s


def java_parse_double(s: str) -> float:
    """Double/parseDouble: surrounding blanks allowed, an optional d/D/f/F suffix."""
    t = s.strip()
    m = re.fullmatch(r"([+-]?(?:NaN|Infinity|(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?))[dDfF]?", t)
    if not m:
        raise ValueError(f"For input string: \"{s}\"")
    return float(m.group(1).replace("Infinity", "inf"))


def _add(circuit: dict, gate: str, params: dict) -> dict:
    g = GATE_ALIASES.get(gate, gate)
    if g not in REGISTRY:
        raise ValueError("Unknown gate type")
    return {**circuit, "operations": [*circuit["operations"], {"operation-type": g, "operation-params": params}]}


# ---------------------------------------------------------------------------
# QASM 2 (qasm2.clj)
# ---------------------------------------------------------------------------
def circuit_to_qasm2_lines(circuit: dict, result_specs: dict | None = None) -> str:
    """circuit-to-qasm (qasm2.clj:88-112); result specs are accepted and not written."""
    n = circuit["num-qubits"]

    def gate(op):
        g, p = op["operation-type"], op.get("operation-params") or {}
        t, c, a = _v(p.get("target")), _v(p.get("control")), _v(p.get("angle"))
        one = {"i": "id", "x": "x", "y": "y", "z": "z", "h": "h", "s": "s", "t": "t", "s-dag": "sdg", "t-dag": "tdg"}
        if g in one:
            return f"{one[g]} q[{t}];"
        if g == "phase":
            return f"p({a}) q[{t}];"
        if g in ("rx", "ry", "rz"):
            return f"{g}({a}) q[{t}];"
        if g in ("cnot", "cx"):
            return f"cx q[{c}],q[{t}];"
        if g in ("cz", "cy"):
            return f"{g} q[{c}],q[{t}];"
        if g in ("swap", "iswap"):
            return f"{g} q[{_v(p.get('qubit1'))}],q[{_v(p.get('qubit2'))}];"
        if g == "toffoli":
            return f"ccx q[{_v(p.get('control1'))}],q[{_v(p.get('control2'))}],q[{t}];"
        if g == "fredkin":
            return f"cswap q[{c}],q[{_v(p.get('target1'))}],q[{_v(p.get('target2'))}];"
        if g in ("crx", "cry", "crz"):
            return f"{g}({a}) q[{c}],q[{t}];"
        glob = {"global-x": ("Global X gate - decomposed to individual X gates", "x"),
                "global-y": ("Global Y gate - decomposed to individual Y gates", "y"),
                "global-z": ("Global Z gate - decomposed to individual Z gates", "z"),
                "global-h": ("Global Hadamard gate - decomposed to individual H gates", "h")}
        if g in glob:
            return f"// {glob[g][0]}\n" + "\n".join(f"{glob[g][1]} q[{k}];" for k in range(n))
        if g in ("global-rx", "global-ry", "global-rz"):
            r = g[-2:]
            return (f"// Global {r.upper()}({a}) gate - decomposed to individual {r.upper()} gates\n"
                    + "\n".join(f"{r}({a}) q[{k}];" for k in range(n)))
        if g == "rydberg-cz":
            return f"// Rydberg CZ gate - decomposed to standard CZ\ncz q[{c}],q[{t}];"
        if g == "rydberg-cphase":
            return f"// Rydberg controlled phase gate - decomposed to CRZ\ncrz({a}) q[{c}],q[{t}];"
        if g == "rydberg-blockade":
            return "// Rydberg blockade gate - cannot be expressed in QASM 2.0\n// Requires hardware-specific backend support"
        if g == "measure":
            return "// Measurement will be handled by final measure statement"
        return f"// Unknown gate: {g}"

    header = f'OPENQASM 2.0;\ninclude "qelib1.inc";\nqreg q[{n}];\ncreg c[{n}];\n\n'
    return header + "\n".join(gate(op) for op in circuit.get("operations") or []) + "\nmeasure q -> c;"


_Q2 = [
    (re.compile(r"^(x|y|z|h|s|t|sdg|tdg|id)\s+q\[(\d+)\]"), lambda m: (m[1], {"target": int(m[2])})),
    (re.compile(r"^c([xyz])\s+q\[(\d+)\],\s*q\[(\d+)\]"),
     lambda m: ({"x": "cnot", "z": "cz", "y": "cy"}[m[1]], {"control": int(m[2]), "target": int(m[3])})),
    (re.compile(r"^swap\s+q\[(\d+)\],\s*q\[(\d+)\]"), lambda m: ("swap", {"qubit1": int(m[1]), "qubit2": int(m[2])})),
    (re.compile(r"^iswap\s+q\[(\d+)\],\s*q\[(\d+)\]"), lambda m: ("iswap", {"qubit1": int(m[1]), "qubit2": int(m[2])})),
    (re.compile(r"^ccx\s+q\[(\d+)\],\s*q\[(\d+)\],\s*q\[(\d+)\]"),
     lambda m: ("toffoli", {"control1": int(m[1]), "control2": int(m[2]), "target": int(m[3])})),
    (re.compile(r"^cswap\s+q\[(\d+)\],\s*q\[(\d+)\],\s*q\[(\d+)\]"),
     lambda m: ("fredkin", {"control": int(m[1]), "target1": int(m[2]), "target2": int(m[3])})),
]


def qasm2_to_circuit_lines(qasm: str) -> dict:
    """qasm-to-circuit (qasm2.clj:257-280)."""
    lines = qasm.splitlines()
    qreg = next((ln for ln in lines if ln.startswith("qreg")), None)
    if qreg is None or not re.search(r"\d+", qreg):
        raise ValueError("no qreg declaration")
    c = {"num-qubits": int(re.search(r"\d+", qreg).group()), "operations": [], "name": "Converted Circuit"}
    return _lines(c, lines, qasm3=False)


def _lines(c: dict, lines, qasm3: bool) -> dict:
    angle = parse_qasm_expression if qasm3 else java_parse_double
    for raw in lines:
        line = raw.strip() if qasm3 else raw
        for rx, mk in _Q2:
            m = rx.search(line)
            if m:
                g, p = mk(m)
                c = _add(c, g, p)
                break
        else:
            m = re.search(r"^cr([xyz])\((.+?)\)\s+q\[(\d+)\],\s*q\[(\d+)\]", line)
            if m:
                c = _add(c, "cr" + m[1], {"control": int(m[3]), "target": int(m[4]), "angle": angle(m[2])})
                continue
            m = re.search(r"^p\((.+?)\)\s+q\[(\d+)\]", line)
            if m:
                c = _add(c, "phase", {"target": int(m[2]), "angle": angle(m[1])})
                continue
            m = re.search(r"^r([xyz])\((.+?)\)\s+q\[(\d+)\]", line)
            if m:
                c = _add(c, "r" + m[1], {"target": int(m[3]), "angle": angle(m[2])})
                continue
            if qasm3:
                m = re.search(r"^c\[(\d+)\]\s*=\s*measure\s+q\[(\d+)\]", line)
                if m:
                    c = {**c, "operations": [*c["operations"], {"operation-type": "measure", "operation-params": {
                        "measurement-qubits": [int(m[2])]}}]}
    return c


# ---------------------------------------------------------------------------
# QASM 3 (qasm3.clj)
# ---------------------------------------------------------------------------
def parse_qasm_expression(expr_str: str) -> float:
    """parse-qasm-expression (qasm3.clj:288-340)."""
    e = expr_str.strip()
    if re.fullmatch(r"-?\d+(\.\d+)?", e):
        return float(e)
    if e == "pi":
        return math.pi
    if e == "-pi":
        return -math.pi
    if re.fullmatch(r"-?pi/\d+(\.\d+)?", e):
        m = re.match(r"^(-?)pi/(.+)$", e)
        d = java_parse_double(m[2])
        return -math.pi / d if m[1] == "-" else math.pi / d
    if re.fullmatch(r"-?\d+(\.\d+)?\*pi", e):
        return java_parse_double(re.match(r"^(.+)\*pi$", e)[1]) * math.pi
    if re.fullmatch(r"-?pi\*\d+(\.\d+)?", e):
        m = re.match(r"^pi\*(.+)$", e)
        if m is None:  # "-pi*n": the reference's destructuring finds no match and fails
            raise ValueError(f"Unsupported QASM expression: {e}")
        return math.pi * java_parse_double(m[1])
    if re.fullmatch(r"-?\d+(\.\d+)?/\d+(\.\d+)?", e):
        a, b = e.split("/")
        return float(a) / float(b)
    try:
        return java_parse_double(e)
    except ValueError:
        raise ValueError(f"Unsupported QASM expression: {e}. Supported: numbers, pi, pi/n, n*pi, pi*n, fractions")


def _pragma(line: str):
    if not line.startswith("#pragma qclojure result"):
        return None
    parts = re.split(r"\s+", line)
    if len(parts) < 4 or not parts[3]:
        return None
    params = {}
    for pair in parts[4:]:
        k, eq, v = pair.partition("=")
        if not eq:
            params[k] = None
        elif re.fullmatch(r"\d+", v):
            params[k] = int(v)
        elif "," in v:
            params[k] = [x.strip() for x in v.split(",")]
        else:
            params[k] = v
    return parts[3], params


def collect_result_specs(lines) -> dict:
    """collect-result-specs-from-qasm (qasm3.clj:342-367)."""
    specs: dict = {}
    for ln in lines:
        if not ln.strip().startswith("#pragma qclojure result"):
            continue
        p = _pragma(ln)
        if p is None:
            continue
        kind, params = p
        if kind in specs and kind in ("expectation", "variance", "sample"):
            ex = dict(specs[kind])
            ex["observables"] = list(ex.get("observables") or []) + [params.get("observable")]
            ex["targets"] = list(ex.get("targets") or []) + [params.get("target")]
            specs[kind] = ex
        else:
            specs[kind] = params
    return specs


def emit_qasm3_pragmas(options: dict | None) -> str:
    """emit-qasm-pragmas (qasm3.clj:44-119)."""
    o = options or {}
    specs = o.get("result-specs")
    tgt = _TARGETS.get(o.get("target", "qclojure"), "qclojure")
    if not specs:
        return ""
    out = []
    for kind, spec in specs.items():
        spec = spec or {}
        head = f"#pragma {tgt} result"
        if kind == "measurements":
            s = f"{head} measurement shots={_v(spec.get('shots', 1000))}"
            if spec.get("qubits") is not None:
                s += " qubits=" + ",".join(_v(q) for q in spec["qubits"])
            out.append(s)
        elif kind in ("expectation", "variance"):
            tg = spec.get("targets", [])
            for i, ob in enumerate(spec.get("observables", [])):
                out.append(f"{head} {kind} observable={_name(ob)}" + (f" target={_v(tg[i])}" if i < len(tg) else ""))
        elif kind == "probability":
            s = f"{head} probability"
            if spec.get("targets") is not None:
                s += " targets=" + ",".join(_v(t) for t in spec["targets"])
            if spec.get("states") is not None:
                s += " states=" + ",".join(_v(t) for t in spec["states"])
            out.append(s)
        elif kind == "amplitude":
            out.append(f"{head} amplitude states=" + ",".join(_v(t) for t in spec.get("states", [])))
        elif kind == "sample":
            tg = spec.get("targets", [])
            for i, ob in enumerate(spec.get("observables", [])):
                out.append(f"{head} sample observable={_name(ob)} shots={_v(spec.get('shots', 1000))}"
                           + (f" target={_v(tg[i])}" if i < len(tg) else ""))
        elif kind in ("state-vector", "density-matrix", "fidelity"):
            out.append(f"{head} {kind.replace('-', '_')} // Simulation-only result")
        else:
            out.append(f"// Unknown result type: {kind}")
    return "\n// Result extraction specifications\n" + "\n".join(out) + "\n" if out else ""


def circuit_to_qasm3_lines(circuit: dict, options: dict | None = None) -> str:
    """circuit-to-qasm (qasm3.clj:221-262); options: "result-specs", "target" ("braket")."""
    o = options or {}
    braket = o.get("target") == "braket"
    n = circuit["num-qubits"]

    def gate(op):
        g, p = op["operation-type"], op.get("operation-params") or {}
        t, c, a = _v(p.get("target")), _v(p.get("control")), _v(p.get("angle"))
        simple = {"i": "id", "x": "x", "y": "y", "z": "z", "h": "h", "s": "s", "t": "t"}
        if g in simple:
            return f"{simple[g]} q[{t}];"
        if g == "s-dag":
            return f"{'si' if braket else 'sdg'} q[{t}];"
        if g == "t-dag":
            return f"{'ti' if braket else 'tdg'} q[{t}];"
        if g in ("rx", "ry", "rz"):
            return f"{g}({a}) q[{t}];"
        if g == "phase":
            return f"{'phaseshift' if braket else 'p'}({a}) q[{t}];"
        if g == "cnot":
            return f"{'cnot' if braket else 'cx'} q[{c}], q[{t}];"
        if g in ("cx", "cz", "cy"):
            return f"{g} q[{c}], q[{t}];"
        if g in ("crx", "cry", "crz"):
            return f"{g}({a}) q[{c}], q[{t}];"
        if g == "controlled":
            return f"ctrl @ {_v(p.get('gate'))} q[{c}], q[{t}];"
        if g in ("swap", "iswap"):
            return f"{g} q[{_v(p.get('qubit1'))}], q[{_v(p.get('qubit2'))}];"
        if g == "toffoli":
            return f"{'ccnot' if braket else 'ccx'} q[{_v(p.get('control1'))}], q[{_v(p.get('control2'))}], q[{t}];"
        if g == "fredkin":
            return f"cswap q[{c}], q[{_v(p.get('target1'))}], q[{_v(p.get('target2'))}];"
        glob = {"global-x": ("Global X gate - apply X to all qubits", "x"),
                "global-y": ("Global Y gate - apply Y to all qubits", "y"),
                "global-z": ("Global Z gate - apply Z to all qubits", "z"),
                "global-h": ("Global Hadamard gate - apply H to all qubits", "h")}
        if g in glob:
            return f"// {glob[g][0]}\n" + "\n".join(f"{glob[g][1]} q[{k}];" for k in range(n))
        if g in ("global-rx", "global-ry", "global-rz"):
            r = g[-2:]
            return (f"// Global {r.upper()}({a}) gate - apply {r.upper()} to all qubits\n"
                    + "\n".join(f"{r}({a}) q[{k}];" for k in range(n)))
        if g == "rydberg-cz":
            return f"// Rydberg CZ gate - decomposed to standard CZ\ncz q[{c}], q[{t}];"
        if g == "rydberg-cphase":
            return f"// Rydberg controlled phase gate - decomposed to CRZ\ncrz({a}) q[{c}], q[{t}];"
        if g == "rydberg-blockade":
            return ("// Rydberg blockade gate - hardware specific\n// Cannot be directly expressed in standard QASM\n"
                    "// Requires hardware-specific backend support")
        if g == "measure":
            qs = p.get("measurement-qubits") or []
            return "\n".join(f"c[{_v(q)}] = measure q[{_v(q)}];" for q in qs)
        return f"// Unknown gate: {g}"

    header = "OPENQASM 3.0;\n" + ("" if braket else 'include "stdgates.inc";\n\n') + f"qubit[{n}] q;\nbit[{n}] c;\n"
    return header + emit_qasm3_pragmas(o) + "\n" + "\n".join(gate(op) for op in circuit.get("operations") or [])


def qasm3_to_circuit_lines(qasm: str) -> dict:
    """qasm-to-circuit (qasm3.clj:466-490): the circuit map with "result-specs"."""
    lines = qasm.splitlines()
    decl = next((ln for ln in lines if ln.strip().startswith("qubit[")), None)
    if decl is None:
        raise ValueError("no qubit declaration")
    c = {"num-qubits": int(re.search(r"\d+", decl).group()), "operations": [], "name": "Converted Circuit"}
    c = _lines(c, lines, qasm3=True)
    return {**c, "result-specs": collect_result_specs(lines)}
