"""OpenQASM 2.0 / 3.0 ingestion and emission, the reference's parser modules restated.

The reference parses QASM with Instaparse grammars (resources/openqasm/qasm2.ebnf,
qasm3.ebnf) and turns the statements it understands into circuit operations
(application/format/qasm2_parser.clj, qasm3_parser.clj). This module follows what
those modules produce:

* QASM 2 (`qasm2_to_circuit`, `circuit_to_qasm2`): the register size is the first
  qreg's; gate calls become operations through the gate aliases; measure, reset,
  barrier, creg, conditional and gate-definition statements add nothing. A gate
  parameter is the first numeric literal of its expression (extract-number-from-expression,
  qasm2_parser.clj:190-202), so `rx(1.5708)` gives 1.5708, while `rx(pi/2)` gives 2.
  `evaluate_expressions=True` evaluates them instead.
* QASM 3 (`qasm3_to_circuit`, `circuit_to_qasm3`): `qubit[n] q;` declares the register;
  gate parameters are evaluated as OpenQASM 3 constant expressions (evaluate-expression,
  qasm3_parser.clj:341-512: operators, pi/tau/euler, the built-in functions); qubit
  indices are the first integer literal of the index.
* Result pragmas (`// #pragma qclojure result ...` in QASM 2, `#pragma qclojure result ...`
  in QASM 3) become result specs; QASM 2 emission writes them back. QASM 3 emission
  passes the specs one level too deep (qasm3_parser.clj:844-846) and so writes none.

Both parsers accept the statement forms their grammars accept for programs of gate
calls and declarations; constructs outside that (gate modifiers, classical control
flow bodies in QASM 2) are refused with "Parse error".
"""
from __future__ import annotations

import math
import re
from typing import Any

from .circuit import GATE_ALIASES

# operation_registry.clj:53-370: id -> (operation-name, operation-type)
REGISTRY = {
    "x": ("X", "single-qubit"), "y": ("Y", "single-qubit"), "z": ("Z", "single-qubit"),
    "i": ("I", "single-qubit"), "h": ("H", "single-qubit"), "s": ("S", "single-qubit"),
    "s-dag": ("S†", "single-qubit"), "t": ("T", "single-qubit"), "t-dag": ("T†", "single-qubit"),
    "rx": ("RX", "parametric"), "ry": ("RY", "parametric"), "rz": ("RZ", "parametric"),
    "phase": ("Phase", "parametric"), "cnot": ("CNOT", "two-qubit"), "cz": ("CZ", "two-qubit"),
    "cy": ("CY", "two-qubit"), "swap": ("SWAP", "two-qubit"), "iswap": ("iSWAP", "two-qubit"),
    "crx": ("CRX", "parametric"), "cry": ("CRY", "parametric"), "crz": ("CRZ", "parametric"),
    "toffoli": ("Toffoli", "multi-qubit"), "fredkin": ("Fredkin", "multi-qubit"),
    "rydberg-cz": ("Rydberg CZ", "two-qubit"), "rydberg-cphase": ("Rydberg CPhase", "parametric"),
    "rydberg-blockade": ("Rydberg Blockade", "multi-qubit"),
    "global-rx": ("Global RX", "global-parametric"), "global-ry": ("Global RY", "global-parametric"),
    "global-rz": ("Global RZ", "global-parametric"), "global-h": ("Global H", "global"),
    "global-x": ("Global X", "global"), "global-y": ("Global Y", "global"), "global-z": ("Global Z", "global"),
    "measure": ("Measure", "single-qubit"),
}


def _canonical(name: str) -> str | None:
    g = GATE_ALIASES.get(name, name)
    return g if g in REGISTRY else None


def clj_str(x) -> str:
    """Clojure's str of a number: longs as digits, doubles as Java's Double.toString."""
    if isinstance(x, bool):
        return "true" if x else "false"
    if isinstance(x, int):
        return str(x)
    if isinstance(x, float):
        if math.isnan(x):
            return "NaN"
        if math.isinf(x):
            return "Infinity" if x > 0 else "-Infinity"
        if x == 0.0:
            return "-0.0" if math.copysign(1.0, x) < 0 else "0.0"
        a = abs(x)
        if 1e-3 <= a < 1e7:
            r = repr(x)
            return r if ("." in r or "e" in r) else r + ".0"
        digits = repr(x)  # shortest round-trip digits
        m = re.match(r"(-?)(\d+)(?:\.(\d+))?(?:e([+-]\d+))?$", digits)
        sign, ip, fp, ex = m.group(1), m.group(2), m.group(3) or "", int(m.group(4) or 0)
        ds = (ip + fp).lstrip("0")
        e10 = ex + len(ip) - 1 - (len(ip + fp) - len((ip + fp).lstrip("0")))
        ds = ds.rstrip("0") or "0"
        return f"{sign}{ds[0]}.{ds[1:] or '0'}E{e10}"
    return str(x)


# ---------------------------------------------------------------------------
# pragmas (qasm2_parser.clj:35-95, :97-175; qasm3_parser.clj:19-154)
# ---------------------------------------------------------------------------
def _pragma_value(v: str):
    if re.fullmatch(r"\d+", v):
        return int(v)
    if "," in v:
        return [int(p) if re.fullmatch(r"\d+", p) else p.strip() for p in v.split(",")]
    return v


def _parse_pragma(line: str, prefixes: tuple[str, ...]):
    if not any(line.startswith(p) for p in prefixes):
        return None
    clean = re.sub(r"^// ", "", line, count=1)
    parts = re.split(r"\s+", clean)
    if len(parts) < 4 or not parts[3]:
        return None
    params = {}
    for pair in parts[4:]:
        k, _, v = pair.partition("=")
        params[k] = _pragma_value(v) if _ else None
    return parts[3], params


def _collect_specs(code: str, qasm3: bool) -> dict:
    prefixes = ("#pragma qclojure result",) if qasm3 else ("// #pragma qclojure result", "#pragma qclojure result")
    specs: dict[str, Any] = {}
    for line in code.splitlines():
        t = line.strip()
        if not any(t.startswith(p) for p in prefixes):
            continue
        parsed = _parse_pragma(line, prefixes)
        if parsed is None:
            continue
        kind, params = parsed
        if kind not in specs:
            specs[kind] = params
        elif kind in ("expectation", "variance", "sample"):
            ex = dict(specs[kind])
            ex["observables"] = list(ex.get("observables") or []) + [params.get("observable")]
            ex["targets"] = list(ex.get("targets") or []) + [params.get("target")]
            specs[kind] = ex
        elif not qasm3 and kind == "measurement":
            ex = dict(specs[kind])
            ex["qubits"] = list(ex.get("qubits") or []) + list(params.get("qubits") or [])
            specs[kind] = ex
        elif not qasm3 and kind in ("probability", "amplitude"):
            ex = dict(specs[kind])
            ex["states"] = list(ex.get("states") or []) + list(params.get("states") or [])
            specs[kind] = ex
        else:
            specs[kind] = params
    return specs


def result_specs_to_qasm2_pragmas(specs: dict | None) -> str:
    if not specs:
        return ""
    out = []

    def obs_targets(spec):
        obs = spec["observables"] if spec.get("observables") else [spec.get("observable")]
        tg = spec["targets"] if spec.get("targets") else [spec.get("target")]
        return obs, tg

    for kind, spec in specs.items():
        spec = spec or {}
        if kind == "measurement":
            out.append(f"// #pragma qclojure result measurement shots={clj_str(spec.get('shots', 1000))} "
                       f"qubits={','.join(clj_str(q) for q in (spec.get('qubits') or []))}")
        elif kind in ("expectation", "variance"):
            obs, tg = obs_targets(spec)
            for i, o in enumerate(obs):
                out.append(f"// #pragma qclojure result {kind} observable={_name(o)}"
                           + (f" target={_s(tg[i])}" if i < len(tg) else ""))
        elif kind == "probability":
            s = "// #pragma qclojure result probability"
            if spec.get("targets"):
                s += " targets=" + ",".join(_s(t) for t in spec["targets"])
            if spec.get("states"):
                s += " states=" + ",".join(_s(t) for t in spec["states"])
            out.append(s)
        elif kind == "amplitude":
            out.append("// #pragma qclojure result amplitude states="
                       + ",".join(_s(t) for t in (spec.get("states") or [])))
        elif kind == "sample":
            obs, tg = obs_targets(spec)
            for i, o in enumerate(obs):
                out.append(f"// #pragma qclojure result sample observable={_name(o)} "
                           f"shots={clj_str(spec.get('shots', 1000))}"
                           + (f" target={_s(tg[i])}" if i < len(tg) else ""))
        elif kind in ("state-vector", "density-matrix", "fidelity"):
            out.append(f"// Simulation-only result: {kind}")
        else:
            out.append(f"// Unknown result type: {kind}")
    return "\n" + "\n".join(out) + "\n" if out else ""


def _name(o) -> str:
    s = str(o)
    return s[1:] if s.startswith(":") else s


def _s(v) -> str:
    return "" if v is None else clj_str(v) if isinstance(v, (int, float)) else str(v)


# ---------------------------------------------------------------------------
# lexing
# ---------------------------------------------------------------------------
def _strip_comments(code: str) -> str:
    """preprocess-qasm: block comments, then line comments (qasm2_parser.clj:15-31)."""
    code = re.sub(r"/\*.*?\*/", "", code, flags=re.S)
    return re.sub(r"//.*?(?=\r?\n|$)", "", code)


_TOKEN = re.compile(r"""
    (?P<ws>\s+)
  | (?P<str>"[^"]*"|'[^']*')
  | (?P<num>(?:\d+\.\d*|\.\d+|\d+)(?:[eE][+-]?\d+)?)
  | (?P<hw>\$\d+)
  | (?P<id>[A-Za-z_À-￿][A-Za-z0-9_À-￿]*)
  | (?P<op>\*\*|->|==|!=|<=|>=|&&|\|\||<<|>>|[-+*/%()\[\]{};,=<>!~&|^@:.])
""", re.X)


class _Tok:
    __slots__ = ("kind", "text")

    def __init__(self, kind, text):
        self.kind, self.text = kind, text

    def __repr__(self):
        return f"{self.kind}:{self.text}"


def _lex(code: str) -> list[_Tok]:
    out, pos = [], 0
    while pos < len(code):
        m = _TOKEN.match(code, pos)
        if not m:
            raise ValueError("Parse error")
        pos = m.end()
        if m.lastgroup != "ws":
            out.append(_Tok(m.lastgroup, m.group()))
    return out


class _Stream:
    def __init__(self, toks):
        self.t, self.i = toks, 0

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else None

    def at(self, text, k=0):
        p = self.peek(k)
        return p is not None and p.text == text

    def take(self, text=None, kind=None):
        p = self.peek()
        if p is None or (text is not None and p.text != text) or (kind is not None and p.kind != kind):
            raise ValueError("Parse error")
        self.i += 1
        return p

    def done(self):
        return self.i >= len(self.t)


# ---------------------------------------------------------------------------
# expressions: a tree of (op, children) or ("num", value) / ("id", name)
# ---------------------------------------------------------------------------
_BIN = [["||"], ["&&"], ["|"], ["^"], ["&"], ["==", "!="], ["<", ">", "<=", ">="], ["<<", ">>"], ["+", "-"],
        ["*", "/", "%"]]


def _expr(s: _Stream, level=0):
    if level == len(_BIN):
        return _unary(s)
    node = _expr(s, level + 1)
    while s.peek() is not None and s.peek().text in _BIN[level]:
        op = s.take().text
        node = ("bin", op, node, _expr(s, level + 1))
    return node


def _unary(s: _Stream):
    p = s.peek()
    if p is not None and p.text in ("-", "+", "!", "~"):
        s.take()
        return ("un", p.text, _unary(s))
    return _power(s)


def _power(s: _Stream):
    base = _primary(s)
    if s.at("**"):
        s.take()
        return ("bin", "**", base, _unary(s))
    return base


def _primary(s: _Stream):
    p = s.peek()
    if p is None:
        raise ValueError("Parse error")
    if p.text == "(":
        s.take()
        e = _expr(s)
        s.take(")")
        return e
    if p.kind == "num":
        s.take()
        t = p.text
        return ("num", int(t) if re.fullmatch(r"\d+", t) else float(t))
    if p.kind == "id":
        s.take()
        if s.at("("):
            s.take()
            args = []
            if not s.at(")"):
                args.append(_expr(s))
                while s.at(","):
                    s.take()
                    args.append(_expr(s))
            s.take(")")
            return ("call", p.text, args)
        if p.text in ("true", "false"):
            return ("bool", p.text == "true")
        return ("id", p.text)
    raise ValueError("Parse error")


def _first_number(e):
    """The first numeric literal of an expression, depth first (qasm2_parser.clj:190-202)."""
    if e[0] == "num":
        return e[1]
    for c in e[1:]:
        if isinstance(c, tuple):
            v = _first_number(c)
            if v is not None:
                return v
        elif isinstance(c, list):
            for x in c:
                v = _first_number(x)
                if v is not None:
                    return v
    return None


def _first_int(e):
    """parse-simple-integer (qasm3_parser.clj:185-196): the first integer literal."""
    if e[0] == "num":
        return e[1] if isinstance(e[1], int) else None
    for c in e[1:]:
        items = c if isinstance(c, list) else [c]
        for x in items:
            if isinstance(x, tuple):
                v = _first_int(x)
                if v is not None:
                    return v
    return None


_CONSTS = {"pi": math.pi, "π": math.pi, "tau": 2.0 * math.pi, "τ": 2.0 * math.pi, "euler": math.e, "ℇ": math.e}


def _to_long(v):
    if v is None:
        return 0
    if isinstance(v, bool):
        return int(v)
    if isinstance(v, int):
        return v
    return int(math.floor(v))


def _to_double(v):
    if v is None:
        return 0.0
    return float(v)


def _to_bool(v):
    return v if isinstance(v, bool) else float(v) != 0.0


def _wrap64(v: int) -> int:
    v &= (1 << 64) - 1
    return v - (1 << 64) if v >= 1 << 63 else v


def _is_int(v):
    return isinstance(v, int) and not isinstance(v, bool)


def evaluate(e):
    """evaluate-expression (qasm3_parser.clj:341-512)."""
    k = e[0]
    if k == "num":
        return e[1]
    if k == "bool":
        return e[1]
    if k == "id":
        if e[1] in _CONSTS:
            return _CONSTS[e[1]]
        raise ValueError("Failed to evaluate OpenQASM expression: unknown identifier " + e[1])
    if k == "call":
        return _function(e[1], [evaluate(a) for a in e[2]])
    if k == "un":
        v = evaluate(e[2])
        return {"-": lambda: -_to_double(v), "+": lambda: _to_double(v), "!": lambda: not _to_bool(v),
                "~": lambda: _wrap64(~_to_long(v))}[e[1]]()
    op, a, b = e[1], evaluate(e[2]), evaluate(e[3])
    both_int = _is_int(a) and _is_int(b) or (isinstance(a, bool) or isinstance(b, bool)) and \
        not isinstance(a, float) and not isinstance(b, float)
    if op == "**":
        return math.pow(_to_double(a), _to_double(b))
    if op == "*":
        return _wrap64(_to_long(a) * _to_long(b)) if both_int else _to_double(a) * _to_double(b)
    if op == "/":
        return _to_double(a) / _to_double(b)
    if op == "%":
        if _is_int(a) and _is_int(b):
            return _to_long(a) % _to_long(b)
        ad, bd = _to_double(a), _to_double(b)
        return ad - math.floor(ad / bd) * bd
    if op in ("+", "-"):
        if both_int:
            return _wrap64(_to_long(a) + _to_long(b) if op == "+" else _to_long(a) - _to_long(b))
        return _to_double(a) + _to_double(b) if op == "+" else _to_double(a) - _to_double(b)
    if op in ("<", ">", "<=", ">="):
        x, y = _to_double(a), _to_double(b)
        return {"<": x < y, ">": x > y, "<=": x <= y, ">=": x >= y}[op]
    if op in ("==", "!="):
        return (_to_double(a) == _to_double(b)) == (op == "==")
    if op == "&":
        return _to_long(a) & _to_long(b)
    if op == "^":
        return _to_long(a) ^ _to_long(b)
    if op == "|":
        return _to_long(a) | _to_long(b)
    if op == "&&":
        return _to_bool(a) and _to_bool(b)
    if op == "||":
        return _to_bool(a) or _to_bool(b)
    raise ValueError("Failed to evaluate OpenQASM expression: operator " + op)


def _function(name: str, args: list):
    f = name.lower()
    d = lambda i=0: _to_double(args[i])  # noqa: E731
    table = {"sin": lambda: math.sin(d()), "cos": lambda: math.cos(d()), "tan": lambda: math.tan(d()),
             "arcsin": lambda: math.asin(d()), "arccos": lambda: math.acos(d()), "arctan": lambda: math.atan(d()),
             "exp": lambda: math.exp(d()), "sqrt": lambda: math.sqrt(d()), "floor": lambda: float(math.floor(d())),
             "ceiling": lambda: float(math.ceil(d())), "ceil": lambda: float(math.ceil(d())),
             "pow": lambda: math.pow(d(0), d(1)), "real": lambda: d(), "imag": lambda: 0.0}
    if f in table:
        return table[f]()
    if f == "log":
        if len(args) == 1:
            return math.log(d())
        if len(args) == 2:
            return math.log(d(0)) / math.log(d(1))
        raise ValueError("log expects 1 or 2 args")
    if f == "mod":
        a, b = args
        if _is_int(a) and _is_int(b):
            return a % b
        ad, bd = _to_double(a), _to_double(b)
        return ad - math.floor(ad / bd) * bd
    if f == "popcount":
        return bin(_to_long(args[0]) & ((1 << 64) - 1)).count("1")
    if f in ("rotl", "rotr"):
        v, n = _to_long(args[0]) & ((1 << 64) - 1), _to_long(args[1]) % 64
        r = ((v << n) | (v >> (64 - n))) if f == "rotl" else ((v >> n) | (v << (64 - n)))
        return _wrap64(r)
    raise ValueError("Unsupported or unknown function " + f)


# ---------------------------------------------------------------------------
# gate calls -> operations (parse-gate-call, qasm2_parser.clj:248-345, qasm3_parser.clj:564-674)
# ---------------------------------------------------------------------------
def _operation(name: str, params: list, qubits: list, qasm3: bool):
    g = _canonical(name)
    if g is None:
        return None  # "Unknown gate ... not found in operation registry"
    q = list(qubits)

    def need(k):
        if len(q) < k or any(x is None for x in q[:k]):
            raise IndexError
        return q[:k]

    a = params[0] if params else 0.0
    try:
        if g in ("h", "x", "y", "z", "s", "s-dag", "t", "t-dag", "i"):
            if g == "i" and qasm3:
                raise KeyError  # generic branch below
            return {"operation-type": g, "operation-params": {"target": need(1)[0]}}
        if g in ("rx", "ry", "rz", "phase"):
            return {"operation-type": g, "operation-params": {"target": need(1)[0], "angle": a}}
        if g in ("cnot", "cz", "cy"):
            c, t = need(2)
            return {"operation-type": g, "operation-params": {"control": c, "target": t}}
        if g in ("swap", "iswap"):
            c, t = need(2)
            return {"operation-type": g, "operation-params": {"qubit1": c, "qubit2": t}}
        if g in ("crx", "cry", "crz"):
            c, t = need(2)
            return {"operation-type": g, "operation-params": {"control": c, "target": t, "angle": a}}
        if g == "toffoli":
            c1, c2, t = need(3)
            return {"operation-type": g, "operation-params": {"control1": c1, "control2": c2, "target": t}}
        if g == "fredkin":
            c, t1, t2 = need(3)
            return {"operation-type": g, "operation-params": {"control": c, "target1": t1, "target2": t2}}
        if qasm3 and g == "rydberg-cz":
            c, t = need(2)
            return {"operation-type": g, "operation-params": {"control": c, "target": t}}
        if qasm3 and g == "rydberg-cphase":
            c, t = need(2)
            return {"operation-type": g, "operation-params": {"control": c, "target": t, "angle": a}}
        if qasm3 and g in ("global-h", "global-x", "global-y", "global-z"):
            return {"operation-type": g}
        if qasm3 and g in ("global-rx", "global-ry", "global-rz"):
            return {"operation-type": g, "operation-params": {"angle": a}}
    except (IndexError, KeyError):
        if g != "i":
            return None  # "Error creating gate ..."
    # generic add-gate by operand count
    keys = {1: ["target"], 2: ["control", "target"], 3: ["control1", "control2", "target"]}.get(len(q), [])
    prm = dict(zip(keys, q))
    if params and not qasm3:
        prm["angle"] = params[0]
    op = {"operation-type": g}
    if prm:
        op["operation-params"] = prm
    return op


def _id_index(s: _Stream):
    """id = Identifier designator? -> (name, index expression or None)."""
    name = s.take(kind="id").text
    idx = None
    if s.at("["):
        s.take()
        idx = _expr(s)
        s.take("]")
    return name, idx


def _skip_block(s: _Stream):
    depth = 0
    while not s.done():
        t = s.take().text
        if t == "{":
            depth += 1
        elif t == "}":
            depth -= 1
            if depth == 0:
                return
    raise ValueError("Parse error")


# ---------------------------------------------------------------------------
# QASM 2
# ---------------------------------------------------------------------------
def qasm2_to_circuit(code: str, evaluate_expressions: bool = False) -> dict:
    """qasm-to-circuit (qasm2_parser.clj:484-497): {"circuit": ..., "result-specs": ...}."""
    s = _Stream(_lex(_strip_comments(code)))
    num_qubits = None
    ops = []
    param_of = (lambda e: evaluate(e)) if evaluate_expressions else _first_number
    if s.at("OPENQASM"):
        s.take()
        s.take(kind="num")
        s.take(";")
    while not s.done():
        p = s.peek()
        t = p.text
        if t == "include":
            s.take()
            s.take(kind="str")
            s.take(";")
        elif t in ("qreg", "creg") and s.peek(1) is not None and s.peek(1).kind == "id":
            s.take()
            _, idx = _id_index(s)
            if idx is None:
                raise ValueError("Parse error")
            s.take(";")
            if t == "qreg" and num_qubits is None:
                num_qubits = _first_number(idx)
        elif t in ("gate", "opaque") and s.peek(1) is not None and s.peek(1).kind == "id":
            s.take()
            s.take(kind="id")
            s.take("(")
            while not s.at(")"):
                s.take()
            s.take(")")
            s.take("(")
            while not s.at(")"):
                s.take()
            s.take(")")
            if t == "gate":
                if not s.at("{"):
                    raise ValueError("Parse error")
                _skip_block(s)
            else:
                s.take(";")
        elif t == "measure":
            s.take()
            _id_index(s)
            s.take("->")
            _id_index(s)
            s.take(";")
        elif t == "reset":
            s.take()
            _id_index(s)
            s.take(";")
        elif t == "barrier":
            s.take()
            _id_index(s)
            while s.at(","):
                s.take()
                _id_index(s)
            s.take(";")
        elif t == "if":
            s.take()
            s.take("(")
            s.take(kind="id")
            s.take("==")
            s.take(kind="num")
            s.take(")")
            _gate_call(s, param_of, qasm3=False)  # the conditional gate adds nothing
        elif p.kind == "id":
            op = _gate_call(s, param_of, qasm3=False)
            if op is not None:
                ops.append(op)
        else:
            raise ValueError("Parse error")
    circuit = {"num-qubits": int(num_qubits or 0), "operations": ops, "name": "Parsed QASM2 Circuit"}
    return {"circuit": circuit, "result-specs": _collect_specs(code, qasm3=False)}


def _gate_call(s: _Stream, param_of, qasm3: bool):
    name = s.take(kind="id").text
    params = []
    if s.at("("):
        s.take()
        if not s.at(")"):
            params.append(param_of(_expr(s)))
            while s.at(","):
                s.take()
                params.append(param_of(_expr(s)))
        s.take(")")
    qubits = []
    if not s.at(";"):
        while True:
            if qasm3 and s.peek() is not None and s.peek().kind == "hw":
                s.take()
                qubits.append(None)
            else:
                _, idx = _id_index(s)
                qubits.append(None if idx is None else (_first_int(idx) if qasm3 else _first_number(idx)))
            if not s.at(","):
                break
            s.take()
    s.take(";")
    params = [p for p in params if p is not None]
    qubits = [q for q in qubits if q is not None]
    return _operation(name, params, qubits, qasm3)


def gate_to_qasm2(op: dict) -> str:
    """gate-to-qasm2 (qasm2_parser.clj:420-480)."""
    g = op["operation-type"]
    p = op.get("operation-params") or {}
    info = REGISTRY.get(GATE_ALIASES.get(g, g))
    if info is None:
        return f"// Unknown gate: {g}"
    qname, kind = info[0].lower(), info[1]
    v = lambda k: _s(p.get(k))  # noqa: E731
    if kind == "single-qubit":
        special = {"s-dag": "sdg", "t-dag": "tdg", "i": "id"}
        return f"{special.get(g, qname)} q[{v('target')}];"
    if kind == "parametric":
        nm = "p" if g == "phase" else qname
        return f"{nm}({v('angle')}) q[{v('target')}];"
    if kind == "two-qubit":
        if g == "cnot":
            return f"cx q[{v('control')}], q[{v('target')}];"
        if g in ("swap", "iswap"):
            return f"{g} q[{v('qubit1')}], q[{v('qubit2')}];"
        return f"{qname} q[{v('control')}], q[{v('target')}];"
    if kind == "multi-qubit":
        if g == "toffoli":
            return f"ccx q[{v('control1')}], q[{v('control2')}], q[{v('target')}];"
        if g == "fredkin":
            return f"cswap q[{v('control')}], q[{v('target1')}], q[{v('target2')}];"
        return f"// Multi-qubit gate: {g}"
    return f"// Unsupported gate type: :{kind}"


def circuit_to_qasm2(circuit: dict, result_specs: dict | None = None) -> str:
    """circuit-to-qasm (qasm2_parser.clj:499-524)."""
    n = circuit["num-qubits"]
    header = f'OPENQASM 2.0;\ninclude "qelib1.inc";\n\nqreg q[{n}];\ncreg c[{n}];\n\n'
    body = "\n".join(gate_to_qasm2(op) for op in circuit.get("operations") or [])
    pragmas = result_specs_to_qasm2_pragmas(result_specs) if result_specs else ""
    return header + body + pragmas + "\nmeasure q -> c;"


# ---------------------------------------------------------------------------
# QASM 3
# ---------------------------------------------------------------------------
_SKIP3 = {"if", "for", "while", "def", "defcal", "cal", "box", "switch", "extern", "input", "output", "const",
          "int", "uint", "float", "angle", "bool", "complex", "duration", "stretch", "let", "return", "break",
          "continue", "end", "delay", "array", "gate", "opaque", "reset", "barrier", "measure", "bit", "creg",
          "qreg", "pragma", "durationof", "gphase"}


def _skip_statement(s: _Stream):
    """Consume one statement: up to its ';' or its brace-delimited block (and an else block)."""
    depth = 0
    while not s.done():
        t = s.take().text
        if t == "{":
            depth += 1
        elif t == "}":
            depth -= 1
            if depth == 0:
                if s.at("else"):
                    s.take()
                    continue
                return
        elif t == ";" and depth == 0:
            return
    if depth:
        raise ValueError("Parse error")


def qasm3_to_circuit(code: str) -> dict:
    """qasm-to-circuit (qasm3_parser.clj:741-758): the circuit map with "result-specs"."""
    lines = []
    for ln in _strip_comments(code).splitlines():
        lines.append("" if ln.strip().startswith("#pragma") else ln)  # pragma lines carry result specs only
    s = _Stream(_lex("\n".join(lines)))
    num_qubits = None
    ops = []
    if s.at("OPENQASM"):
        s.take()
        s.take(kind="num")
        s.take(";")
    while not s.done():
        p = s.peek()
        t = p.text
        if t == "include":
            s.take()
            s.take(kind="str")
            s.take(";")
        elif t == "qubit":
            s.take()
            size = None
            if s.at("["):
                s.take()
                e = _expr(s)
                s.take("]")
                size = _first_int(e)
                if size is None:
                    size = evaluate(e)
            s.take(kind="id")
            s.take(";")
            if num_qubits is None and size is not None:
                num_qubits = size
        elif p.kind == "id" and t in _SKIP3:
            _skip_statement(s)
        elif p.kind == "id" and (s.at("=", 1) or s.at("[", 1) and _assignment_ahead(s)):
            _skip_statement(s)  # c[0] = measure q[0]; and other assignments
        elif p.kind == "id":
            op = _gate_call(s, evaluate, qasm3=True)
            if op is not None:
                ops.append(op)
        else:
            raise ValueError("Parse error")
    circuit = {"num-qubits": int(num_qubits or 0), "operations": ops, "name": "Parsed QASM3 Circuit",
               "result-specs": _collect_specs(code, qasm3=True)}
    return circuit


def _assignment_ahead(s: _Stream) -> bool:
    depth = 0
    k = 1
    while True:
        p = s.peek(k)
        if p is None:
            return False
        if p.text == "[":
            depth += 1
        elif p.text == "]":
            depth -= 1
            if depth == 0:
                nx = s.peek(k + 1)
                return nx is not None and nx.text == "="
        k += 1


def gate_to_qasm3(op: dict, options: dict | None = None) -> str:
    """gate-to-qasm3 (qasm3_parser.clj:760-824)."""
    g = op["operation-type"]
    p = op.get("operation-params") or {}
    info = REGISTRY.get(GATE_ALIASES.get(g, g))
    if info is None:
        return f"// Unknown gate: {g}"
    qname = {"phase": "p", "s-dag": "sdg", "t-dag": "tdg"}.get(g, info[0].lower())
    kind = info[1]
    v = lambda k: _s(p.get(k))  # noqa: E731
    if kind == "single-qubit":
        return f"{qname} q[{v('target')}];"
    if kind == "parametric":
        return f"{qname}({v('angle')}) q[{v('target')}];"
    if kind == "two-qubit":
        if g == "cnot":
            return f"cx q[{v('control')}], q[{v('target')}];"
        if g in ("swap", "iswap"):
            return f"{g} q[{v('qubit1')}], q[{v('qubit2')}];"
        return f"{qname} q[{v('control')}], q[{v('target')}];"
    if kind == "multi-qubit":
        if g == "toffoli":
            return f"ccx q[{v('control1')}], q[{v('control2')}], q[{v('target')}];"
        if g == "fredkin":
            return f"cswap q[{v('control')}], q[{v('target1')}], q[{v('target2')}];"
        return f"// Multi-qubit gate: {g}"
    if kind == "global":
        return f"// Global gate: {g}"
    if kind == "global-parametric":
        return f"// Global parametric gate: {g}({v('angle')})"
    return f"// Unsupported gate type: :{kind}"


def circuit_to_qasm3(circuit: dict, options: dict | None = None) -> str:
    """circuit-to-qasm (qasm3_parser.clj:826-850). Result pragmas are not written (the
    reference hands the specs, not the options, to its pragma emitter)."""
    o = options or {}
    n = circuit["num-qubits"]
    header = "OPENQASM 3.0;\n" + ("" if o.get("target") == "braket" else 'include "stdgates.inc";\n\n') + \
        f"qubit[{n}] q;\nbit[{n}] c;\n\n"
    return header + "\n".join(gate_to_qasm3(op, o) for op in circuit.get("operations") or [])
