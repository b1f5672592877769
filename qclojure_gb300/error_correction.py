"""Stabilizer error-correction codes and the optimisation pipeline's error-correction stage.

Restates domain/error_correction.clj:
  * Pauli-string helpers (domain/observables.clj:42-109) and syndrome helpers
    (error_correction.clj:53-77);
  * `build_syndrome_table` (error_correction.clj:80-112): every single-qubit X/Y/Z error
    keyed by the syndrome it leaves (one bit per generator: 1 where the error and the
    generator anticommute). Where two errors leave one syndrome the later one (qubit
    order, then X, Y, Z) wins, as `into {}` keeps the last entry;
  * the five codes (error_correction.clj:115-216) with their generator strings as
    written there, the Shor code's eight-character logical Z included;
  * the circuit builders of the bit-flip, five-qubit, Steane and Shor codes
    (error_correction.clj:255-1000): encoding, syndrome measurement, correction from a
    syndrome, decoding;
  * `apply_error_correction` (error_correction.clj:1155-1245): encode every logical qubit
    into a block of physical qubits, translate the circuit's operations onto the blocks,
    and append each block's syndrome measurement on its own ancillas;
  * the result analysis (error_correction.clj:1615-1860): ancilla bits per logical qubit,
    syndrome decoding and the classical bit-flip correction of measurement data.

The builders add gates to the circuit maps of `circuit.py`; the state they act on is the
GPU state vector (or the oracle in tests), so an encoded circuit runs, and its syndrome
measurements collapse, like any other circuit. The gate sequences are data here (one
table per builder) and produce the reference's operation lists gate for gate.
"""
from __future__ import annotations

from . import circuit as C
from .clj import hash_long, map_order
from .optimization import OptimizationError


class ErrorCorrectionError(OptimizationError):
    """Raised where error_correction.clj throws ex-info (an unknown code or syndrome)."""


def _truthy(v) -> bool:
    """Clojure truthiness: everything but nil and false."""
    return v is not None and v is not False


# ---------------------------------------------------------------------------
# Pauli strings and syndromes
# ---------------------------------------------------------------------------
def pauli_string_p(s) -> bool:
    """pauli-string? (observables.clj:42-59)."""
    return isinstance(s, str) and all(c in "IXYZ" for c in s)


def pauli_weight(p: str) -> int:
    """pauli-weight (observables.clj:61-78)."""
    if not pauli_string_p(p):
        raise ValueError("not a Pauli string")
    return sum(c != "I" for c in p)


def pauli_commute(p1: str, p2: str) -> bool:
    """pauli-commute? (observables.clj:80-109): two Pauli strings commute when the positions
    where both are non-identity and differ are even in number."""
    if not (pauli_string_p(p1) and pauli_string_p(p2) and len(p1) == len(p2)):
        raise ValueError("Pauli strings of equal length expected")
    return sum(a != "I" and b != "I" and a != b for a, b in zip(p1, p2)) % 2 == 0


def _check_syndrome(s) -> None:
    if not isinstance(s, (list, tuple)) or any(b not in (0, 1) or isinstance(b, bool) for b in s):
        raise ValueError("syndrome must be a vector of 0 and 1")


def syndrome_weight(syndrome) -> int:
    """syndrome-weight (error_correction.clj:53-63)."""
    _check_syndrome(syndrome)
    return sum(1 for b in syndrome if b == 1)


def trivial_syndrome(syndrome) -> bool:
    """trivial-syndrome? (error_correction.clj:65-77)."""
    _check_syndrome(syndrome)
    return all(b == 0 for b in syndrome)


# ---------------------------------------------------------------------------
# codes (error_correction.clj:115-237)
# ---------------------------------------------------------------------------
def _code(name, n, generators, lx, lz, description):
    return {"name": name, "num-physical-qubits": n, "num-logical-qubits": 1,
            "stabilizer-generators": list(generators), "logical-operators": {"X": lx, "Z": lz},
            "distance": 3, "description": description}


BIT_FLIP_CODE = _code("Bit-flip code", 3, ["ZZI", "IZZ"], "XXX", "ZII",
                      "Three-qubit repetition code protecting against bit-flip errors")
PHASE_FLIP_CODE = _code("Phase-flip code", 3, ["XXI", "IXX"], "XII", "ZZZ",
                        "Three-qubit code protecting against phase-flip errors")
SHOR_CODE = _code("Shor code", 9,
                  ["ZZIIIIIII", "IZZIIIIII", "IIIIZZIII", "IIIIIZZII", "IIIIIIZZI", "IIIIIIIZZ",
                   "XXXXXXIII", "IIIXXXXXX"],
                  "XXXXXXXXX", "ZIIIIIII",
                  "Nine-qubit code protecting against arbitrary single-qubit errors")
STEANE_CODE = _code("Steane code", 7,
                    ["IIIXXXX", "IXXIIXX", "XIXIXIX", "IIIZZZZ", "IZZIIZZ", "ZIZIZIZ"],
                    "XXXXXXX", "ZZZZZZZ", "Seven-qubit CSS code with efficient encoding")
FIVE_QUBIT_CODE = _code("Five-qubit code", 5, ["XZZXI", "IXZZX", "XIXZZ", "ZXIXZ"], "XXXXX", "ZZZZZ",
                        "Smallest perfect code correcting arbitrary single-qubit errors")

AVAILABLE_CODES = {"bit-flip": BIT_FLIP_CODE, "phase-flip": PHASE_FLIP_CODE, "shor": SHOR_CODE,
                   "steane": STEANE_CODE, "five-qubit": FIVE_QUBIT_CODE}


def get_code(code_key: str):
    """get-code (error_correction.clj:226-235): the code, or None."""
    return AVAILABLE_CODES.get(code_key)


def list_available_codes() -> list[dict]:
    """list-available-codes (error_correction.clj:237-250)."""
    return [{"key": k, "name": c["name"], "description": c["description"],
             "physical-qubits": c["num-physical-qubits"], "logical-qubits": c["num-logical-qubits"],
             "distance": c["distance"]} for k, c in AVAILABLE_CODES.items()]


def _check_code(code) -> None:
    ok = (isinstance(code, dict) and isinstance(code.get("name"), str)
          and isinstance(code.get("num-physical-qubits"), int) and code["num-physical-qubits"] > 0
          and isinstance(code.get("num-logical-qubits"), int) and code["num-logical-qubits"] > 0
          and isinstance(code.get("stabilizer-generators"), list)
          and all(pauli_string_p(g) for g in code["stabilizer-generators"]))
    if not ok:
        raise ValueError("not a stabilizer code")


def build_syndrome_table(code: dict) -> dict[tuple, str]:
    """build-syndrome-table (error_correction.clj:80-112). Keys are syndrome tuples."""
    _check_code(code)
    n = code["num-physical-qubits"]
    table: dict[tuple, str] = {}
    for i in range(n):
        for p in "XYZ":
            err = "I" * i + p + "I" * (n - i - 1)
            table[tuple(0 if pauli_commute(err, g) else 1 for g in code["stabilizer-generators"])] = err
    return table


# ---------------------------------------------------------------------------
# gate tables of the builders
#
# One entry per gate in the order the reference adds them: "h q1" is a Hadamard on the
# block's qubit 1, "cnot a0 q3" a CNOT from ancilla 0 to block qubit 3.
# ---------------------------------------------------------------------------
def _table(text: str) -> list[tuple]:
    out = []
    for item in text.split(";"):
        w = item.split()
        if w:
            out.append((w[0], *w[1:]))
    return out


ENCODE = {
    # error_correction.clj:255-274
    "bit-flip": _table("cnot q0 q1; cnot q0 q2"),
    # error_correction.clj:379-425
    "five-qubit": _table("cnot q0 q1; cnot q0 q2; cnot q0 q3; cnot q0 q4; h q1; h q2; h q3; h q4;"
                         "cnot q1 q2; cnot q2 q3; cnot q3 q4; cnot q4 q1"),
    # error_correction.clj:563-616
    "steane": _table("cnot q0 q1; cnot q0 q2; cnot q0 q3; cnot q1 q4; cnot q2 q4; cnot q3 q4;"
                     "cnot q1 q5; cnot q2 q5; cnot q0 q5; cnot q1 q6; cnot q3 q6; cnot q0 q6"),
    # error_correction.clj:771-821
    "shor": _table("cnot q0 q3; cnot q0 q6; h q0; h q3; h q6; cnot q0 q1; cnot q0 q2; cnot q3 q4;"
                   "cnot q3 q5; cnot q6 q7; cnot q6 q8"),
    # the phase-flip entry of get-encoding-function (error_correction.clj:1013-1020)
    "phase-flip": _table("h q0; cnot q0 q1; cnot q0 q2; h q0; h q1; h q2"),
}

DECODE = {
    # error_correction.clj:356-377
    "bit-flip": _table("cnot q0 q2; cnot q0 q1"),
    # error_correction.clj:525-561
    "five-qubit": _table("cnot q4 q1; cnot q3 q4; cnot q2 q3; cnot q1 q2; h q4; h q3; h q2; h q1;"
                         "cnot q0 q4; cnot q0 q3; cnot q0 q2; cnot q0 q1"),
    # error_correction.clj:731-769
    "steane": _table("cnot q0 q6; cnot q3 q6; cnot q1 q6; cnot q0 q5; cnot q2 q5; cnot q1 q5;"
                     "cnot q3 q4; cnot q2 q4; cnot q1 q4; cnot q0 q3; cnot q0 q2; cnot q0 q1"),
    # error_correction.clj:962-1000
    "shor": _table("cnot q0 q2; cnot q0 q1; cnot q3 q5; cnot q3 q4; cnot q6 q8; cnot q6 q7;"
                   "h q0; h q3; h q6; cnot q0 q6; cnot q0 q3"),
}

_SHOR_H = "; ".join(f"h q{i}" for i in range(9))
SYNDROME = {
    # error_correction.clj:276-309: Z0Z1 onto a0, Z1Z2 onto a1
    "bit-flip": _table("cnot q0 a0; cnot q1 a0; cnot q1 a1; cnot q2 a1"),
    # error_correction.clj:427-484: one Hadamard-conjugated ancilla per generator
    "five-qubit": _table("h a0; cnot a0 q0; cnot q1 a0; cnot q2 a0; cnot a0 q3; h a0;"
                         "h a1; cnot a1 q1; cnot q2 a1; cnot q3 a1; cnot a1 q4; h a1;"
                         "h a2; cnot a2 q0; cnot a2 q2; cnot q3 a2; cnot q4 a2; h a2;"
                         "h a3; cnot q0 a3; cnot a3 q1; cnot a3 q3; cnot q4 a3; h a3"),
    # error_correction.clj:618-687: X-type generators through H-conjugated ancillas, then Z-type
    "steane": _table("h a0; cnot a0 q3; cnot a0 q4; cnot a0 q5; cnot a0 q6; h a0;"
                     "h a1; cnot a1 q1; cnot a1 q2; cnot a1 q5; cnot a1 q6; h a1;"
                     "h a2; cnot a2 q0; cnot a2 q2; cnot a2 q4; cnot a2 q6; h a2;"
                     "cnot q3 a3; cnot q4 a3; cnot q5 a3; cnot q6 a3;"
                     "cnot q1 a4; cnot q2 a4; cnot q5 a4; cnot q6 a4;"
                     "cnot q0 a5; cnot q2 a5; cnot q4 a5; cnot q6 a5"),
    # error_correction.clj:823-894: ancillas a0..a5 take the three blocks' bit parities,
    # a6 and a7 the X parities of blocks 1+2 and 2+3 (all nine data qubits in the H basis)
    "shor": _table("cnot q0 a0; cnot q1 a0; cnot q1 a1; cnot q2 a1; cnot q3 a2; cnot q4 a2;"
                   "cnot q4 a3; cnot q5 a3; cnot q6 a4; cnot q7 a4; cnot q7 a5; cnot q8 a5;"
                   + _SHOR_H + ";"
                   "cnot q0 a6; cnot q1 a6; cnot q2 a6; cnot q3 a6; cnot q4 a6; cnot q5 a6;"
                   "cnot q3 a7; cnot q4 a7; cnot q5 a7; cnot q6 a7; cnot q7 a7; cnot q8 a7;"
                   + _SHOR_H),
}


def _emit(circuit: dict, table, data, ancillas=()) -> dict:
    def qubit(tok):
        return (data if tok[0] == "q" else ancillas)[int(tok[1:])]

    for gate, *args in table:
        if gate == "h":
            circuit = C.h_gate(circuit, qubit(args[0]))
        else:
            circuit = C.cnot_gate(circuit, qubit(args[0]), qubit(args[1]))
    return circuit


def _check_circuit(circuit) -> None:
    if not (isinstance(circuit, dict) and isinstance(circuit.get("num-qubits"), int)
            and circuit["num-qubits"] > 0 and isinstance(circuit.get("operations"), list)):
        raise ValueError("not a circuit")


def _encoder(key: str, size: int):
    def encode(circuit: dict, logical_qubit: int) -> dict:
        _check_circuit(circuit)
        if not (logical_qubit >= 0 and logical_qubit + size - 1 < circuit["num-qubits"]):
            raise ValueError(f"qubits {logical_qubit}..{logical_qubit + size - 1} are not in the circuit")
        return _emit(circuit, ENCODE[key], list(range(logical_qubit, logical_qubit + size)))
    encode.__name__ = f"encode_{key.replace('-', '_')}"
    return encode


def _decoder(key: str, size: int):
    def decode(circuit: dict, encoded_qubits) -> dict:
        _check_circuit(circuit)
        if len(encoded_qubits) != size:
            raise ValueError(f"{size} encoded qubits expected")
        return _emit(circuit, DECODE[key], list(encoded_qubits))
    decode.__name__ = f"decode_{key.replace('-', '_')}"
    return decode


def _syndrome(key: str, size: int, n_anc: int):
    def measure(circuit: dict, encoded_qubits, ancilla_qubits) -> dict:
        _check_circuit(circuit)
        if len(encoded_qubits) != size or len(ancilla_qubits) != n_anc:
            raise ValueError(f"{size} encoded qubits and {n_anc} ancillas expected")
        circuit = _emit(circuit, SYNDROME[key], list(encoded_qubits), list(ancilla_qubits))
        return C.measure_operation(circuit, list(ancilla_qubits))
    measure.__name__ = f"measure_{key.replace('-', '_')}_syndrome"
    return measure


encode_bit_flip, decode_bit_flip = _encoder("bit-flip", 3), _decoder("bit-flip", 3)
encode_five_qubit, decode_five_qubit = _encoder("five-qubit", 5), _decoder("five-qubit", 5)
encode_steane, decode_steane = _encoder("steane", 7), _decoder("steane", 7)
encode_shor, decode_shor = _encoder("shor", 9), _decoder("shor", 9)
measure_bit_flip_syndrome = _syndrome("bit-flip", 3, 2)
measure_five_qubit_syndrome = _syndrome("five-qubit", 5, 4)
measure_steane_syndrome = _syndrome("steane", 7, 6)
_measure_shor = _syndrome("shor", 9, 8)


def measure_shor_syndrome(circuit: dict, encoded_qubits, bit_flip_ancillas, phase_flip_ancillas) -> dict:
    """measure-shor-syndrome (error_correction.clj:823-894): one measurement of the six
    bit-flip ancillas followed by the two phase-flip ancillas."""
    if len(bit_flip_ancillas) != 6 or len(phase_flip_ancillas) != 2:
        raise ValueError("6 bit-flip and 2 phase-flip ancillas expected")
    return _measure_shor(circuit, encoded_qubits, [*bit_flip_ancillas, *phase_flip_ancillas])


# the block position a two-bit repetition-code syndrome points at (error_correction.clj:311-354)
_REPETITION = {(0, 0): None, (1, 0): 0, (1, 1): 1, (0, 1): 2}


def correct_bit_flip_error(circuit: dict, encoded_qubits, syndrome) -> dict:
    """correct-bit-flip-error (error_correction.clj:311-354): X on the qubit the syndrome
    names; an unknown syndrome raises."""
    _check_circuit(circuit)
    if len(encoded_qubits) != 3 or len(syndrome) != 2:
        raise ValueError("3 encoded qubits and a 2-bit syndrome expected")
    key = tuple(syndrome)
    if key not in _REPETITION:
        raise ErrorCorrectionError("Unknown syndrome for bit-flip code")
    pos = _REPETITION[key]
    return circuit if pos is None else C.x_gate(circuit, encoded_qubits[pos])


def correct_five_qubit_error(circuit: dict, encoded_qubits, syndrome, syndrome_table=None) -> dict:
    """correct-five-qubit-error (error_correction.clj:486-523): nothing for the trivial
    syndrome; otherwise the entry {"qubit-index", "error-type"} of the caller's table, and
    an unknown syndrome (always, without a table) raises."""
    _check_circuit(circuit)
    if len(encoded_qubits) != 5 or len(syndrome) != 4:
        raise ValueError("5 encoded qubits and a 4-bit syndrome expected")
    if all(b == 0 for b in syndrome):
        return circuit
    info = (syndrome_table or {}).get(tuple(syndrome))
    if info is None:
        raise ErrorCorrectionError("Unknown syndrome for 5-qubit code")
    target = encoded_qubits[info.get("qubit-index")]
    gate = {"x": C.x_gate, "y": C.y_gate, "z": C.z_gate}.get(info.get("error-type"))
    return circuit if gate is None else gate(circuit, target)


def correct_steane_error(circuit: dict, encoded_qubits, syndrome) -> dict:
    """correct-steane-error (error_correction.clj:689-729): the first three bits read as
    x0 + 2 x1 + 4 x2 name the qubit (minus one) for an X, the last three likewise for a Z."""
    _check_circuit(circuit)
    if len(encoded_qubits) != 7 or len(syndrome) != 6:
        raise ValueError("7 encoded qubits and a 6-bit syndrome expected")
    x0, x1, x2, z0, z1, z2 = syndrome
    xv, zv = 4 * x2 + 2 * x1 + x0, 4 * z2 + 2 * z1 + z0
    if xv > 0:
        circuit = C.x_gate(circuit, encoded_qubits[xv - 1])
    if zv > 0:
        circuit = C.z_gate(circuit, encoded_qubits[zv - 1])
    return circuit


def correct_shor_error(circuit: dict, encoded_qubits, bit_flip_syndrome, phase_flip_syndrome) -> dict:
    """correct-shor-error (error_correction.clj:896-960): an X in each block whose pair of
    bits names a qubit, then Z on the three qubits of the block the phase pair names."""
    _check_circuit(circuit)
    if len(encoded_qubits) != 9 or len(bit_flip_syndrome) != 6 or len(phase_flip_syndrome) != 2:
        raise ValueError("9 encoded qubits, 6 bit-flip and 2 phase-flip bits expected")
    q = list(encoded_qubits)
    for block in range(3):
        pos = _REPETITION.get(tuple(bit_flip_syndrome[2 * block:2 * block + 2]))
        if pos is not None:
            circuit = C.x_gate(circuit, q[3 * block + pos])
    pb = _REPETITION.get(tuple(phase_flip_syndrome))
    if pb is not None:
        for k in range(3):
            circuit = C.z_gate(circuit, q[3 * pb + k])
    return circuit


_ENCODING_FUNCTIONS = {"bit-flip": encode_bit_flip, "shor": encode_shor, "steane": encode_steane,
                       "five-qubit": encode_five_qubit}


def get_encoding_function(code_key: str):
    """get-encoding-function (error_correction.clj:1002-1025)."""
    if code_key in _ENCODING_FUNCTIONS:
        return _ENCODING_FUNCTIONS[code_key]
    if code_key == "phase-flip":
        def encode_phase_flip(circuit, q):
            return _emit(circuit, ENCODE["phase-flip"], [q, q + 1, q + 2])
        return encode_phase_flip
    raise ErrorCorrectionError("No encoding function for code")


# ---------------------------------------------------------------------------
# the pipeline stage
# ---------------------------------------------------------------------------
_SINGLE = frozenset({"x", "y", "z", "h", "s", "t", "sdg", "tdg"})


def translate_operation_to_physical(op: dict, logical_to_physical: dict) -> list[dict]:
    """translate-operation-to-physical (error_correction.clj:1027-1096), with its gaps kept:
    a one-qubit gate of the set {x y z h s t sdg tdg} goes to every qubit of its block;
    a "cnot", "cz" or "swap" with control and target becomes one gate per pair of block
    qubits (a "swap", whose qubits are qubit1/qubit2, passes unchanged); a "toffoli" or
    "ccnot" with "controls" goes to each target block qubit with its controls kept; a
    measurement covers every block qubit of the qubits it names; every other operation
    (rotations, s-dag, t-dag, ...) passes unchanged, on its logical indices."""
    t = op.get("operation-type")
    p = op.get("operation-params") or {}

    def with_params(**kv):
        return {**op, "operation-params": {**p, **{k.replace("_", "-"): v for k, v in kv.items()}}}

    if t in _SINGLE:
        block = logical_to_physical.get(p.get("target"))
        return [with_params(target=q) for q in block] if block else [op]
    if t in ("cnot", "cz", "swap"):
        cb, tb = logical_to_physical.get(p.get("control")), logical_to_physical.get(p.get("target"))
        if cb and tb:
            return [with_params(control=c, target=x) for c in cb for x in tb]
        return [op]
    if t in ("ccnot", "toffoli"):
        tb = logical_to_physical.get(p.get("target"))
        if _truthy(p.get("controls")) and tb:
            return [with_params(target=x) for x in tb]
        return [op]
    if t == "measure":
        qubits = p.get("measurement-qubits")
        if qubits is None:
            qubits = p.get("qubits")
        if isinstance(qubits, (list, tuple)):
            phys = [x for q in qubits for x in logical_to_physical.get(q, [q])]
            return [with_params(measurement_qubits=phys)]
        block = logical_to_physical.get(p.get("target"))
        if block:
            return [{**op, "operation-params": {"measurement-qubits": list(block)}}]
        return [op]
    return [op]


def clj_map_key_order(keys: list[int]) -> list[int]:
    """The order in which a Clojure map built by `into {}` from these integer keys yields
    them (insertion order up to 8 entries, else the hash trie's order)."""
    return map_order(keys, hash_long)


def inject_syndrome_measurements(circuit: dict, code_key: str, logical_to_physical: dict,
                                 logical_to_ancillas: dict) -> dict:
    """inject-syndrome-measurements (error_correction.clj:1098-1153): each logical qubit's
    syndrome measurement, in the order the reference's map yields the logical qubits. The
    phase-flip code has no syndrome builder and raises."""
    _check_circuit(circuit)
    if not isinstance(logical_to_physical, dict) or not isinstance(logical_to_ancillas, dict):
        raise ValueError("qubit maps expected")
    for lq in clj_map_key_order(list(logical_to_physical)):
        phys, anc = logical_to_physical.get(lq), logical_to_ancillas.get(lq)
        if code_key == "bit-flip":
            circuit = measure_bit_flip_syndrome(circuit, phys, anc)
        elif code_key == "shor":
            circuit = measure_shor_syndrome(circuit, phys, anc[0:6], anc[6:8])
        elif code_key == "steane":
            circuit = measure_steane_syndrome(circuit, phys, anc)
        elif code_key == "five-qubit":
            circuit = measure_five_qubit_syndrome(circuit, phys, anc)
        else:
            raise ErrorCorrectionError("Unsupported error correction code for syndrome measurement")
    return circuit


ANCILLAS_PER_LOGICAL = {"bit-flip": 2, "shor": 8, "steane": 6, "five-qubit": 4}


def apply_error_correction(ctx: dict) -> dict:
    """apply-error-correction (error_correction.clj:1155-1245): with the option
    "apply-error-correction?" set, logical qubit i becomes physical qubits
    [i*b, (i+1)*b) of a b-qubit code, its ancillas follow all blocks, the encoders run
    first, then the translated operations, then the syndrome measurements. The context
    gains the code, both qubit maps, the syndrome table and two flags; without the option
    it is returned unchanged."""
    options = ctx.get("options") or {}
    if not _truthy(options.get("apply-error-correction?", False)):
        return ctx
    key = options.get("error-correction-code", "bit-flip")
    code = get_code(key)
    if code is None:
        raise ErrorCorrectionError("Unknown error correction code")
    original = ctx["circuit"]
    n_logical = original["num-qubits"]
    per = code["num-physical-qubits"]
    n_physical = n_logical * per
    with_syndrome = options.get("include-syndrome-measurement?", True)
    anc_per = ANCILLAS_PER_LOGICAL.get(key, 0) if _truthy(with_syndrome) else 0
    l2p = {q: list(range(q * per, (q + 1) * per)) for q in range(n_logical)}
    l2a = ({q: list(range(n_physical + q * anc_per, n_physical + (q + 1) * anc_per)) for q in range(n_logical)}
           if _truthy(with_syndrome) else None)
    encode = get_encoding_function(key)
    physical = C.create_circuit(n_physical + n_logical * anc_per)
    for q in range(n_logical):
        physical = encode(physical, q * per)
    translated = [x for op in original["operations"] for x in translate_operation_to_physical(op, l2p)]
    physical = {**physical, "operations": [*physical["operations"], *translated]}
    if _truthy(with_syndrome):
        physical = inject_syndrome_measurements(physical, key, l2p, l2a)
    return {**ctx, "circuit": physical, "error-correction-code": code, "logical-to-physical": l2p,
            "logical-to-ancillas": l2a, "syndrome-table": build_syndrome_table(code),
            "error-correction-applied?": True, "syndrome-measurement-included?": with_syndrome}


# ---------------------------------------------------------------------------
# results (error_correction.clj:1615-1860)
# ---------------------------------------------------------------------------
def extract_syndrome_bits(results: dict, ctx: dict):
    """extract-syndrome-bits (error_correction.clj:1615-1653): the ancilla bits of each
    logical qubit from the result's "measurements" map (a missing qubit reads 0), keyed by
    the original qubit through the inverse qubit mapping; None without measurements or
    ancillas."""
    if not isinstance(results, dict) or not isinstance(ctx, dict):
        raise ValueError("maps expected")
    l2a, inv, meas = ctx.get("logical-to-ancillas"), ctx.get("inverse-qubit-mapping"), results.get("measurements")
    if not (_truthy(meas) and _truthy(l2a)):
        return None
    inv = inv or {}
    return {inv.get(lq, lq): [meas.get(a, 0) for a in anc] for lq, anc in l2a.items()}


def decode_syndrome_bits(syndrome_bits, code_key: str, syndrome_table) -> dict:
    """decode-syndrome-bits (error_correction.clj:1655-1691)."""
    if not isinstance(syndrome_bits, (list, tuple)) or not isinstance(code_key, str):
        raise ValueError("syndrome vector and code key expected")
    pattern = (syndrome_table or {}).get(tuple(syndrome_bits))
    clean = all(b == 0 for b in syndrome_bits)
    return {"syndrome": list(syndrome_bits), "error-detected?": not clean,
            "error-location": pattern if pattern is not None else "I...",
            "error-type": "none" if clean else {"bit-flip": "x", "shor": "both"}.get(code_key, "unknown"),
            "correction-needed?": not clean}


def apply_classical_correction(measurements: dict, syndrome_info: dict, ctx: dict, code_key: str) -> dict:
    """apply-classical-correction (error_correction.clj:1693-1772): for the bit-flip code,
    flip the measured bit of the block qubit the syndrome names (a missing or non-1 value
    becomes 1); for the Shor code, record that a correction is needed."""
    corrected = dict(measurements)
    applied = []
    l2p, qmap = ctx.get("logical-to-physical") or {}, ctx.get("qubit-mapping") or {}
    for original, dec in syndrome_info.items():
        if not _truthy(dec.get("correction-needed?")):
            continue
        block = l2p.get(qmap.get(original, original))
        syn = tuple(dec.get("syndrome") or ())
        if code_key == "bit-flip":
            pos = _REPETITION.get(syn)
            if pos is not None:
                q = block[pos]
                corrected[q] = 0 if corrected.get(q) == 1 else 1
                applied.append({"logical-qubit": original, "physical-qubit": q, "correction": "x"})
        elif code_key == "shor":
            applied.append({"logical-qubit": original, "syndrome": list(syn), "correction": "complex-shor-correction",
                            "note": "Shor correction requires full syndrome analysis"})
    return {"original-measurements": measurements, "corrected-measurements": corrected,
            "corrections-applied": applied, "syndrome-info": syndrome_info}


def analyze_error_correction_results(results: dict, ctx: dict) -> dict:
    """analyze-error-correction-results (error_correction.clj:1774-1861). The error rate is
    a float where the reference keeps a ratio."""
    if not (isinstance(results, dict) and isinstance(ctx, dict) and _truthy(ctx.get("logical-to-ancillas"))
            and _truthy(ctx.get("inverse-qubit-mapping"))):
        raise ValueError("an error-corrected context with reverse mappings expected")
    key = (ctx.get("options") or {}).get("error-correction-code")
    bits = extract_syndrome_bits(results, ctx)
    decoded = ({o: decode_syndrome_bits(b, key, ctx.get("syndrome-table")) for o, b in bits.items()}
               if bits is not None else None)
    detected = None
    if decoded is not None:
        detected = next((True for d in decoded.values() if d["error-detected?"]), None)
    corr = apply_classical_correction(results.get("measurements"), decoded, ctx, key) if decoded is not None else None
    n_logical = len(ctx.get("qubit-mapping") or {})
    n_err = sum(1 for d in decoded.values() if d["error-detected?"]) if decoded is not None else None
    rate = n_err / n_logical if n_err is not None and n_logical > 0 else None
    return {"raw-results": results, "syndrome-bits": bits, "decoded-syndromes": decoded,
            "error-detected?": detected,
            "corrected-measurements": corr["corrected-measurements"] if corr else None,
            "corrections-applied": corr["corrections-applied"] if corr else None,
            "error-rate": rate, "num-logical-qubits": n_logical, "num-errors": n_err}
