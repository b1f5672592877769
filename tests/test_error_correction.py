"""The error-correction stage: the reference's tests restated
(test/org/soulspace/qclojure/domain/error_correction_test.clj), the encoded circuits run on
the oracle (encode -> error -> syndrome measurement -> correction -> decode), and the stage
inside the optimisation pipeline."""
import numpy as np
import pytest

from qclojure_gb300 import circuit as C
from qclojure_gb300 import error_correction as E
from qclojure_gb300.clj import hash_long
from qclojure_gb300.optimization import optimize

SIZES = {"bit-flip": (3, 2), "shor": (9, 8), "steane": (7, 6), "five-qubit": (5, 4)}


def types(c):
    return [o["operation-type"] for o in c["operations"]]


def params(c, k):
    return c["operations"][k]["operation-params"]


# ---------------------------------------------------------------------------
# error_correction_test.clj:11-62
def test_codes_and_syndromes():
    codes = E.list_available_codes()
    assert len(codes) >= 5 and all({"key", "name", "description"} <= set(c) for c in codes)
    for key, name, n in [("bit-flip", "Bit-flip code", 3), ("shor", "Shor code", 9),
                         ("steane", "Steane code", 7), ("five-qubit", "Five-qubit code", 5)]:
        code = E.get_code(key)
        assert code["name"] == name and code["num-physical-qubits"] == n and code["num-logical-qubits"] == 1
    assert E.get_code("nonexistent") is None
    assert [E.syndrome_weight(s) for s in ([0, 0, 0], [1, 0, 0], [1, 1, 0], [1, 1, 1])] == [0, 1, 2, 3]
    assert E.trivial_syndrome([0, 0, 0]) and E.trivial_syndrome([0, 0, 0, 0])
    assert not any(E.trivial_syndrome(s) for s in ([1, 0, 0], [0, 1, 0], [1, 1, 1]))
    with pytest.raises(ValueError):
        E.syndrome_weight([2, 0])


def test_pauli_helpers():
    """observables.clj:42-109 and its examples."""
    assert E.pauli_string_p("XYZII") and not E.pauli_string_p("ABC")
    assert E.pauli_weight("XYZII") == 3 and E.pauli_weight("IIIII") == 0
    assert E.pauli_commute("XII", "IXI") and not E.pauli_commute("XII", "ZII")
    assert E.pauli_commute("XYZ", "ZYX")  # two positions differ: they commute


def test_syndrome_tables():
    t = E.build_syndrome_table(E.BIT_FLIP_CODE)
    # X and Y on qubit 0 anticommute with ZZI only, Z errors with neither generator; where
    # errors share a syndrome the last one (qubit order, then X, Y, Z) is kept
    assert t == {(1, 0): "YII", (0, 0): "IIZ", (1, 1): "IYI", (0, 1): "IIY"}
    five = E.build_syndrome_table(E.FIVE_QUBIT_CODE)
    assert len(five) == 15 and (0, 0, 0, 0) not in five  # a perfect code: 15 distinct syndromes
    assert len(E.build_syndrome_table(E.STEANE_CODE)) == 21
    shor = E.build_syndrome_table(E.SHOR_CODE)
    assert len(shor) == 20 and shor[(0,) * 6 + (1, 0)] == "IIZIIIIII"


# error_correction_test.clj:67-134
def test_bit_flip_builders():
    enc = E.encode_bit_flip(C.create_circuit(3), 0)
    assert enc["num-qubits"] == 3 and types(enc) == ["cnot", "cnot"]
    assert (params(enc, 0)["control"], params(enc, 0)["target"]) == (0, 1)
    assert (params(enc, 1)["control"], params(enc, 1)["target"]) == (0, 2)
    m = E.measure_bit_flip_syndrome(C.create_circuit(5), [0, 1, 2], [3, 4])
    assert m["num-qubits"] == 5 and len(m["operations"]) == 5
    assert {p["target"] for o, p in zip(types(m), (x.get("operation-params") for x in m["operations"]))
            if o == "cnot"} == {3, 4}
    assert params(m, 4) == {"measurement-qubits": [3, 4]}
    for syn, q in [([1, 0], 0), ([1, 1], 1), ([0, 1], 2)]:
        c = E.correct_bit_flip_error(C.create_circuit(3), [0, 1, 2], syn)
        assert types(c)[-1] == "x" and params(c, -1)["target"] == q
    assert E.correct_bit_flip_error(C.create_circuit(3), [0, 1, 2], [0, 0])["operations"] == []
    with pytest.raises(E.ErrorCorrectionError):
        E.correct_bit_flip_error(C.create_circuit(3), [0, 1, 2], [2, 0])
    dec = E.decode_bit_flip(C.create_circuit(3), [0, 1, 2])
    assert types(dec) == ["cnot", "cnot"] and params(dec, 0)["target"] == 2


# error_correction_test.clj:136-180
def test_five_qubit_builders():
    enc = E.encode_five_qubit(C.create_circuit(5), 0)
    assert enc["num-qubits"] == 5 and len(enc["operations"]) == 12 and {"cnot", "h"} == set(types(enc))
    m = E.measure_five_qubit_syndrome(C.create_circuit(9), [0, 1, 2, 3, 4], [5, 6, 7, 8])
    assert m["num-qubits"] == 9 and len(m["operations"]) == 25
    assert any(o["operation-type"] == "cnot" and o["operation-params"]["target"] >= 5 for o in m["operations"])
    assert E.correct_five_qubit_error(C.create_circuit(5), [0, 1, 2, 3, 4], [0, 0, 0, 0])["operations"] == []
    with pytest.raises(E.ErrorCorrectionError):
        E.correct_five_qubit_error(C.create_circuit(5), [0, 1, 2, 3, 4], [1, 0, 0, 0])
    table = {(1, 0, 0, 0): {"qubit-index": 2, "error-type": "y"}}
    c = E.correct_five_qubit_error(C.create_circuit(5), [0, 1, 2, 3, 4], [1, 0, 0, 0], syndrome_table=table)
    assert types(c) == ["y"] and params(c, 0)["target"] == 2
    dec = E.decode_five_qubit(C.create_circuit(5), [0, 1, 2, 3, 4])
    assert len(dec["operations"]) == 12 and set(types(dec)) <= {"cnot", "h"}


# error_correction_test.clj:182-224
def test_steane_builders():
    enc = E.encode_steane(C.create_circuit(7), 0)
    assert enc["num-qubits"] == 7 and len(enc["operations"]) == 12 and set(types(enc)) == {"cnot"}
    m = E.measure_steane_syndrome(C.create_circuit(13), list(range(7)), list(range(7, 13)))
    assert m["num-qubits"] == 13 and len(m["operations"]) == 31
    assert E.correct_steane_error(C.create_circuit(7), list(range(7)), [0] * 6)["operations"] == []
    c = E.correct_steane_error(C.create_circuit(7), list(range(7)), [1, 0, 0, 0, 1, 1])
    assert types(c) == ["x", "z"] and params(c, 0)["target"] == 0 and params(c, 1)["target"] == 5
    dec = E.decode_steane(C.create_circuit(7), list(range(7)))
    assert len(dec["operations"]) == 12 and set(types(dec)) <= {"cnot", "h"}


# error_correction_test.clj:226-279
def test_shor_builders():
    enc = E.encode_shor(C.create_circuit(9), 0)
    assert enc["num-qubits"] == 9 and len(enc["operations"]) == 11 and {"h", "cnot"} == set(types(enc))
    m = E.measure_shor_syndrome(C.create_circuit(17), list(range(9)), list(range(9, 15)), [15, 16])
    assert m["num-qubits"] == 17 and len(m["operations"]) == 12 + 9 + 12 + 9 + 1
    assert params(m, -1) == {"measurement-qubits": list(range(9, 17))}
    assert E.correct_shor_error(C.create_circuit(9), list(range(9)), [0] * 6, [0, 0])["operations"] == []
    c = E.correct_shor_error(C.create_circuit(9), list(range(9)), [1, 0, 0, 0, 0, 0], [0, 0])
    assert types(c) == ["x"] and params(c, 0)["target"] == 0
    c = E.correct_shor_error(C.create_circuit(9), list(range(9)), [0, 0, 1, 1, 0, 0], [0, 1])
    assert types(c) == ["x", "z", "z", "z"] and [params(c, k)["target"] for k in range(4)] == [4, 6, 7, 8]
    dec = E.decode_shor(C.create_circuit(9), list(range(9)))
    assert len(dec["operations"]) == 11 and set(types(dec)) <= {"cnot", "h"}


def test_builder_preconditions():
    with pytest.raises(ValueError):
        E.encode_shor(C.create_circuit(8), 0)
    with pytest.raises(ValueError):
        E.measure_bit_flip_syndrome(C.create_circuit(5), [0, 1], [3, 4])
    with pytest.raises(E.ErrorCorrectionError):
        E.get_encoding_function("nope")
    pf = E.get_encoding_function("phase-flip")(C.create_circuit(3), 0)
    assert types(pf) == ["h", "cnot", "cnot", "h", "h", "h"]


# ---------------------------------------------------------------------------
# error_correction_test.clj:281-398
def test_stage_disabled_returns_context():
    c = C.create_circuit(2)
    ctx = {"circuit": c, "options": {"apply-error-correction?": False}}
    out = E.apply_error_correction(ctx)
    assert out["circuit"] is c and "error-correction-applied?" not in out and "logical-to-physical" not in out


def test_stage_bit_flip():
    c = C.cnot_gate(C.h_gate(C.create_circuit(2), 0), 0, 1)
    out = E.apply_error_correction({"circuit": c, "options": {"apply-error-correction?": True},
                                    "error-correction-code": "bit-flip"})
    assert out["error-correction-applied?"] is True and out["error-correction-code"]["name"] == "Bit-flip code"
    assert out["logical-to-physical"] == {0: [0, 1, 2], 1: [3, 4, 5]}
    assert out["logical-to-ancillas"] == {0: [6, 7], 1: [8, 9]}
    assert out["circuit"]["num-qubits"] == 10
    ops = out["circuit"]["operations"]
    # 4 encoding CNOTs, 3 Hadamards, 9 block CNOTs, 2 x (4 CNOTs + a measurement)
    assert len(ops) == 4 + 3 + 9 + 10
    assert types(out["circuit"])[4:7] == ["h"] * 3
    assert [(p["control"], p["target"]) for p in (o["operation-params"] for o in ops[7:16])] == \
        [(c_, t) for c_ in (0, 1, 2) for t in (3, 4, 5)]
    one = E.apply_error_correction({"circuit": C.h_gate(C.create_circuit(1), 0),
                                    "options": {"apply-error-correction?": True}})
    assert "h" in types(one["circuit"]) and len(one["circuit"]["operations"]) >= 3


@pytest.mark.parametrize("key,name,total", [("shor", "Shor code", 17), ("five-qubit", "Five-qubit code", 9),
                                            ("steane", "Steane code", 13)])
def test_stage_other_codes(key, name, total):
    out = E.apply_error_correction({"circuit": C.create_circuit(1),
                                    "options": {"apply-error-correction?": True, "error-correction-code": key}})
    assert out["error-correction-code"]["name"] == name and out["circuit"]["num-qubits"] == total
    assert len(out["logical-to-physical"][0]) == SIZES[key][0]


def test_stage_multi_qubit_and_measurement():
    c = C.cnot_gate(C.cnot_gate(C.h_gate(C.create_circuit(3), 0), 0, 1), 1, 2)
    out = E.apply_error_correction({"circuit": c, "options": {"apply-error-correction?": True,
                                                              "error-correction-code": "bit-flip"}})
    assert out["circuit"]["num-qubits"] == 15 and all(len(v) == 3 for v in out["logical-to-physical"].values())
    c = C.measure_all_operation(C.h_gate(C.create_circuit(2), 0))
    out = E.apply_error_correction({"circuit": c, "options": {"apply-error-correction?": True}})
    ms = [o for o in out["circuit"]["operations"] if o["operation-type"] == "measure"]
    assert ms[0]["operation-params"]["measurement-qubits"] == [0, 1, 2, 3, 4, 5]
    C.validate_circuit(out["circuit"])


def test_stage_quirks():
    """Operations outside the translated sets keep their logical indices, a SWAP (qubit1/
    qubit2) passes unchanged, the phase-flip code has no syndrome builder, and an unknown
    code raises."""
    c = C.swap_gate(C.rx_gate(C.s_dag_gate(C.create_circuit(2), 1), 1, 0.3), 0, 1)
    out = E.apply_error_correction({"circuit": c, "options": {"apply-error-correction?": True,
                                                              "include-syndrome-measurement?": False}})
    assert out["circuit"]["operations"][4:] == c["operations"] and out["logical-to-ancillas"] is None
    assert out["circuit"]["num-qubits"] == 6
    with pytest.raises(E.ErrorCorrectionError, match="Unsupported"):
        E.apply_error_correction({"circuit": c, "options": {"apply-error-correction?": True,
                                                            "error-correction-code": "phase-flip"}})
    with pytest.raises(E.ErrorCorrectionError, match="Unknown error correction code"):
        E.apply_error_correction({"circuit": c, "options": {"apply-error-correction?": True,
                                                            "error-correction-code": "nope"}})
    # Clojure truthiness: 0 switches the stage on
    assert E.apply_error_correction({"circuit": c, "options": {"apply-error-correction?": 0}})[
        "error-correction-applied?"]


def test_syndrome_order_beyond_eight_logical_qubits():
    """A map of more than eight logical qubits yields them in the Clojure hash map's order
    (for 0..9: 0 7 1 4 6 3 2 9 5 8), and the syndrome measurements follow it."""
    assert E.clj_map_key_order(list(range(10))) == [0, 7, 1, 4, 6, 3, 2, 9, 5, 8]
    assert hash_long(1) == 1392991556
    out = E.apply_error_correction({"circuit": C.create_circuit(10), "options": {"apply-error-correction?": True}})
    ms = [o["operation-params"]["measurement-qubits"] for o in out["circuit"]["operations"]
          if o["operation-type"] == "measure"]
    assert ms == [out["logical-to-ancillas"][q] for q in [0, 7, 1, 4, 6, 3, 2, 9, 5, 8]]


# error_correction_test.clj:400-418 and the pipeline order of hardware_optimization.clj:70-100
def test_stage_in_the_pipeline():
    c = C.cnot_gate(C.h_gate(C.create_circuit(2), 0), 0, 1)
    ctx = optimize(c, {"supported-operations": {"h", "x", "z", "cnot"}},
                   {"apply-error-correction?": True, "error-correction-code": "bit-flip", "optimize-gates?": False,
                    "optimize-qubits?": False, "optimize-topology?": False, "transform-operations?": False})
    assert ctx["error-correction-applied?"] and ctx["circuit"]["num-qubits"] == 10
    assert ctx["physical-to-logical"][4] == 1 and ctx["ancilla-to-logical"][8] == 1
    assert ctx["pipeline-order"][2] == "error-correction"
    C.validate_circuit(ctx["circuit"])


def test_result_analysis():
    c = C.cnot_gate(C.h_gate(C.create_circuit(2), 0), 0, 1)
    ctx = optimize(c, None, {"apply-error-correction?": True, "optimize-topology?": False,
                             "transform-operations?": False, "error-correction-code": "bit-flip"})
    meas = {q: 0 for q in range(10)}
    meas.update({3: 1, 4: 1, 5: 0, 8: 1, 9: 1})  # block 1 syndrome [1 1]: qubit 4 flipped
    a = E.analyze_error_correction_results({"measurements": meas}, ctx)
    assert a["syndrome-bits"] == {0: [0, 0], 1: [1, 1]}
    assert a["decoded-syndromes"][1]["error-type"] == "x" and a["decoded-syndromes"][0]["error-type"] == "none"
    assert a["error-detected?"] is True and a["num-errors"] == 1 and a["error-rate"] == 0.5
    assert a["corrected-measurements"][4] == 0 and a["corrections-applied"] == [
        {"logical-qubit": 1, "physical-qubit": 4, "correction": "x"}]


# ---------------------------------------------------------------------------
# the encoded circuits on the oracle
def _embed(v, n):
    s = np.zeros(1 << n, complex)
    s[0], s[1 << (n - 1)] = v
    return s


def ec_round_trip(run, measure, key, error, qubit, v):
    """Encode v on qubit 0, apply one Pauli error, measure the syndrome on the ancillas,
    correct from the bits read and decode; returns (bits, probability, final state)."""
    size, nanc = SIZES[key]
    n = size + nanc
    data, anc = list(range(size)), list(range(size, n))
    c = E.get_encoding_function(key)(C.create_circuit(n), 0)
    if error:
        c = C.add_gate(c, error, target=qubit)
    c = E._emit(c, E.SYNDROME[key], data, anc)
    s = run(c, _embed(v, n))
    s, o, p = measure(s, anc)
    bits = [(o >> k) & 1 for k in range(nanc)]
    c = C.create_circuit(n)
    if key == "bit-flip":
        c = E.correct_bit_flip_error(c, data, bits)
    else:
        c = E.correct_shor_error(c, data, bits[:6], bits[6:])
    c = E.decode_shor(c, data) if key == "shor" else E.decode_bit_flip(c, data)
    return bits, p, run(c, s)


def _fidelity_on_qubit0(s, v):
    m = s.reshape(2, -1)
    w = m[:, np.argmax(np.abs(m).sum(0))]
    return abs(np.vdot(v, w)) ** 2


CASES = [("bit-flip", None, 0)] + [("bit-flip", "x", q) for q in range(3)] + \
    [("shor", None, 0)] + [("shor", e, q) for e in "xyz" for q in range(9)]


@pytest.mark.parametrize("key,error,qubit", CASES)
def test_oracle_round_trip_recovers(oracle, key, error, qubit):
    """The reference's bit-flip circuits correct any X error and its Shor circuits any
    single X, Y or Z error: the syndrome is certain and decoding returns the logical state."""
    v = np.array([0.6, 0.8j * np.exp(0.3j)])

    def measure(s, anc):
        return oracle.measure(s, anc, 7, 0)

    bits, p, s = ec_round_trip(lambda c, s0: oracle.run(c, s0), measure, key, error, qubit, v)
    assert abs(p - 1) < 1e-12 and abs(_fidelity_on_qubit0(s, v) - 1) < 1e-12
    if key == "bit-flip":
        assert bits == [[0, 0], [1, 0], [1, 1], [0, 1]][0 if error is None else qubit + 1]


def test_oracle_steane_and_five_qubit_encoders_leave_the_code_space(oracle):
    """The reference's Steane and five-qubit encoders do not prepare a state their
    generators stabilise: with no error the syndrome measurement is not certain."""
    for key in ("steane", "five-qubit"):
        size, nanc = SIZES[key]
        n = size + nanc
        c = E._emit(E.get_encoding_function(key)(C.create_circuit(n), 0), E.SYNDROME[key],
                    list(range(size)), list(range(size, n)))
        s = oracle.run(c, _embed(np.array([0.6, 0.8]), n))
        _, _, p = oracle.measure(s, list(range(size, n)), 7, 0)
        assert p < 0.99


def test_stage_then_routing():
    """The encoded circuit goes on through topology routing on a linear coupling; with no
    native SWAP each inserted SWAP becomes three CNOTs."""
    from qclojure_gb300 import topology as T

    c = C.cnot_gate(C.h_gate(C.create_circuit(2), 0), 0, 1)
    base = {"supported-operations": {"h", "cnot", "x", "z", "measure"}, "coupling": T.linear_coupling(12)}
    routed = optimize(c, base, {"apply-error-correction?": True, "optimize-topology?": True})
    native = optimize(c, {**base, "supported-operations": base["supported-operations"] | {"swap"}},
                      {"apply-error-correction?": True, "optimize-topology?": True})
    assert routed["swap-count"] == native["swap-count"] > 0
    assert len(routed["circuit"]["operations"]) == len(native["circuit"]["operations"]) + 2 * native["swap-count"]
    assert "swap" not in types(routed["circuit"])
    C.validate_circuit(routed["circuit"])
