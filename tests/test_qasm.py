"""OpenQASM 2/3 ingestion and emission (qclojure_gb300.qasm), with the cases of the
reference's parser tests (test/org/soulspace/qclojure/application/format/
qasm2_parser_test.clj, qasm3_parser_test.clj) restated. CPU only."""
import math

import numpy as np
import pytest

from qclojure_gb300 import qasm as Q

H2 = 'OPENQASM 2.0;\ninclude "qelib1.inc";\n'
H3 = 'OPENQASM 3.0;\ninclude "stdgates.inc";\n'


def _ops(c):
    return [(o["operation-type"], o.get("operation-params")) for o in c["operations"]]


@pytest.mark.parametrize("version", [2, 3])
def test_single_qubit_gates(version):
    # qasm2_parser_test.clj:33-86, qasm3_parser_test.clj:33-75
    head, reg = (H2, "qreg q[4];") if version == 2 else (H3, "qubit[4] q;")
    code = head + reg + "\nh q[0];\nx q[1];\ny q[2];\nz q[3];\ns q[0];\nt q[1];\nsdg q[2];\ntdg q[3];"
    c = Q.qasm2_to_circuit(code)["circuit"] if version == 2 else Q.qasm3_to_circuit(code)
    assert c["num-qubits"] == 4
    assert [t for t, _ in _ops(c)] == ["h", "x", "y", "z", "s", "t", "s-dag", "t-dag"]
    emitted = Q.circuit_to_qasm2(c) if version == 2 else Q.circuit_to_qasm3(c)
    for line in ("h q[0];", "x q[1];", "y q[2];", "z q[3];", "sdg q[2];", "tdg q[3];"):
        assert line in emitted


def test_identity_gate():
    # qasm2_parser_test.clj:77-86
    c = Q.qasm2_to_circuit(H2 + "qreg q[1];\nid q[0];")["circuit"]
    assert _ops(c) == [("i", {"target": 0})]
    assert "id q[0];" in Q.circuit_to_qasm2(c)


@pytest.mark.parametrize("version", [2, 3])
def test_parametric_gates(version):
    # qasm2_parser_test.clj:91-121, qasm3_parser_test.clj:79-111
    head, reg = (H2, "qreg q[3];") if version == 2 else (H3, "qubit[3] q;")
    code = head + reg + "\nrx(1.5708) q[0];\nry(0.7854) q[1];\nrz(3.1416) q[2];\np(1.2345) q[0];"
    c = Q.qasm2_to_circuit(code)["circuit"] if version == 2 else Q.qasm3_to_circuit(code)
    assert _ops(c) == [("rx", {"target": 0, "angle": 1.5708}), ("ry", {"target": 1, "angle": 0.7854}),
                       ("rz", {"target": 2, "angle": 3.1416}), ("phase", {"target": 0, "angle": 1.2345})]
    emitted = Q.circuit_to_qasm2(c) if version == 2 else Q.circuit_to_qasm3(c)
    for line in ("rx(1.5708) q[0];", "ry(0.7854) q[1];", "rz(3.1416) q[2];", "p(1.2345) q[0];"):
        assert line in emitted


@pytest.mark.parametrize("version", [2, 3])
def test_multi_qubit_gates(version):
    # qasm2_parser_test.clj:126-216, qasm3_parser_test.clj:116-199
    head, reg = (H2, "qreg q[4];") if version == 2 else (H3, "qubit[4] q;")
    code = head + reg + ("\ncx q[0], q[1];\ncy q[0], q[1];\ncz q[2], q[3];\nswap q[0], q[3];\niswap q[1], q[2];"
                         "\nccx q[0], q[1], q[2];\ncswap q[1], q[2], q[3];")
    c = Q.qasm2_to_circuit(code)["circuit"] if version == 2 else Q.qasm3_to_circuit(code)
    assert _ops(c) == [("cnot", {"control": 0, "target": 1}), ("cy", {"control": 0, "target": 1}),
                       ("cz", {"control": 2, "target": 3}), ("swap", {"qubit1": 0, "qubit2": 3}),
                       ("iswap", {"qubit1": 1, "qubit2": 2}),
                       ("toffoli", {"control1": 0, "control2": 1, "target": 2}),
                       ("fredkin", {"control": 1, "target1": 2, "target2": 3})]
    emitted = Q.circuit_to_qasm2(c) if version == 2 else Q.circuit_to_qasm3(c)
    for line in ("cx q[0], q[1];", "cy q[0], q[1];", "cz q[2], q[3];", "swap q[0], q[3];", "iswap q[1], q[2];",
                 "ccx q[0], q[1], q[2];", "cswap q[1], q[2], q[3];"):
        assert line in emitted


def test_qasm2_result_pragmas():
    # qasm2_parser_test.clj:221-258
    code = H2 + "// #pragma qclojure result measurement shots=1000 qubits=0,1,2\nqreg q[3];\nh q[0];\ncx q[0], q[1];"
    r = Q.qasm2_to_circuit(code)
    assert r["result-specs"] == {"measurement": {"shots": 1000, "qubits": [0, 1, 2]}}
    assert "// #pragma qclojure result measurement" in Q.circuit_to_qasm2(r["circuit"], r["result-specs"])
    code = (H2 + "// #pragma qclojure result expectation observable=pauli-z target=0\n"
            "// #pragma qclojure result variance observable=pauli-x target=1\nqreg q[2];\nh q[0];\nx q[1];")
    r = Q.qasm2_to_circuit(code)
    assert r["result-specs"] == {"expectation": {"observable": "pauli-z", "target": 0},
                                 "variance": {"observable": "pauli-x", "target": 1}}
    em = Q.circuit_to_qasm2(r["circuit"], r["result-specs"])
    assert "// #pragma qclojure result expectation" in em and "// #pragma qclojure result variance" in em


ROUND_TRIP_GATES = ("h q[0];\nx q[1];\ny q[2];\nz q[3];\ns q[4];\nt q[0];\nsdg q[1];\ntdg q[2];\n{rx} q[3];\n"
                    "ry(0.7854) q[4];\n{rz} q[0];\np(0.5236) q[1];\ncx q[0], q[1];\ncy q[1], q[2];\n"
                    "cz q[2], q[3];\nswap q[0], q[4];\niswap q[1], q[3];\nccx q[0], q[1], q[2];\n"
                    "cswap q[2], q[3], q[4];")


def test_qasm2_round_trip():
    # qasm2_parser_test.clj:263-303
    code = (H2 + "// #pragma qclojure result measurement shots=2000 qubits=0,1,2,3\nqreg q[5];\n"
            + ROUND_TRIP_GATES.format(rx="rx(1.5708)", rz="rz(3.1416)"))
    r = Q.qasm2_to_circuit(code)
    em = Q.circuit_to_qasm2(r["circuit"], r["result-specs"])
    r2 = Q.qasm2_to_circuit(em)
    assert len(r["circuit"]["operations"]) == 19 and len(r["result-specs"]) == 1
    assert r2["circuit"]["operations"] == r["circuit"]["operations"]
    assert r2["result-specs"] == r["result-specs"]
    for line in ("swap q[0], q[4];", "iswap q[1], q[3];", "ccx q[0], q[1], q[2];", "cswap q[2], q[3], q[4];"):
        assert line in em


def test_qasm3_round_trip_with_expressions():
    # qasm3_parser_test.clj:204-239: rx(pi/2), rz(pi) evaluated
    c = Q.qasm3_to_circuit(H3 + "qubit[5] q;\n" + ROUND_TRIP_GATES.format(rx="rx(pi/2)", rz="rz(pi)"))
    assert len(c["operations"]) == 19
    assert c["operations"][8]["operation-params"]["angle"] == math.pi / 2
    assert c["operations"][10]["operation-params"]["angle"] == math.pi
    em = Q.circuit_to_qasm3(c)
    c2 = Q.qasm3_to_circuit(em)
    assert c2["operations"] == c["operations"]
    assert "rx(1.5707963267948966) q[3];" in em


def test_empty_invalid_and_unknown():
    # qasm2_parser_test.clj:305-331, qasm3_parser_test.clj:241-265
    c = Q.qasm2_to_circuit(H2 + "qreg q[1];")["circuit"]
    assert c["operations"] == [] and "qreg q[1];" in Q.circuit_to_qasm2(c)
    c = Q.qasm3_to_circuit(H3 + "qubit[1] q;")
    assert c["operations"] == [] and "qubit[1] q;" in Q.circuit_to_qasm3(c)
    with pytest.raises(ValueError):
        Q.qasm2_to_circuit("INVALID QASM CONTENT")
    with pytest.raises(ValueError):
        Q.qasm3_to_circuit("INVALID QASM CONTENT")
    assert Q.qasm2_to_circuit(H2 + "qreg q[1];\nunsupported_gate q[0];")["circuit"]["operations"] == []


def test_comments_and_ignored_statements():
    # qasm3_parser_test.clj:268-334; measure/barrier/reset/creg add nothing
    code = ("OPENQASM 3.0;\n// Line comment at start\n/* Block comment */ include \"stdgates.inc\"; // eol\n"
            "qubit[3] q;\nbit[3] c;\n// Before gate operations\nh q[0]; /* Inline block */ y q[1]; // another\n"
            "/* Multi-line block\n   comment here */\ncx q[0], q[1]; // Final comment\nbarrier q;\n"
            "c[0] = measure q[0];\nmeasure q[1] -> c[1];\nreset q[2];")
    assert [o["operation-type"] for o in Q.qasm3_to_circuit(code)["operations"]] == ["h", "y", "cnot"]
    code2 = (H2 + "qreg q[2];\ncreg c[2];\nh q[0];\nbarrier q[0], q[1];\nmeasure q[0] -> c[0];\n"
             "if (c == 1) x q[1];\nreset q[1];\ncx q[0], q[1];")
    assert [o["operation-type"] for o in Q.qasm2_to_circuit(code2)["circuit"]["operations"]] == ["h", "cnot"]


def test_parameter_semantics():
    # QASM 2 takes the first numeric literal of a parameter expression (qasm2_parser.clj:190-202)
    c = Q.qasm2_to_circuit(H2 + "qreg q[1];\nrx(pi/2) q[0];\nrz(-0.25) q[0];\nry(pi) q[0];")["circuit"]
    assert [o["operation-params"]["angle"] for o in c["operations"]] == [2, 0.25, 0.0]
    c = Q.qasm2_to_circuit(H2 + "qreg q[1];\nrx(pi/2) q[0];", evaluate_expressions=True)["circuit"]
    assert c["operations"][0]["operation-params"]["angle"] == math.pi / 2
    # QASM 3 evaluates constant expressions (qasm3_parser.clj:341-512)
    c = Q.qasm3_to_circuit(H3 + "qubit[1] q;\nrx(2*pi/3) q[0];\nry(-tau/4) q[0];\nrz(sqrt(2)**2) q[0];\n"
                           "p(euler) q[0];\nrx(7 % 3 + 1) q[0];\nry(arccos(0)) q[0];")
    got = [o["operation-params"]["angle"] for o in c["operations"]]
    assert got == [2 * math.pi / 3, -(2 * math.pi) / 4, math.pow(math.sqrt(2), 2), math.e, 2, math.acos(0)]
    with pytest.raises(ValueError):
        Q.qasm3_to_circuit(H3 + "qubit[1] q;\nrx(theta) q[0];")


def test_qasm3_result_pragmas_and_emission():
    code = (H3 + "#pragma qclojure result measurement shots=500 qubits=0,1\n"
            "#pragma qclojure result expectation observable=pauli-z target=0\n"
            "#pragma qclojure result expectation observable=pauli-x target=1\nqubit[2] q;\nh q[0];")
    c = Q.qasm3_to_circuit(code)
    assert c["result-specs"] == {"measurement": {"shots": 500, "qubits": [0, 1]},
                                 "expectation": {"observable": "pauli-z", "target": 0,
                                                 "observables": ["pauli-x"], "targets": [1]}}
    em = Q.circuit_to_qasm3(c, {"result-specs": c["result-specs"]})
    assert "#pragma" not in em  # qasm3_parser.clj:844-846 hands the specs one level too deep
    assert 'include "stdgates.inc"' not in Q.circuit_to_qasm3(c, {"target": "braket"})


def test_number_formatting():
    assert [Q.clj_str(x) for x in (2, 2.0, 1.5708, 1e-05, 12345678.9, 0.000123, 1e22, -0.0)] == \
        ["2", "2.0", "1.5708", "1.0E-5", "1.23456789E7", "1.23E-4", "1.0E22", "-0.0"]


def test_parsed_circuit_runs_like_the_built_one(oracle):
    from qclojure_gb300 import workloads

    built = workloads.layered_circuit(6, 4, seed=3)
    em = Q.circuit_to_qasm3(built)
    parsed = Q.qasm3_to_circuit(em)
    assert np.array_equal(oracle.run(parsed), oracle.run(built))
