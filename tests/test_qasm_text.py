"""The line-based OpenQASM converters (qclojure_gb300.qasm_text) with the cases of the
reference's tests (test/org/soulspace/qclojure/application/format/qasm2_test.clj,
qasm3_test.clj) restated. CPU only."""
import math

import pytest

from qclojure_gb300 import qasm_text as T


def g(t, **p):
    return {"operation-type": t, "operation-params": p}


def C(n, *ops):
    return {"num-qubits": n, "operations": list(ops)}


def types(c):
    return [o["operation-type"] for o in c["operations"]]


def test_qasm2_parsing():
    # qasm2_test.clj:75-119
    c = T.qasm2_to_circuit_lines('OPENQASM 2.0;\ninclude "qelib1.inc";\nqreg q[2];\ncreg c[2];\nh q[0];\ncx q[0], q[1];')
    assert c["num-qubits"] == 2 and types(c) == ["h", "cnot"]
    c = T.qasm2_to_circuit_lines('OPENQASM 2.0;\ninclude "qelib1.inc";\nqreg q[2];\nry(0.785) q[0];\nrz(1.571) q[1];')
    assert c["operations"] == [g("ry", target=0, angle=0.785), g("rz", target=1, angle=1.571)]
    c = T.qasm2_to_circuit_lines('OPENQASM 2.0;\nqreg q[3];\nswap q[0], q[2];\niswap q[1], q[2];')
    assert c["operations"] == [g("swap", qubit1=0, qubit2=2), g("iswap", qubit1=1, qubit2=2)]
    # lines must start with the gate; angles are Java double literals
    assert types(T.qasm2_to_circuit_lines("qreg q[1];\n  h q[0];\nid q[0];\nsdg q[0];")) == ["i", "s-dag"]
    with pytest.raises(ValueError):
        T.qasm2_to_circuit_lines("qreg q[1];\nrx(pi/2) q[0];")


def test_qasm2_emission_and_round_trip():
    # qasm2_test.clj:143-200
    c = C(3, g("h", target=0), g("cnot", control=0, target=1), g("swap", qubit1=0, qubit2=2),
          g("iswap", qubit1=1, qubit2=2), g("rx", target=0, angle=0.5), g("ry", target=1, angle=0.25),
          g("rz", target=2, angle=1.5), g("s-dag", target=0), g("phase", target=1, angle=0.75),
          g("crz", control=0, target=2, angle=0.125), g("toffoli", control1=0, control2=1, target=2))
    text = T.circuit_to_qasm2_lines(c)
    for line in ("OPENQASM 2.0;", 'include "qelib1.inc";', "qreg q[3];", "h q[0];", "cx q[0],q[1];",
                 "swap q[0],q[2];", "iswap q[1],q[2];", "rx(0.5) q[0];", "sdg q[0];", "p(0.75) q[1];",
                 "crz(0.125) q[0],q[2];", "ccx q[0],q[1],q[2];", "measure q -> c;"):
        assert line in text
    back = T.qasm2_to_circuit_lines(text)
    assert back["operations"] == c["operations"] and back["num-qubits"] == 3


def test_qasm3_emission():
    # qasm3_test.clj:70-164
    c = C(4, g("x", target=0), g("s-dag", target=0), g("t-dag", target=1), g("cnot", control=0, target=1),
          g("cz", control=1, target=2), g("rx", target=0, angle=math.pi / 2), g("phase", target=0, angle=math.pi / 4),
          g("swap", qubit1=0, qubit2=1), g("toffoli", control1=0, control2=1, target=2),
          g("fredkin", control=3, target1=0, target2=2), g("crx", control=0, target=1, angle=math.pi / 4),
          {"operation-type": "measure", "operation-params": {"measurement-qubits": [0, 1]}},
          g("unknown-gate", target=0))
    text = T.circuit_to_qasm3_lines(c)
    lines = text.splitlines()
    assert text.startswith("OPENQASM 3.0;") and "qubit[4] q;" in lines and "bit[4] c;" in lines
    for line in ("x q[0];", "sdg q[0];", "tdg q[1];", "cx q[0], q[1];", "cz q[1], q[2];",
                 f"rx({math.pi / 2!r}) q[0];", f"p({math.pi / 4!r}) q[0];", "swap q[0], q[1];", "ccx q[0], q[1], q[2];",
                 "cswap q[3], q[0], q[2];", f"crx({math.pi / 4!r}) q[0], q[1];", "c[0] = measure q[0];",
                 "c[1] = measure q[1];", "// Unknown gate: unknown-gate"):
        assert line in lines
    assert "measure q -> c;" not in text and "OPENQASM 2.0;" not in text
    bk = T.circuit_to_qasm3_lines(c, {"target": "braket"})
    assert 'include "stdgates.inc";' not in bk
    for line in ("si q[0];", "ti q[1];", "cnot q[0], q[1];", "ccnot q[0], q[1], q[2];", f"phaseshift({math.pi / 4!r}) q[0];"):
        assert line in bk.splitlines()
    spec = {"measurements": {"shots": 1000, "qubits": [0, 1]}, "expectation": {"observables": ["pauli-z"], "targets": [0]},
            "state-vector": True}
    withp = T.circuit_to_qasm3_lines(c, {"result-specs": spec})
    assert "// Result extraction specifications" in withp
    assert "#pragma qclojure result measurement shots=1000 qubits=0,1" in withp
    assert "#pragma qclojure result expectation observable=pauli-z target=0" in withp
    assert "#pragma qclojure result state_vector // Simulation-only result" in withp


def test_qasm3_parsing():
    # qasm3_test.clj:166-260
    c = T.qasm3_to_circuit_lines("OPENQASM 3.0;\n\nqubit[2] q;\nbit[2] c;\n\nh q[0];\ncx q[0], q[1];\n"
                                 "c[0] = measure q[0];\nc[1] = measure q[1];")
    assert c["num-qubits"] == 2 and types(c) == ["h", "cnot", "measure", "measure"]
    assert c["operations"][3]["operation-params"] == {"measurement-qubits": [1]}
    c = T.qasm3_to_circuit_lines("qubit[3] q;\nx q[0];\ny q[1];\nz q[2];\nh q[0];\ns q[1];\nt q[2];\nsdg q[0];\ntdg q[1];")
    assert types(c) == ["x", "y", "z", "h", "s", "t", "s-dag", "t-dag"]
    c = T.qasm3_to_circuit_lines("qubit[2] q;\n  rx(pi/2) q[0];\nry(-pi/4) q[1];\nrz(2*pi) q[0];\np(pi*0.5) q[1];\n"
                                 "crz(1/8) q[0], q[1];\nrx(pi) q[0];")
    assert [o["operation-params"]["angle"] for o in c["operations"]] == \
        [math.pi / 2, -math.pi / 4, 2 * math.pi, math.pi * 0.5, 0.125, math.pi]
    with pytest.raises(ValueError):
        T.qasm3_to_circuit_lines("qubit[1] q;\nrx(theta) q[0];")
    with pytest.raises(ValueError):  # the reference's "-pi*n" branch destructures a failed match
        T.qasm3_to_circuit_lines("qubit[1] q;\nrx(-pi*2) q[0];")
    c = T.qasm3_to_circuit_lines("qubit[4] q;\nswap q[0], q[1];\niswap q[1], q[2];\nccx q[0], q[1], q[2];\n"
                                 "cswap q[3], q[0], q[2];")
    assert types(c) == ["swap", "iswap", "toffoli", "fredkin"]


def test_qasm3_pragmas_and_round_trip():
    c = C(2, g("h", target=0), g("cnot", control=0, target=1), g("ry", target=1, angle=0.123456789012345))
    spec = {"measurements": {"shots": 100, "qubits": [0, 1]},
            "expectation": {"observables": ["pauli-z", "pauli-x"], "targets": [0, 1]}}
    text = T.circuit_to_qasm3_lines(c, {"result-specs": spec})
    back = T.qasm3_to_circuit_lines(text)
    assert back["operations"] == c["operations"]  # parameter precision (qasm3_test.clj:357-370)
    assert back["result-specs"] == {"measurement": {"shots": 100, "qubits": ["0", "1"]},
                                    "expectation": {"observable": "pauli-z", "target": 0,
                                                    "observables": ["pauli-x"], "targets": [1]}}
