"""OpenQASM programs run on the device through the job API and checked against the oracle.

QASM 2 and 3 texts are parsed by qasm.py (the reference's qasm2_parser.clj and
qasm3_parser.clj restated) and by the line-based converters of qasm_text.py (qasm2.clj,
qasm3.clj); the parsed circuits are submitted with qg_submit (backend.submit_circuit) and
their final states, probabilities and shot outcomes compared with the oracle's run of the
same parsed circuit. Every gate a QASM program can name appears at least once. Tolerances:
complex128 exact arithmetic bit-exact, double-float <= 1e-12 per amplitude, outcomes
identical; complex64 probability TVD <= 1e-5.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

QASM2 = """OPENQASM 2.0;
include "qelib1.inc";
// #pragma qclojure result measurement shots=900 qubits=0,1,2,3,4,5
qreg q[6];
creg c[6];
h q[0];
x q[1];
y q[2];
z q[3];
s q[4];
sdg q[5];
t q[0];
tdg q[1];
rx(0.7) q[2];
ry(1.3) q[3];
rz(-0.4) q[4];
p(2.1) q[5];
cx q[0], q[3];
cz q[1], q[4];
swap q[2], q[5];
crx(0.9) q[3], q[0];
cry(1.7) q[4], q[1];
crz(2.5) q[5], q[2];
ccx q[0], q[1], q[2];
cswap q[3], q[4], q[5];
h q[1];
iswap q[0], q[4];
rx(pi/3) q[5];
measure q -> c;
"""

QASM3 = """OPENQASM 3.0;
include "stdgates.inc";
#pragma qclojure result measurement shots=700 qubits=0,1,2,3,4,5,6
qubit[7] q;
bit[7] c;
h q[0];
x q[1];
y q[2];
z q[3];
s q[4];
sdg q[5];
t q[6];
tdg q[0];
rx(pi/4) q[1];
ry(2*pi/3) q[2];
rz(-pi/8) q[3];
p(0.5) q[4];
cx q[0], q[5];
cz q[1], q[6];
swap q[2], q[4];
iswap q[3], q[0];
crx(pi/5) q[4], q[1];
cry(1.1) q[5], q[2];
crz(0.3) q[6], q[3];
ccx q[0], q[1], q[2];
cswap q[3], q[4], q[5];
h q[2];
c = measure q;
"""


def _sv(r):
    return np.asarray(r["results"]["final-state"]["state-vector"])


def _run(sim, circuit, shots, seed):
    jid = sim.submit_circuit(circuit, {"result-specs": {"measurements": {"shots": shots}, "probabilities": {},
                                                        "state-vector": True}, "seed": seed})
    assert sim.wait(jid, 300_000) == "completed", sim.job_result(jid)
    r = sim.job_result(jid)
    sim.free_job(jid)
    return r


def _parsed_programs():
    from qclojure_gb300 import qasm as Q
    from qclojure_gb300 import qasm_text as QT
    from qclojure_gb300 import workloads

    out = []
    p2 = Q.qasm2_to_circuit(QASM2, evaluate_expressions=True)
    out.append(("qasm2 evaluated", p2["circuit"], p2["result-specs"]))
    p2q = Q.qasm2_to_circuit(QASM2)  # the reference's first-literal parameter rule
    out.append(("qasm2 first literal", p2q["circuit"], p2q["result-specs"]))
    p3 = Q.qasm3_to_circuit(QASM3)
    out.append(("qasm3", {k: v for k, v in p3.items() if k != "result-specs"}, p3["result-specs"]))
    # emitted by one side, read by the other: a random layered circuit through both formats
    lc = workloads.layered_circuit(9, 6, seed=21)
    out.append(("qasm3 round trip", {k: v for k, v in Q.qasm3_to_circuit(Q.circuit_to_qasm3(lc)).items()
                                     if k != "result-specs"}, None))
    out.append(("qasm2 round trip", Q.qasm2_to_circuit(Q.circuit_to_qasm2(lc), evaluate_expressions=True)["circuit"],
                None))
    out.append(("qasm3 lines", QT.qasm3_to_circuit_lines(QT.circuit_to_qasm3_lines(lc)), None))
    out.append(("qasm2 lines", QT.qasm2_to_circuit_lines(QT.circuit_to_qasm2_lines(lc)), None))
    return out


def test_parsed_programs_cover_every_gate():
    progs = _parsed_programs()
    kinds = {op["operation-type"] for _, c, _ in progs for op in c["operations"]}
    # the Rydberg and global gates' registry names (rydberg-cz, global-h, ...) are not QASM
    # identifiers, so no program text can name them; every other gate of the registry appears
    want = {"h", "x", "y", "z", "s", "s-dag", "t", "t-dag", "rx", "ry", "rz", "phase", "cnot", "cz", "swap",
            "iswap", "crx", "cry", "crz", "toffoli", "fredkin"}
    assert want <= kinds, want - kinds


@pytest.mark.parametrize("arith,tol", [("exact", 0.0), ("double-float", 1e-12)])
def test_qasm_programs_on_device_c128(oracle, arith, tol):
    from qclojure_gb300.backend import create_simulator

    sim = create_simulator({"precision": "c128", "fusion": "tiled", "workers": 2, "seed": 4, "arithmetic": arith})
    try:
        for name, circ, specs in _parsed_programs():
            shots = (specs or {}).get("measurements", {}).get("shots", 500)
            r = _run(sim, circ, shots, seed=13)
            ref = oracle.run(circ)
            err = float(np.max(np.abs(_sv(r) - ref)))
            assert err <= tol, (name, err)
            p = np.asarray(r["results"]["probability-results"]["all-probabilities"])
            assert float(np.max(np.abs(p - oracle.probabilities(ref)))) <= max(tol, 1e-15), name
            got = np.array(r["results"]["measurement-results"]["measurement-outcomes"], np.uint64)
            assert np.array_equal(got, oracle.sample(ref, shots, 13)), name
    finally:
        sim.close()


def test_qasm_programs_on_device_c64(oracle):
    from qclojure_gb300.backend import create_simulator

    sim = create_simulator({"precision": "c64", "fusion": "tiled", "workers": 2, "seed": 4})
    try:
        for name, circ, specs in _parsed_programs():
            r = _run(sim, circ, 200, seed=3)
            pref = oracle.probabilities(oracle.run(circ))
            p = np.asarray(r["results"]["probability-results"]["all-probabilities"])
            tvd = 0.5 * float(np.abs(p - pref).sum())
            assert tvd <= 1e-5, (name, tvd)
    finally:
        sim.close()


def test_qasm2_first_literal_rule_changes_the_state(oracle):
    """rx(pi/3) parses as rx(3) under the reference's default rule (first numeric literal,
    qasm2_parser.clj:190-202) and as rx(pi/3) when evaluated; the device follows each."""
    from qclojure_gb300 import qasm as Q

    a = Q.qasm2_to_circuit(QASM2)["circuit"]["operations"][-1]
    b = Q.qasm2_to_circuit(QASM2, evaluate_expressions=True)["circuit"]["operations"][-1]
    assert a["operation-params"]["angle"] == 3 and math.isclose(b["operation-params"]["angle"], math.pi / 3)
