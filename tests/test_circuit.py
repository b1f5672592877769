"""Host logic: circuit builders, alias resolution, encoding and metadata."""
import math

import numpy as np
import pytest

from qclojure_gb300 import _abi as A
from qclojure_gb300 import circuit as qc
from qclojure_gb300 import workloads


def test_builders_produce_reference_maps():
    c = qc.cnot_gate(qc.h_gate(qc.create_circuit(2, "Bell"), 0), 0, 1)
    assert c["operations"] == [{"operation-type": "h", "operation-params": {"target": 0}},
                               {"operation-type": "cnot", "operation-params": {"control": 0, "target": 1}}]
    c = qc.rydberg_blockade_gate(qc.create_circuit(3), [0, 2], 0.5)
    assert c["operations"][0]["operation-params"] == {"qubit-indices": [0, 2], "angle": 0.5}
    c = qc.measure_all_operation(qc.create_circuit(3))
    assert c["operations"][0] == {"operation-type": "measure", "operation-params": {"measurement-qubits": [0, 1, 2]}}
    assert qc.global_x_gate(qc.create_circuit(2))["operations"][0] == {"operation-type": "global-x"}


@pytest.mark.parametrize("alias,canon", [("cx", "cnot"), ("not", "x"), ("p", "phase"), ("sdg", "s-dag"),
                                         ("ccx", "toffoli"), ("cswap", "fredkin"), ("ti", "t-dag")])
def test_aliases(alias, canon):
    assert qc.resolve_gate_alias(alias) == canon


def test_encoding_fields():
    op = qc.encode_operation({"operation-type": "cx", "operation-params": {"control": 3, "target": 1}})[0]
    assert op.opcode == A.OP["cnot"] and op.nq == 2 and list(op.q[:2]) == [3, 1]
    op = qc.encode_operation({"operation-type": "rydberg-cphase",
                              "operation-params": {"control": 0, "target": 2, "angle": 0.25}})[0]
    assert op.opcode == A.OP["rydberg_cphase"] and op.angle == 0.25
    op = qc.encode_operation({"operation-type": "measure", "operation-params": {"measurement-qubits": [4, 1]}})[0]
    assert op.opcode == A.OP["measure"] and list(op.q[:2]) == [4, 1]
    # default target 0 for single-qubit gates without :target (circuit.clj:966-982)
    assert qc.encode_operation({"operation-type": "s"})[0].q[0] == 0


def test_controlled_dispatch_like_reference():
    enc = lambda g: qc.encode_operation({"operation-type": "controlled", "operation-params": {  # noqa: E731
        "control-qubits": [0], "target-gate": g, "target-qubits": [1]}})
    assert enc("x")[0].opcode == A.OP["cnot"]
    assert enc("y")[0].opcode == A.OP["cy"]
    assert enc("h")[0].opcode == A.OP["h"] and enc("h")[0].q[0] == 1  # applied uncontrolled
    assert enc("rx") == []                                             # unchanged state
    with pytest.raises(qc.CircuitError):
        qc.encode_operation({"operation-type": "controlled", "operation-params": {
            "control-qubits": [0, 2], "target-gate": "x", "target-qubits": [1]}})


@pytest.mark.parametrize("op", [
    {"operation-type": "i", "operation-params": {"target": 0}},
    {"operation-type": "cy", "operation-params": {"control": 0, "target": 1}},
    {"operation-type": "cnot", "operation-params": {"control": 0}},
    {"operation-type": "crz", "operation-params": {"control": 0, "target": 1}},
    {"operation-type": "swap", "operation-params": {"qubit1": 0}},
    {"operation-type": "global-rx"},
])
def test_reference_errors(op):
    with pytest.raises(qc.CircuitError):
        qc.encode_operation(op)


def test_circuit_depth_examples():
    assert qc.circuit_depth(qc.bell_state_circuit()) == 2
    c = qc.create_circuit(3)
    c = qc.h_gate(qc.h_gate(qc.h_gate(c, 0), 1), 2)
    assert qc.circuit_depth(c) == 1
    c = qc.cnot_gate(c, 0, 2)           # span [0,2] blocks qubit 1 too
    c = qc.x_gate(c, 1)
    assert qc.circuit_depth(c) == 3
    assert qc.circuit_metadata(c) == {"circuit-depth": 3, "circuit-operation-count": 5, "circuit-gate-count": 5}
    assert qc.circuit_depth(qc.create_circuit(2)) == 0


def test_workloads_are_seeded_and_shaped():
    a = workloads.layered_circuit(10, 20, seed=0)
    b = workloads.layered_circuit(10, 20, seed=0)
    assert a == b
    assert len(a["operations"]) == 20 * (10 + 5)
    big = workloads.large_circuit(30, 40, seed=1)
    assert len(big["operations"]) == 40 * 45 + 30 + 435 + 15
    q = workloads.qaoa_maxcut(12, 3, seed=4)
    deg = np.zeros(12, int)
    for a_, b_ in q["edges"]:
        deg[a_] += 1
        deg[b_] += 1
    assert len(q["edges"]) == 18 and np.all(deg == 3)
    assert len(q["operations"]) == 12 + 3 * (18 + 12)
    tr = workloads.serving_trace(200, 1000.0, seed=1)
    ns = np.array([j["n"] for j in tr])
    assert ns.min() >= 8 and ns.max() <= 28
    assert all(10 <= j["depth"] <= 200 for j in tr)
    assert 0.8 < np.mean(["measurements" in j["result-specs"] for j in tr]) < 1.0
    arr = np.array([j["arrival-s"] for j in tr])
    assert np.all(np.diff(arr) > 0)


def test_qft_op_counts():
    ops = workloads.qft_ops(30)
    kinds = [o["operation-type"] for o in ops]
    assert kinds.count("h") == 30 and kinds.count("rydberg-cphase") == 435 and kinds.count("swap") == 15
    assert all(o["operation-params"]["angle"] == math.pi / 2 ** (o["operation-params"]["control"]
                                                                - o["operation-params"]["target"])
               for o in ops if o["operation-type"] == "rydberg-cphase")


def test_circuit_depth_per_qubit_cover_equals_span_scan():
    """circuit_depth keeps the latest covering-span layer per qubit; it must agree
    with the scan over every span (the reference's form) on mixed circuits."""
    from qclojure_gb300 import workloads
    from qclojure_gb300.circuit import _circuit_depth_by_spans, circuit_depth
    from test_gpu_parity import every_gate_circuit

    for seed in range(12):
        for c in (workloads.large_circuit(10, 4, seed), every_gate_circuit(8, seed),
                  workloads.layered_circuit(6, 7, seed), workloads.qaoa_maxcut(12, 2, seed)):
            assert circuit_depth(c) == _circuit_depth_by_spans(c)
