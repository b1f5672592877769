"""Device maps (qclojure_gb300.device), restating domain/device.clj's normalisation and
queries, and the hardware simulator normalising a device it is given."""
from qclojure_gb300 import device as D


def test_supported_operations_and_validation():
    d = {"name": "d", "num-qubits": 3, "native-gates": {"h", "cnot"}, "virtual-gates": {"swap"},
         "topology": "linear"}
    v = D.validate_device(d)
    assert v["supported-operations"] == frozenset({"h", "cnot", "swap"})
    assert v["coupling"] == [[1], [0, 2], [1]]
    own = D.validate_device({**d, "supported-operations": {"x"}, "coupling": [[1], [0]]})
    assert own["supported-operations"] == {"x"} and own["coupling"] == [[1], [0]]
    bare = D.validate_device({"name": "b", "num-qubits": 1})
    assert bare["supported-operations"] == frozenset() and bare["coupling"] is None
    assert [x["supported-operations"] for x in D.validate_devices([d])] == [v["supported-operations"]]


def test_fidelities_and_noise():
    d = {"performance": {"two-qubit-gate-fidelity": 0.99, "single-qubit-gate-fidelity": 0.999}}
    assert D.gate_fidelity(d) == 0.99 and D.gate_fidelity({}) is None
    assert D.estimated_fidelity(d, 3) == 0.99 ** 3
    assert D.estimated_fidelity(d, 0) is None and D.estimated_fidelity({}, 3) is None
    assert D.noise_model({}) == {} and D.noise_model({"noise-model": {"a": 1}}) == {"a": 1}


def test_circuit_checks_and_comparison():
    c = {"num-qubits": 2, "operations": [{"operation-type": "h"}, {"operation-type": "cz"},
                                         {"operation-type": "h"}, {"operation-type": "rx"}]}
    r = D.validate_circuit({"supported-operations": {"h", "cnot"}}, c)
    assert r == {"all-gates-supported?": False, "unsupported-gates": ["cz", "rx"]}
    assert D.validate_circuit({}, c)["unsupported-gates"] == ["h", "cz", "rx"]
    cmp = D.compare_gate_support({"supported-operations": {"h", "x"}}, {"supported-operations": {"x", "y"}})
    assert cmp["shared-operations"] == {"x"} and cmp["device1-only"] == {"h"} and cmp["device2-only"] == {"y"}
    assert cmp["total-unique-operations"] == {"h", "x", "y"}


def test_simulator_normalises_its_device(monkeypatch):
    from qclojure_gb300 import hardware as H
    from qclojure_gb300 import state

    class FakeContext:
        def __init__(self, *a, **k):
            pass

        def close(self):
            pass

    monkeypatch.setattr(state, "Context", FakeContext)
    sim = H.create_hardware_simulator(device={"id": "d", "name": "d", "num-qubits": 4,
                                              "native-gates": {"h", "cnot", "swap"}, "topology": "ring"})
    try:
        assert sim.device()["supported-operations"] == frozenset({"h", "cnot", "swap"})
        assert sim.device()["coupling"] == [[3, 1], [0, 2], [1, 3], [2, 0]]  # the ring's neighbour order
    finally:
        sim.close()
