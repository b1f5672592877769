"""Device normalisation (qclojure_gb300.device, domain/device.clj:50-73) and the hardware
simulator normalising a device it is given."""
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


def test_topology_without_qubit_count_names_the_problem():
    import pytest

    with pytest.raises(ValueError, match="num-qubits"):
        D.validate_device({"id": "t", "topology": "ring"})
    with pytest.raises(ValueError, match="num-qubits"):
        D.validate_device({"id": "t", "topology": "linear", "num-qubits": -1})


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
