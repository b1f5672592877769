"""The EDN reader and the device-catalogue loader (qclojure_gb300.edn,
hardware.load_devices), on catalogue text in the reference's format
(resources/simulator-devices.edn: a vector of device maps)."""
import pytest

from qclojure_gb300 import edn

CATALOGUE = """
[;; two devices in the catalogue's layout
 {:id :test-ideal
  :name "Test ideal device"
  :num-qubits 34
  :topology :all-to-all
  :coupling :all-to-all
  :native-gates #{:x :h :cnot :rz}
  :noise-model {}
  :performance {:gate-fidelity 1.0 :gate-times {:all 0} :max-shots 100000}}

 {:id :test-noisy, :name "Test \\"noisy\\" device\\n"
  :num-qubits 3
  :coupling [[1 2] [0 2] [0 1]]
  :native-gates #{:h :cnot}
  #_{:discarded :map}
  :noise-model {:gate-noise {:h {:noise-type :depolarizing :noise-strength 1.5e-3 :t1-time 120.0}
                             :cnot {:noise-type :amplitude-damping :noise-strength 0.01}}
                :readout-error {:prob-0-to-1 0.005 :prob-1-to-0 0.008
                                :correlated-errors {0 1.0 1 1.2 2 0.8}}}
  :ratio 1/4 :big 12N :neg -3 :flag true :nothing nil}]
"""


def test_reader_forms():
    v = edn.loads(CATALOGUE)
    assert isinstance(v, list) and [d["id"] for d in v] == ["test-ideal", "test-noisy"]
    a, b = v
    assert a["native-gates"] == frozenset({"x", "h", "cnot", "rz"}) and a["coupling"] == "all-to-all"
    assert a["performance"] == {"gate-fidelity": 1.0, "gate-times": {"all": 0}, "max-shots": 100000}
    assert b["name"] == 'Test "noisy" device\n' and b["coupling"] == [[1, 2], [0, 2], [0, 1]]
    assert b["noise-model"]["gate-noise"]["h"] == {"noise-type": "depolarizing", "noise-strength": 1.5e-3,
                                                   "t1-time": 120.0}
    assert b["noise-model"]["readout-error"]["correlated-errors"] == {0: 1.0, 1: 1.2, 2: 0.8}
    assert (b["ratio"], b["big"], b["neg"], b["flag"], b["nothing"]) == (0.25, 12, -3, True, None)
    assert "discarded" not in b
    assert edn.loads("#{[1 2] #{:a}}") == frozenset({(1, 2), frozenset({"a"})})
    assert edn.loads("(1 \\a sym ns/kw :ns/kw)") == [1, "a", "sym", "ns/kw", "ns/kw"]


@pytest.mark.parametrize("bad", ["{:a}", "[1 2", "\"open", "#inst \"2020\"", "1 2", ")"])
def test_reader_errors(bad):
    with pytest.raises(edn.EdnError):
        edn.loads(bad)


def test_catalogue_loads_into_the_hardware_simulator(tmp_path, monkeypatch):
    from qclojure_gb300 import hardware as H
    from qclojure_gb300 import state

    class FakeContext:
        def __init__(self, *a, **k):
            pass

        def close(self):
            pass

    monkeypatch.setattr(state, "Context", FakeContext)
    path = tmp_path / "devices.edn"
    path.write_text(CATALOGUE)
    devices = H.load_devices(str(path))
    sim = H.create_hardware_simulator(devices=devices)
    try:
        assert sim.device()["id"] == "test-ideal"  # the catalogue's first device, as the reference starts
        assert [d["id"] for d in sim.devices()] == ["test-ideal", "test-noisy"]
        assert sim.select_device("test-noisy")["num-qubits"] == 3
    finally:
        sim.close()
    (tmp_path / "bad.edn").write_text("{:id :x}")
    with pytest.raises(edn.EdnError):
        H.load_devices(str(tmp_path / "bad.edn"))


def test_flat_correlation_rows_adjust_nothing(oracle):
    """A catalogue row {qubit factor} is not a map of targets: the reference's `get` on the
    factor gives nil, so the readout noise is that of a model without correlations."""
    from qclojure_gb300 import circuit as C
    from qclojure_gb300.hardware import NoiseSpec

    flat = edn.loads(CATALOGUE)[1]["noise-model"]
    c = C.measure_all_operation(C.cnot_gate(C.h_gate(C.create_circuit(3), 0), 0, 1))
    assert NoiseSpec(c, flat).model.num_correlations == 0
    strong = {"prob-0-to-1": 0.4, "prob-1-to-0": 0.4, "correlated-errors": {0: 2.0, 1: {2: 0.1}}}
    weak = {"prob-0-to-1": 0.4, "prob-1-to-0": 0.4, "correlated-errors": {1: {2: 0.1}}}
    for shot in range(200):
        assert oracle.readout_noise(5, 3, strong, 9, shot) == oracle.readout_noise(5, 3, weak, 9, shot)
