"""Noise-model estimates (qclojure_gb300.noise_analysis), restating
test/org/soulspace/qclojure/application/noise_analysis_test.clj with exact values."""
import pytest

from qclojure_gb300 import circuit as C
from qclojure_gb300 import noise_analysis as N
from qclojure_gb300.clj import hash_keyword, lazy_seq_of_keywords_str, map_order

MODEL = {"gate-noise": {"h": {"noise-type": "depolarizing", "noise-strength": 0.001, "t1-time": 125.0,
                              "t2-time": 89.0, "gate-time": 35.6},
                        "x": {"noise-type": "amplitude-damping", "noise-strength": 0.0005, "t1-time": 125.0,
                              "t2-time": 89.0, "gate-time": 35.6},
                        "cnot": {"noise-type": "depolarizing", "noise-strength": 0.006, "t1-time": 125.0,
                                 "t2-time": 89.0, "gate-time": 476.0}},
         "readout-error": {"prob-0-to-1": 0.013, "prob-1-to-0": 0.028}}


def bell():
    return C.cnot_gate(C.h_gate(C.create_circuit(2), 0), 0, 1)


def test_fidelity_estimates():
    d = N.estimate_circuit_fidelity(bell(), MODEL)
    assert d["total-estimated-error"] == 0.0 + 1 * 0.001 + 1 * 0.006
    assert d["estimated-fidelity"] == 1.0 - d["total-estimated-error"]
    assert d["gate-counts"] == {"h": 1, "cnot": 1}
    assert d["dominant-error-sources"] == [("cnot", 0.006), ("h", 0.001)]
    c = bell()
    for q in (1, 2):
        c = C.h_gate(c, 0)
    empty = N.estimate_circuit_fidelity(C.create_circuit(1), MODEL)
    assert empty["estimated-fidelity"] == 1.0 and empty["total-estimated-error"] == 0.0
    assert N.estimate_circuit_fidelity(c, MODEL)["estimated-fidelity"] < 1.0
    custom = {"num-qubits": 1, "operations": [{"operation-type": "custom-gate", "operation-params": {"target": 0}}]}
    d = N.estimate_circuit_fidelity(custom, {"gate-noise": {"h": {"noise-type": "depolarizing",
                                                                   "noise-strength": 0.01}}})
    assert d["estimated-fidelity"] == 1.0 and d["total-estimated-error"] == 0.0
    huge = N.estimate_circuit_fidelity(bell(), {"gate-noise": {"h": {"noise-type": "d", "noise-strength": 0.9},
                                                               "cnot": {"noise-type": "d", "noise-strength": 0.9}}})
    assert huge["estimated-fidelity"] == 0.0


def test_platform_comparison():
    platforms = {"ibm-test": {"gate-noise": {"h": {"noise-type": "depolarizing", "noise-strength": 0.005},
                                             "cnot": {"noise-type": "depolarizing", "noise-strength": 0.01}},
                              "readout-error": {"prob-0-to-1": 0.02, "prob-1-to-0": 0.03}},
                 "ionq-test": {"gate-noise": {"h": {"noise-type": "coherent"},
                                              "cnot": {"noise-type": "depolarizing", "noise-strength": 0.003}},
                               "readout-error": {"prob-0-to-1": 0.001, "prob-1-to-0": 0.002}},
                 "mystery": {"gate-noise": {"h": {"noise-type": "depolarizing", "t1-time": 50.0}}}}
    r = N.compare_hardware_platforms(C.ghz_state_circuit(3), platforms)
    assert r["ibm-test"]["platform-type"] == "superconducting" and r["ionq-test"]["platform-type"] == "trapped-ion"
    assert r["mystery"]["platform-type"] == "unknown"
    assert r["ibm-test"]["total-estimated-error"] == 0.005 + 2 * 0.01
    assert r["ionq-test"]["coherence-times"] == {"t1-time": "N/A", "t2-time": "N/A"}
    assert r["mystery"]["coherence-times"]["t1-time"] == 50.0
    assert r["mystery"]["readout-fidelity"] == {"prob-0-to-1": "N/A", "prob-1-to-0": "N/A"}


def test_noise_aware_depth():
    assert N.noise_aware_circuit_depth(bell(), MODEL) == 2 + 2 * 0.006 * 10
    d0 = N.noise_aware_circuit_depth(C.create_circuit(1), MODEL)
    assert d0 == 0 and isinstance(d0, int)


def test_recommendations():
    low = N.recommend_error_mitigation(C.h_gate(C.create_circuit(1), 0),
                                       {"gate-noise": {"h": {"noise-type": "depolarizing", "noise-strength": 0.0001}}})
    assert low == []
    c = C.cnot_gate(C.h_gate(C.cnot_gate(C.h_gate(C.create_circuit(2), 0), 0, 1), 0), 0, 1)
    high = N.recommend_error_mitigation(c, {"gate-noise": {"h": {"noise-type": "d", "noise-strength": 0.1},
                                                           "cnot": {"noise-type": "d", "noise-strength": 0.2}}})
    assert [r["strategy"] for r in high] == ["noise-reduction", "selective-mitigation"]
    # `str` of a lazy sequence prints its class and hash code, not the gate types
    assert high[1]["suggestion"] == "Focus mitigation on: " + lazy_seq_of_keywords_str(["cnot", "h"])
    assert high[1]["suggestion"].startswith("Focus mitigation on: clojure.lang.LazySeq@")
    deep = C.create_circuit(2)
    for k in range(25):
        deep = C.h_gate(deep, k % 2)
    assert any(r["strategy"] == "circuit-cutting" for r in N.recommend_error_mitigation(deep, MODEL))


def test_many_gate_types_follow_the_hash_order():
    """Beyond eight gate types the counts iterate in the keyword hash trie's order, and the
    stable sort of the error sources keeps that order among equal contributions."""
    names = ["x", "y", "z", "h", "s", "t", "rx", "ry", "rz", "cnot"]
    c = C.create_circuit(2)
    for n in names:
        c = C.add_operation(c, n, {"target": 0})
    d = N.estimate_circuit_fidelity(c, {"gate-noise": {}})
    assert list(d["gate-counts"]) == map_order(names, hash_keyword) != names
    assert [t for t, _ in d["dominant-error-sources"]] == list(d["gate-counts"])
    with pytest.raises(ValueError):
        N.estimate_circuit_fidelity({"operations": []}, {})


def test_clojure_hashes():
    """Clojure's `hash` of 1 is 1392991556 and of :a is -2123407586."""
    from qclojure_gb300.clj import hash_long

    assert hash_long(1) == 1392991556
    assert hash_keyword("a") - (1 << 32) == -2123407586
