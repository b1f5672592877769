"""Gate and qubit optimisation (qclojure_gb300.optimization) with the cases of the
reference's tests (test/org/soulspace/qclojure/domain/gate_optimization_test.clj,
qubit_optimization_test.clj) restated. CPU only."""
import math

import numpy as np
import pytest

from qclojure_gb300 import optimization as O


def g(t, **p):
    return {"operation-type": t, "operation-params": p}


def C(n, *ops):
    return {"num-qubits": n, "operations": list(ops)}


def types(c):
    return [o["operation-type"] for o in c["operations"]]


def test_cancellation_pairs():
    # gate_optimization_test.clj:49-94
    h, x, y = g("h", target=0), g("x", target=0), g("y", target=1)
    cn = g("cnot", control=0, target=1)
    assert O.find_cancellation_pairs([]) == [] and O.find_cancellation_pairs([h]) == []
    assert O.find_cancellation_pairs([h, h]) == [(0, 1)] and O.find_cancellation_pairs([cn, cn]) == [(0, 1)]
    assert O.find_cancellation_pairs([h, x]) == [] and O.find_cancellation_pairs([h, x, h]) == []
    assert O.find_cancellation_pairs([h, h, x, x]) == [(0, 1), (2, 3)]
    assert O.find_cancellation_pairs([h, y, h]) == [(0, 2)]
    assert O.remove_pairs([h, h, y], [(0, 1)]) == [y]


def test_optimize_gates_cases():
    # gate_optimization_test.clj:96-170, :220-265
    for c in (C(2), C(1, g("h", target=0), g("h", target=0)),
              C(3, g("h", target=0), g("h", target=0), g("x", target=1), g("x", target=1), g("y", target=2),
                g("y", target=2)),
              C(1, g("h", target=0), g("h", target=0), g("x", target=0), g("x", target=0))):
        with pytest.raises(O.OptimizationError, match="Optimization resulted in an empty circuit"):
            O.optimize_gates(c)
    r = O.optimize_gates(C(2, g("h", target=0), g("h", target=0), g("x", target=1), g("y", target=1),
                           g("y", target=1)))
    assert types(r) == ["x"]
    assert types(O.optimize_gates(C(2, g("h", target=0), g("cnot", control=0, target=1)))) == ["h", "cnot"]
    assert types(O.optimize_gates(C(2, g("h", target=0), g("cnot", control=0, target=1), g("h", target=0)))) == \
        ["h", "cnot", "h"]
    assert len(O.optimize_gates(C(2, g("cz", control=0, target=1), g("swap", qubit1=0, qubit2=1),
                                  g("cz", control=0, target=1)))["operations"]) == 3
    assert types(O.optimize_gates(C(3, g("h", target=0), g("x", target=1), g("y", target=2),
                                    g("h", target=0)))) == ["x", "y"]
    # SWAP is symmetric; S/S-dagger and T/T-dagger cancel
    assert types(O.optimize_gates(C(2, g("swap", qubit1=0, qubit2=1), g("swap", qubit1=1, qubit2=0),
                                    g("x", target=0)))) == ["x"]
    assert types(O.optimize_gates(C(1, g("s", target=0), g("s-dag", target=0), g("x", target=0)))) == ["x"]


def test_rotation_folding():
    # gate_optimization_test.clj:432-560
    r = O.combine_rotations(g("rx", target=0, angle=0.5), g("rx", target=0, angle=1.0))
    assert r == g("rx", target=0, angle=1.5)
    assert O.combine_rotations(g("rz", target=0, angle=1.0), g("rz", target=0, angle=-1.0)) is None
    s_t = O.combine_rotations(g("s", target=0), g("t", target=0))
    assert s_t["operation-type"] == "rz" and s_t["operation-params"]["angle"] == pytest.approx(3 * math.pi / 4)
    assert O.normalize_angle(0.5) == 0.5 and O.normalize_angle(math.pi) == math.pi
    assert O.normalize_angle(1e-15) == 0.0 and O.normalize_angle(-1e-15) == 0.0
    assert O.normalize_angle(2 * math.pi - 1e-14) == 0.0
    assert O.find_rotation_folding_pairs([]) == []
    assert O.find_rotation_folding_pairs([g("rx", target=0, angle=0.5), g("ry", target=0, angle=1.0)]) == []
    assert O.find_rotation_folding_pairs([g("rx", target=0, angle=0.5), g("rx", target=1, angle=1.0)]) == []
    ((ij, comb),) = O.find_rotation_folding_pairs([g("rx", target=0, angle=0.5), g("rx", target=0, angle=1.0)])
    assert ij == (0, 1) and comb == g("rx", target=0, angle=1.5)
    out = O.optimize_gates(C(1, g("rx", target=0, angle=0.3), g("rx", target=0, angle=0.4),
                             g("rx", target=0, angle=0.5), g("h", target=0)))
    assert out["operations"][0] == g("rx", target=0, angle=pytest.approx(1.2)) and types(out) == ["rx", "h"]


def test_qubit_usage():
    # gate_optimization_test.clj:382-418, qubit_optimization.clj
    c = O.optimize_gates(C(3, g("h", target=0), g("h", target=0), g("x", target=2), g("y", target=2)))
    c2, mapping = O.optimize_qubit_usage(c)
    assert c2["num-qubits"] == 1 and mapping == {2: 0}
    assert c2["operations"] == [g("x", target=0), g("y", target=0)]
    c3, _ = O.optimize_qubit_usage(O.optimize_gates(C(2, g("h", target=0), g("x", target=1))))
    assert c3["num-qubits"] == 2
    a = O.analyze_qubit_usage(C(5, g("cnot", control=1, target=3)))
    assert a["used-qubits"] == {1, 3} and a["unused-qubits"] == {0, 2, 4} and a["max-qubit-id"] == 3


def test_optimised_circuit_same_state_up_to_phase(oracle):
    """Folding S/T/phase into RZ changes only a global phase."""
    from qclojure_gb300 import workloads

    c = workloads.layered_circuit(6, 12, seed=9)
    opt = O.optimize_gates(c)
    assert len(opt["operations"]) <= len(c["operations"])
    a, b = oracle.run(c), oracle.run(opt)
    assert abs(abs(np.vdot(a, b)) - 1.0) <= 1e-12


def test_transform_circuit_cases():
    # circuit_transformation_test.clj:25-136
    c = C(2, g("h", target=0), g("t", target=1), g("cnot", control=0, target=1))
    r = O.transform_circuit(c, {"supported-operations": {"h", "x", "z", "rz", "cnot"}})
    assert set(types(r["circuit"])) <= {"h", "x", "z", "rz", "cnot"}
    assert r["circuit"]["operations"][1] == g("rz", target=1, angle=math.pi / 4)
    bell = C(2, g("h", target=0), g("cnot", control=0, target=1))
    r = O.transform_circuit(bell, {"supported-operations": {"h", "cnot"}})
    assert r["transformed-operation-count"] == 0 and r["unsupported-operations"] == [] and r["circuit"] == bell
    assert O.transform_circuit(C(1, g("t", target=0)), {"supported-operations": {"h"}},
                               {"transform-operations?": False})["circuit"] == C(1, g("t", target=0))
    r = O.transform_circuit(C(1, g("h", target=0)), {"supported-operations": set()})
    assert r["unsupported-operations"] == ["h"]
    r = O.transform_circuit(C(1), {"supported-operations": {"h"}})
    assert r["transformed-operation-count"] == 0 and r["unsupported-operations"] == []


def test_decomposition_rules():
    sup = {"h", "rz", "cnot", "t", "t-dag"}
    # toffoli: the 15-step CNOT+T form; cz through H-CNOT-H
    tof = O.decompose_operation(g("toffoli", control1=0, control2=1, target=2), sup)
    assert len(tof) == 15 and tof[1] == g("cnot", control=1, target=2) and tof[8] == g("t", target=1)
    assert O.decompose_operation(g("cz", control=0, target=1), sup) == \
        [g("h", target=1), g("cnot", control=0, target=1), g("h", target=1)]
    # fixed-angle gates through the parametric form when RZ is supported
    assert O.decompose_operation(g("s", target=0), sup) == [g("rz", target=0, angle=math.pi / 2)]
    assert O.decompose_operation(g("x", target=3), sup) == [g("ry", target=3, angle=math.pi)]
    # rotations through their universal form, keeping the angle
    assert O.decompose_operation(g("rx", target=0, angle=0.3), sup) == \
        [g("h", target=0), g("rz", target=0, angle=0.3), g("h", target=0)]
    # the phase gate's entry is a bare [:rz]: the angle is not carried over
    assert O.decompose_operation(g("phase", target=0, angle=0.3), sup) == [g("rz", target=0)]
    # SWAP's steps name target1/target2, which a SWAP operation does not have
    assert O.decompose_operation(g("swap", qubit1=0, qubit2=1), sup)[0] == g("cnot", control=None, target=None)
    # an operation without a usable decomposition stays, and is left alone afterwards
    assert O.decompose_operation(g("h", target=0), {"cnot"}) == [g("h", target=0)]
    assert O.transform_operations([g("h", target=0)] * 3, {"cnot"}) == [g("h", target=0)] * 3


def test_transform_iteration_limit():
    ops = [g("s", target=q % 4) for q in range(150)]
    with pytest.raises(O.OptimizationError, match="Maximum iterations"):
        O.transform_operations(ops, {"h", "rz", "cnot"}, 100)
    assert len(O.transform_operations(ops[:40], {"h", "rz", "cnot"}, 100)) == 40


def test_pipeline_on_submission_shapes():
    dev = {"native-gates": {"h", "cnot", "rz", "x"}}
    r = O.optimize(C(3, g("h", target=0), g("t", target=2), g("cnot", control=0, target=2)), dev)
    assert r["circuit"]["num-qubits"] == 2 and r["qubit-mapping"] == {0: 0, 2: 1}
    assert types(r["circuit"]) == ["h", "rz", "cnot"]
    # validation looks the supported set up on the context, where the pipeline never puts it
    assert r["all-gates-supported?"] is False and r["final-unsupported-gates"] == ["h", "rz", "cnot"]
    with pytest.raises(O.OptimizationError):
        O.optimize(C(1, g("h", target=0), g("h", target=0)), dev)


def test_reverse_mappings():
    # qubit_mapping.clj docstring examples and the lookup chain
    assert O.compose_mappings({0: 10, 1: 20}, {10: 100, 20: 200}) == {0: 100, 1: 200}
    assert O.invert_simple_mapping({0: 0, 2: 1, 4: 2}) == {0: 0, 1: 2, 2: 4}
    assert O.invert_vector_mapping({0: [0, 1, 2], 1: [3, 4, 5]}) == {0: 0, 1: 0, 2: 0, 3: 1, 4: 1, 5: 1}
    ctx = O.create_all_reverse_mappings({"qubit-mapping": {0: 0, 2: 1}, "logical-to-physical": {0: 5, 1: 7}})
    assert ctx["inverse-qubit-mapping"] == {0: 0, 1: 2} and ctx["physical-to-logical"] == {5: 0, 7: 1}
    assert O.map_measurements_to_original({5: 1, 7: 0, 9: 1}, ctx) == {0: 1, 2: 0}
    only_compaction = O.create_all_reverse_mappings({"qubit-mapping": {0: 0, 2: 1}})
    assert O.map_qubit_to_original(1, only_compaction) is None  # needs a physical-to-logical step
    r = O.optimize(C(3, g("h", target=0), g("x", target=2)), {"native-gates": {"h", "x"}})
    assert r["inverse-qubit-mapping"] == {0: 0, 1: 2}
