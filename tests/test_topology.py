"""Topologies and topology-aware routing (qclojure_gb300.topology) with the cases of
the reference's topology tests (test/org/soulspace/qclojure/application/topology_test.clj)
restated. CPU only."""
import pytest

from qclojure_gb300 import topology as T


def g(t, **p):
    return {"operation-type": t, "operation-params": p}


def C(n, *ops):
    return {"num-qubits": n, "operations": list(ops)}


def test_couplings():
    # topology_test.clj:30-83
    assert T.linear_coupling(4) == [[1], [0, 2], [1, 3], [2]]
    assert T.ring_coupling(4) == [[3, 1], [0, 2], [1, 3], [2, 0]]
    assert T.star_coupling(4) == [[1, 2, 3], [0], [0], [0]]
    assert T.grid_coupling(2, 2) == [[2, 1], [3, 0], [0, 3], [1, 2]]
    hh = T.heavy_hex_coupling(7)
    assert len(hh) == 7 and T.validate_coupling(hh)
    with pytest.raises(T.TopologyError):
        T.heavy_hex_coupling(0)
    assert T.linear_coupling(1) == [[]] and T.ring_coupling(1) == [[]] and T.star_coupling(1) == [[]]
    assert T.coupling_for_topology("all-to-all", 3) == [[1, 2], [0, 2], [0, 1]]
    assert T.coupling_for_topology("grid", 6) == T.grid_coupling(2, 3)
    with pytest.raises(T.TopologyError):
        T.coupling_for_topology("moebius", 4)


def test_validation_and_analysis():
    # topology_test.clj:85-160
    assert T.validate_coupling([[1], [0]]) and T.validate_coupling([[1, 2], [0], [0]])
    assert not T.validate_coupling([[0, 1], [0]]) and not T.validate_coupling([[1], []])
    a = T.analyze_coupling_connectivity(T.linear_coupling(4))
    assert (a["num-qubits"], a["total-edges"], a["max-degree"], a["min-degree"], a["is-connected"]) == (4, 3, 2, 1, True)
    a = T.analyze_coupling_connectivity(T.star_coupling(4))
    assert (a["total-edges"], a["max-degree"], a["min-degree"]) == (3, 3, 1)
    assert not T.analyze_coupling_connectivity([[1], [0], [], []])["is-connected"]
    a = T.analyze_coupling_connectivity([[]])
    assert (a["num-qubits"], a["total-edges"], a["max-degree"], a["is-connected"]) == (1, 0, 0, True)
    assert T.analyze_coupling_connectivity([])["num-qubits"] == 0
    info = T.get_coupling_info(T.star_coupling(5), "Star-5")
    assert "Star-5" in info and "Qubits: 5" in info and "degree:" in info
    assert "Connected: true" in T.get_coupling_info(T.linear_coupling(4), "Linear-4")
    assert "∞ (disconnected)" in T.get_coupling_info([[1], [0], [], []], "Disconnected")


def test_distances_and_paths():
    # topology_test.clj:190-250
    d = T.calculate_distance_matrix(T.linear_coupling(4))
    assert (d[0][0], d[0][1], d[0][2], d[0][3], d[1][3]) == (0, 1, 2, 3, 2)
    d = T.calculate_distance_matrix(T.star_coupling(4))
    assert (d[1][2], d[2][3]) == (2, 2)
    d = T.calculate_distance_matrix(T.ring_coupling(4))
    assert (d[0][2], d[0][3]) == (2, 1)
    assert T.find_shortest_path(T.linear_coupling(4), 0, 3) == [0, 1, 2, 3]
    assert T.find_shortest_path(T.star_coupling(4), 1, 2) == [1, 0, 2]
    assert T.find_shortest_path(T.linear_coupling(3), 1, 1) == [1]
    assert T.generate_swap_operations([0, 1], 0) == [] and T.generate_swap_operations([0], 0) == []
    sw = T.generate_swap_operations([0, 1, 2, 3], 0)
    assert len(sw) == 3 and all(s["operation-type"] == "swap" for s in sw)
    assert T.calculate_distance_matrix([[1], [0], [], []])[0][2] == T.INT_MAX


def test_mapping_and_routing():
    # topology_test.clj:255-335
    c = C(3, g("h", target=0), g("cnot", control=0, target=2))
    lin = [[1], [0, 2], [1]]
    dist = T.calculate_distance_matrix(lin)
    m = T.find_optimal_mapping(c, lin, dist)
    assert len(m) == 3 and 0 in m and 2 in m
    assert len(T.find_optimal_mapping(C(2, g("cnot", control=0, target=1)), T.linear_coupling(5),
                                      T.calculate_distance_matrix(T.linear_coupling(5)))) == 2
    with pytest.raises(T.TopologyError):
        T.find_optimal_mapping(C(4, g("h", target=0)), lin, dist)
    r = T.optimize_for_coupling(c, lin)
    # offset 1 maps 0 -> 1 and 2 -> 0, adjacent on the line: cost 1, no SWAP
    assert r["logical-to-physical"] == {0: 1, 1: 2, 2: 0} and r["swap-count"] == 0 and r["total-cost"] == 1
    assert r["circuit"]["operations"] == [g("h", target=1), g("cnot", control=1, target=0)]
    # a triangle of CNOTs costs 4 under every offset: the identity stays and 0 -> 2 is routed
    tri = C(3, g("cnot", control=0, target=1), g("crz", control=1, target=2, angle=0.5),
            g("cnot", control=0, target=2))
    r = T.optimize_for_coupling(tri, lin)
    assert r["logical-to-physical"] == {0: 0, 1: 1, 2: 2} and r["swap-count"] == 1 and r["total-cost"] == 4
    assert [o["operation-type"] for o in r["circuit"]["operations"]] == ["cnot", "crz", "swap", "cnot"]
    assert r["circuit"]["operations"][1]["operation-params"] == {"control": 1, "target": 2}  # the angle is dropped
    assert r["circuit"]["operations"][3]["operation-params"] == {"control": 1, "target": 2}
    assert "SWAP operations added: 1" in r["topology-summary"]
    r = T.optimize_for_coupling(C(2, g("h", target=0), g("cnot", control=0, target=1)), T.linear_coupling(2),
                                {"insert-swaps?": False})
    assert r["swap-count"] == 0
    cmp = T.compare_couplings(C(3, g("cnot", control=0, target=2)),
                              {"linear": T.linear_coupling(3), "star": T.star_coupling(3), "ring": T.ring_coupling(3)})
    assert len(cmp) == 3 and [x["total-cost"] for x in cmp] == sorted(x["total-cost"] for x in cmp)


def test_topology_stage_in_pipeline():
    from qclojure_gb300 import optimization as O

    c = C(3, g("cnot", control=0, target=1), g("cnot", control=1, target=2), g("cnot", control=0, target=2),
          g("x", target=1))
    dev = {"supported-operations": {"h", "x", "cnot"}, "coupling": [[1], [0, 2], [1]]}
    r = O.optimize(c, dev, {"optimize-topology?": True})
    assert r["swap-count"] == 1 and "swap" not in [o["operation-type"] for o in r["circuit"]["operations"]]
    assert r["physical-to-logical"] == {0: 0, 1: 1, 2: 2}
    # with a native SWAP the routing result replaces the context (device and options are gone)
    dev2 = {"supported-operations": {"h", "x", "cnot", "swap"}, "coupling": [[1], [0, 2], [1]]}
    r2 = O.optimize(c, dev2, {"optimize-topology?": True})
    assert "device" not in r2 and r2["swap-count"] == 1
