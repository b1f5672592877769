"""Noisy trajectories on the GPU (qg_noisy_run) against the oracle's restatement of the
reference's shot loop: the same Kraus choices, final states within tolerance, identical
outcomes after readout noise; the hardware-simulator protocol mirror."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DEPOL = {"gate-noise": {"h": {"noise-type": "depolarizing", "noise-strength": 0.3},
                        "cnot": {"noise-type": "depolarizing", "noise-strength": 0.2},
                        "x": {"noise-type": "depolarizing", "noise-strength": 0.1}},
         "readout-error": {"prob-0-to-1": 0.05, "prob-1-to-0": 0.1, "correlated-errors": {0: {1: 3.0}, 2: {0: 0.5}}}}
MIXED = {"gate-noise": {"h": {"noise-type": "amplitude-damping", "noise-strength": 0.25},
                        "rx": {"noise-type": "phase-damping", "t1-time": 80.0, "t2-time": 40.0, "gate-time": 500.0},
                        "ry": {"noise-type": "coherent", "coherent-error": {"rotation-angle": 0.3, "rotation-axis": "x"}},
                        "rz": {"noise-type": "coherent", "coherent-error": {"rotation-angle": 0.2, "rotation-axis": "y"}},
                        "t": {"noise-type": "depolarizing", "noise-strength": 0.5},
                        "cnot": {"noise-type": "amplitude-damping", "t1-time": 50.0, "gate-time": 900.0},
                        "s": {"noise-type": "unknown-kind"}}}


def _bell(n):
    ops = [{"operation-type": "h", "operation-params": {"target": 0}}]
    ops += [{"operation-type": "cnot", "operation-params": {"control": q, "target": q + 1}} for q in range(n - 1)]
    return {"num-qubits": n, "operations": ops}


def _cases():
    from qclojure_gb300 import workloads

    return [("bell2-depol", _bell(2), DEPOL), ("ghz3-depol", _bell(3), DEPOL), ("one-qubit", _bell(1), DEPOL),
            ("layered6-mixed", workloads.layered_circuit(6, 5, seed=11), MIXED),
            ("layered13-depol", workloads.layered_circuit(13, 3, seed=12), DEPOL),
            ("layered9-mixed", workloads.layered_circuit(9, 6, seed=13), MIXED)]


@pytest.fixture(scope="module")
def contexts(built):
    from qclojure_gb300.state import Context

    ctxs = {"exact": Context(seed=1, arithmetic="exact"), "double-float": Context(seed=1, arithmetic="double-float")}
    yield ctxs
    for c in ctxs.values():
        c.close()


@pytest.mark.parametrize("arith", ["exact", "double-float"])
@pytest.mark.parametrize("name,circuit,noise", _cases(), ids=[c[0] for c in _cases()])
def test_trajectories_match_oracle(contexts, oracle, arith, name, circuit, noise):
    from qclojure_gb300.hardware import run_trajectories

    shots = 48 if circuit["num-qubits"] > 10 else 160
    run = run_trajectories(contexts[arith], circuit, noise, shots, seed=21, max_trajectories=shots)
    outs, states = oracle.noisy_shots(circuit, noise, shots, seed=21)
    assert np.max(np.abs(run["trajectories"] - states)) <= 1e-12
    assert np.array_equal(run["outcomes"], outs)
    assert np.max(np.abs(run["final_state"] - states[-1])) <= 1e-12
    assert run["stats"]["noise-sites"] == sum(
        1 for op in circuit["operations"] if op["operation-type"] in noise["gate-noise"]
        and noise["gate-noise"][op["operation-type"]]["noise-type"] != "unknown-kind")


def test_trajectories_complex64(contexts, oracle):
    from qclojure_gb300 import workloads
    from qclojure_gb300.hardware import run_trajectories

    c = workloads.layered_circuit(7, 5, seed=14)
    run = run_trajectories(contexts["exact"], c, MIXED, 200, seed=5, precision="c64", max_trajectories=200)
    outs, states = oracle.noisy_shots(c, MIXED, 200, seed=5)
    assert np.max(np.abs(run["trajectories"] - states)) <= 2e-5
    assert np.mean(run["outcomes"] == outs) >= 0.99


def test_many_shots_in_batches(contexts, oracle):
    """Shots beyond one batch continue the per-shot draws."""
    from qclojure_gb300.hardware import run_trajectories

    c = _bell(3)
    run = run_trajectories(contexts["double-float"], c, DEPOL, 3000, seed=8, max_trajectories=0)
    outs, _ = oracle.noisy_shots(c, DEPOL, 3000, seed=8)
    assert np.array_equal(run["outcomes"], outs)


def test_ghz_realistic_noise_statistics(contexts):
    """hardware_simulator_test.clj:48-67: realistic noise keeps most GHZ shots ideal."""
    from qclojure_gb300.hardware import run_trajectories

    nm = {"gate-noise": {"h": {"noise-type": "depolarizing", "noise-strength": 0.001},
                         "cnot": {"noise-type": "depolarizing", "noise-strength": 0.01}},
          "readout-error": {"prob-0-to-1": 0.01, "prob-1-to-0": 0.02}}
    run = run_trajectories(contexts["double-float"], _bell(3), nm, 1000, seed=99, max_trajectories=0)
    ideal = np.mean((run["outcomes"] == 0) | (run["outcomes"] == 7))
    assert 0.85 < ideal < 1.0


def test_noise_errors(contexts):
    from qclojure_gb300 import _abi as A
    from qclojure_gb300.hardware import run_trajectories

    bad = {"gate-noise": {"h": {"noise-type": "depolarizing", "noise-strength": 0.8}}}
    with pytest.raises(A.QgError, match="0.75"):
        run_trajectories(contexts["exact"], _bell(2), bad, 10, seed=1)
    zero_time = {"gate-noise": {"h": {"noise-type": "phase-damping", "t2-time": 150.0, "gate-time": 0.0}}}
    with pytest.raises(A.QgError, match="gate-time"):
        run_trajectories(contexts["exact"], _bell(2), zero_time, 10, seed=1)
    measured = {"num-qubits": 1, "operations": [
        {"operation-type": "h", "operation-params": {"target": 0}},
        {"operation-type": "measure", "operation-params": {"measurement-qubits": [0]}}]}
    with pytest.raises(A.QgError):
        run_trajectories(contexts["exact"], measured, DEPOL, 10, seed=1)
    # amplitude damping with gamma = 1 on |1>: the shot's state vanishes
    dead = {"gate-noise": {"x": {"noise-type": "amplitude-damping", "noise-strength": 1.0}}}
    one = {"num-qubits": 1, "operations": [{"operation-type": "x", "operation-params": {"target": 0}}]}
    with pytest.raises(A.QgError, match="normalized"):
        run_trajectories(contexts["exact"], one, dead, 4, seed=1)


def test_execute_circuit_and_protocol(built):
    from qclojure_gb300.hardware import create_hardware_simulator, execute_circuit

    r = execute_circuit(_bell(2), {"noise-model": DEPOL}, {"shots": 300, "result-specs": {
        "measurements": {}, "density-matrix": True, "probability": {}, "hamiltonian": {
            "hamiltonian": [{"coefficient": 1.0, "pauli-string": "ZZ"}]}}}, seed=3)
    assert r["job-status"] == "completed" and r["shots-executed"] == 300
    res = r["results"]
    assert sum(res["measurement-results"]["frequencies"].values()) == 300
    assert res["trajectory-count"] == 100
    assert res["density-matrix-result"]["trace"] == pytest.approx(1.0, abs=1e-12)
    rho = res["density-matrix"]
    zz = np.diag([1, -1, -1, 1]).astype(complex)
    assert res["hamiltonian-result"]["energy-expectation"] == pytest.approx(np.trace(rho @ zz).real, abs=1e-12)
    assert np.allclose(res["probability-results"]["probability-outcomes"], np.diag(rho).real)

    sim = create_hardware_simulator(device={"id": "test-device", "noise-model": DEPOL})
    try:
        assert sim.backend_info()["backend-type"] == "hardware-simulator"
        jid = sim.submit_circuit(_bell(1), {"shots": 100})
        assert sim.wait(jid, 60) == "completed"
        jr = sim.job_result(jid)
        assert jr["job-status"] == "completed" and jr["shots-executed"] == 100
        assert sum(jr["results"]["measurement-results"].values()) == 100
        empty = sim.submit_circuit({"num-qubits": 1, "operations": []}, {"shots": 10})
        assert sim.job_result(empty)["job-status"] == "failed"
        assert sim.job_status("fake-job-id") == "not-found"
        assert sim.job_result("fake-job-id")["job-status"] == "not-found"
        q = sim.queue_status()
        assert {"total-jobs", "active-jobs", "completed-jobs"} <= set(q)
    finally:
        sim.close()


def test_catalogue_device_noise_matches_oracle(contexts, oracle):
    """A device read from catalogue EDN, flat correlation rows included, runs its noisy
    shots as the oracle does."""
    from qclojure_gb300 import edn
    from qclojure_gb300.hardware import run_trajectories

    dev = edn.loads("""
      {:id :catalogue-test
       :noise-model {:gate-noise {:h {:noise-type :depolarizing :noise-strength 0.02}
                                  :cnot {:noise-type :amplitude-damping :noise-strength 0.01
                                         :t1-time 120.0 :t2-time 90.0 :gate-time 300.0}}
                     :readout-error {:prob-0-to-1 0.05 :prob-1-to-0 0.08
                                     :correlated-errors {0 1.0 1 1.2 2 0.8}}}}""")
    c = _bell(3)
    run = run_trajectories(contexts["exact"], c, dev["noise-model"], 200, seed=17, max_trajectories=200)
    outs, states = oracle.noisy_shots(c, dev["noise-model"], 200, seed=17)
    assert np.array_equal(run["outcomes"], outs)
    assert np.max(np.abs(run["trajectories"] - states)) <= 1e-12
