"""The QuantumBackend protocol on the GPU: job lifecycle, result maps, errors.

Mirrors test/org/soulspace/qclojure/adapter/backend/ideal_simulator_test.clj
(submission, status, results, convenience execution, cancellation, queue
status, not-found handling) against the GPU backend, plus batch submission.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_backend_info_and_device(sim):
    info = sim.backend_info()
    assert info["backend-type"] == "simulator"
    assert isinstance(info["backend-name"], str)
    assert "capabilities" in info and "max-qubits" in info
    assert sim.available() is True
    dev = sim.device()
    assert dev["num-qubits"] >= 33  # complex128 on one GB300
    assert "cnot" in dev["native-gates"]


def test_submission_status_and_result(sim):
    from qclojure_gb300 import circuit as qc

    jid = sim.submit_circuit(qc.bell_state_circuit(), {"result-specs": {"measurements": {"shots": 100}}})
    assert isinstance(jid, str)
    assert sim.job_status(jid) in ("queued", "running", "completed")
    assert sim.wait(jid, 10_000) == "completed"
    r = sim.job_result(jid)
    assert r["job-id"] == jid and r["job-status"] == "completed"
    res = r["results"]
    assert "measurement-results" in res
    freqs = res["measurement-results"]["frequencies"]
    assert set(freqs) == {0, 3}
    assert sum(freqs.values()) == 100
    assert res["circuit-metadata"] == {"circuit-depth": 2, "circuit-operation-count": 2, "circuit-gate-count": 2}
    assert res["result-types"] == {"measurements"}
    assert len(res["measurement-results"]["measurement-probabilities"]) == 4


def test_execute_circuit_convenience(sim):
    from qclojure_gb300 import circuit as qc
    from qclojure_gb300.backend import execute_circuit

    r = execute_circuit(sim, qc.bell_state_circuit(), {"result-specs": {"measurements": {"shots": 50}}})
    assert r["job-status"] == "completed"
    f = r["results"]["measurement-results"]["frequencies"]
    assert 0 in f and 3 in f


def test_all_result_types(sim, oracle):
    from qclojure_gb300 import workloads
    from qclojure_gb300.backend import execute_circuit

    n = 6
    c = workloads.layered_circuit(n, 4, seed=3)
    ref = oracle.run(c)
    ref2 = oracle.run(workloads.layered_circuit(n, 4, seed=4))
    pz = [[1, 0], [0, -1]]
    r = execute_circuit(sim, c, {"seed": 5, "result-specs": {
        "measurements": {"shots": 300},
        "expectation": {"observables": [pz, pz], "targets": [0, 5]},
        "variance": {"observables": [pz, pz], "targets": [0, 5]},
        "hamiltonian": [{"coefficient": 0.5, "pauli-string": "ZZIIXY"}, {"coefficient": -1.0, "pauli-string": "IIIIII"}],
        "probabilities": {"targets": [[0, 0, 0, 0, 0, 1], 7]},
        "amplitudes": {"basis-states": [0, 5, 63]},
        "state-vector": True,
        "density-matrix": True,
        "fidelity": {"references": [{"state-vector": ref, "num-qubits": n}, {"state-vector": ref2, "num-qubits": n}]},
    }})
    assert r["job-status"] == "completed", r
    res = r["results"]
    assert np.array_equal(np.asarray(res["final-state"]["state-vector"]), ref)
    assert np.array_equal(np.array(res["measurement-results"]["measurement-outcomes"], np.uint64),
                          oracle.sample(ref, 300, 5))
    e = [x["expectation-value"] for x in res["expectation-results"]]
    assert abs(e[0] - oracle.expectation_1q(ref, pz, 0)) <= 1e-12
    assert abs(e[1] - oracle.expectation_1q(ref, pz, 5)) <= 1e-12
    v = res["variance-results"][0]["variance-value"]
    assert abs(v - (1 - e[0] ** 2)) <= 1e-12
    eh = 0.5 * oracle.pauli_expectation(ref, "ZZIIXY") + -1.0 * oracle.pauli_expectation(ref, "IIIIII")
    assert abs(res["hamiltonian-result"]["energy-expectation"] - eh) <= 1e-12
    pr = res["probability-results"]["probability-outcomes"]
    assert abs(pr[(0, 0, 0, 0, 0, 1)] - abs(ref[1]) ** 2) <= 1e-15 and abs(pr[7] - abs(ref[7]) ** 2) <= 1e-15
    amps = res["amplitude-results"]["amplitude-values"]
    assert amps[63] == ref[63] and amps[5] == ref[5]
    rho = res["density-matrix-result"]["density-matrix"]
    assert np.max(np.abs(rho - np.outer(ref, ref.conj()))) <= 1e-15
    assert res["density-matrix-result"]["trace-valid"]
    f = res["fidelity-results"]["fidelities"]
    assert abs(f["reference-0"] - 1.0) <= 1e-12
    assert abs(f["reference-1"] - abs(oracle.inner(ref, ref2))) <= 1e-12


def test_failed_job_reports_error(sim):
    from qclojure_gb300.backend import execute_circuit

    # :i has no case in the reference dispatch; the encoder refuses it the same way
    from qclojure_gb300.circuit import CircuitError

    with pytest.raises(CircuitError):
        sim.submit_circuit({"num-qubits": 1, "operations": [{"operation-type": "i",
                                                              "operation-params": {"target": 0}}]})
    # an unnormalised initial state fails at sampling (state.clj:901-903)
    bad = np.zeros(2, np.complex128)
    bad[0] = 0.5
    r = execute_circuit(sim, {"num-qubits": 1, "operations": []},
                        {"initial-state": {"state-vector": bad}, "result-specs": {"measurements": {"shots": 10}}})
    assert r["job-status"] == "failed"
    assert "normalized" in r["error-message"]


def test_qubit_range_rejected(sim):
    from qclojure_gb300 import _abi as A

    with pytest.raises(A.QgError) as e:
        sim.submit_circuit({"num-qubits": 2, "operations": [{"operation-type": "h", "operation-params": {"target": 5}}]})
    assert e.value.code == A.QG_ERR_QUBIT_RANGE


def test_not_found_and_cancel(sim):
    from qclojure_gb300 import workloads

    assert sim.job_status("nope") == "not-found"
    assert sim.job_result("nope")["job-status"] == "not-found"
    assert sim.cancel_job("nope") == "not-found"
    # a long job followed by queued ones: cancel a queued job
    big = workloads.layered_circuit(27, 30, seed=1)
    ids = [sim.submit_circuit(big, {}) for _ in range(4)]
    outcomes = [sim.cancel_job(j) for j in ids[::-1]]
    assert set(outcomes) <= {"cancelled", "cannot-cancel"}
    for j in ids:
        assert sim.wait(j, 120_000) in ("completed", "cancelled"), sim.job_result(j)
    assert "cancelled" in {sim.job_status(j) for j in ids}
    done = [j for j in ids if sim.job_status(j) == "completed"]
    for j in done:
        assert sim.cancel_job(j) == "cannot-cancel"
    for j in ids:
        sim.free_job(j)


def test_queue_status_keys(sim):
    q = sim.queue_status()
    for k in ("total-jobs", "queued", "running", "completed", "backend-load", "estimated-wait-time",
              "hbm-free-bytes", "hbm-budget-bytes"):
        assert k in q


def test_batch_submit(sim, oracle):
    from qclojure_gb300 import workloads

    circs = [workloads.layered_circuit(n, 5, seed=n) for n in (4, 9, 12, 4, 9)]
    bid = sim.batch_submit(circs, {"result-specs": {"probabilities": {}}})
    for _ in range(200):
        if sim.batch_status(bid)["status"] == "completed":
            break
        time.sleep(0.05)
    st = sim.batch_status(bid)
    assert st["status"] == "completed" and st["total-jobs"] == 5
    res = sim.batch_results(bid)
    for c, (jid, r) in zip(circs, res.items()):
        assert r["job-status"] == "completed"
        p = r["results"]["probability-results"]["all-probabilities"]
        assert np.array_equal(p, oracle.probabilities(oracle.run(c)))


def test_concurrent_jobs_same_as_alone(sim, oracle):
    """Jobs overlapping on the device give the result they give alone."""
    from qclojure_gb300 import workloads

    circs = [workloads.layered_circuit(n, 12, seed=40 + n) for n in (8, 14, 18, 11, 16, 20, 8, 13)]
    ids = [sim.submit_circuit(c, {"seed": 9, "result-specs": {"measurements": {"shots": 2000}}}) for c in circs]
    for c, j in zip(circs, ids):
        assert sim.wait(j, 60_000) == "completed"
        r = sim.job_result(j)["results"]
        ref = oracle.run(c)
        assert np.array_equal(np.asarray(r["final-state"]["state-vector"]), ref)
        assert np.array_equal(np.array(r["measurement-results"]["measurement-outcomes"], np.uint64),
                              oracle.sample(ref, 2000, 9))
        sim.free_job(j)


def test_cleanup_completed(sim):
    from qclojure_gb300 import circuit as qc

    j = sim.submit_circuit(qc.bell_state_circuit(), {})
    sim.wait(j, 10_000)
    time.sleep(0.01)
    assert sim.cleanup_completed_jobs(0) >= 1
    assert sim.job_result(j)["job-status"] in ("not-found",)
