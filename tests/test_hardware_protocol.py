"""The hardware simulator's job protocol (qclojure_gb300.hardware.HardwareSimulator) on
the CPU, with the device execution stubbed: submission through the optimisation
pipeline, job states, failures, cancellation, queue status (hardware_simulator.clj:262-395,
hardware_simulator_test.clj:70-149)."""
import threading

import pytest


@pytest.fixture
def sim(monkeypatch):
    from qclojure_gb300 import hardware as H
    from qclojure_gb300 import state

    class FakeContext:
        def __init__(self, *a, **k):
            pass

        def close(self):
            pass

    gate = threading.Event()
    calls = []

    def fake_execute(circuit, device, options, ctx=None, seed=None):
        gate.wait(10)
        calls.append(circuit)
        return {"job-status": "completed", "circuit": circuit, "shots-executed": options.get("shots", 1024),
                "results": {"measurement-results": {"0": options.get("shots", 1024)}}}

    monkeypatch.setattr(state, "Context", FakeContext)
    monkeypatch.setattr(H, "execute_circuit", fake_execute)
    s = H.create_hardware_simulator(device={"id": "dev", "noise-model": {}, "native-gates": {"h", "cnot", "x"}})
    s.gate, s.calls = gate, calls
    yield s
    gate.set()
    s.close()


def _bell():
    return {"num-qubits": 2, "operations": [{"operation-type": "h", "operation-params": {"target": 0}},
                                            {"operation-type": "cnot", "operation-params": {"control": 0, "target": 1}}]}


def test_submit_run_and_result(sim):
    jid = sim.submit_circuit(_bell(), {"shots": 10})
    assert sim.job_status(jid) in ("queued", "running")
    sim.gate.set()
    assert sim.wait(jid, 10) == "completed"
    r = sim.job_result(jid)
    assert r["job-status"] == "completed" and r["job-id"] == jid and r["shots-executed"] == 10
    assert sim.calls == [_bell()]  # the original circuit runs, not the optimised one
    q = sim.queue_status()
    assert q["total-jobs"] == 1 and q["completed-jobs"] == 1 and q["active-jobs"] == 0


def test_pipeline_failures_fail_the_job(sim):
    empty = sim.submit_circuit({"num-qubits": 1, "operations": []}, {"shots": 10})
    hh = sim.submit_circuit({"num-qubits": 1, "operations": [{"operation-type": "h", "operation-params": {"target": 0}}] * 2})
    many = sim.submit_circuit({"num-qubits": 1, "operations": [
        {"operation-type": "s", "operation-params": {"target": 0}}, {"operation-type": "x", "operation-params": {"target": 0}}] * 120})
    for jid, msg in ((empty, "empty circuit"), (hh, "empty circuit"), (many, "Maximum iterations")):
        r = sim.job_result(jid)
        assert sim.job_status(jid) == "failed" and r["job-status"] == "failed" and msg in r["error-message"]


def test_cancel_and_not_found(sim):
    a = sim.submit_circuit(_bell(), {"shots": 1})
    b = sim.submit_circuit(_bell(), {"shots": 1})
    assert sim.cancel_job(b) == "cancelled" and sim.job_status(b) == "cancelled"
    sim.gate.set()
    assert sim.wait(a, 10) == "completed"
    assert sim.cancel_job(a) == "already-completed"
    assert sim.cancel_job("nope") == "not-found"
    assert sim.job_status("fake-job-id") == "not-found"
    assert sim.job_result("fake-job-id")["job-status"] == "not-found"
    assert sim.backend_info()["backend-type"] == "hardware-simulator" and sim.available()
    assert sim.select_device("dev")["id"] == "dev"


def test_submission_runs_error_correction(sim):
    """Every submitted option reaches the pipeline (`merge` over its defaults): error
    correction encodes the circuit there, the original circuit runs, and an unknown code
    fails the job."""
    ok = sim.submit_circuit(_bell(), {"shots": 5, "apply-error-correction?": True, "error-correction-code": "shor"})
    bad = sim.submit_circuit(_bell(), {"apply-error-correction?": True, "error-correction-code": "nope"})
    r = sim.job_result(bad)
    assert r["job-status"] == "failed" and "Unknown error correction code" in r["error-message"]
    sim.gate.set()
    assert sim.wait(ok, 10) == "completed" and sim.calls == [_bell()]
