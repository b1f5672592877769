"""Serving: a mixed stream of jobs behind the job API with continuous batching.

Jobs of 5..12 qubits (one tile per state) are compiled by the worker that admits
them and run by the batcher, which groups everything ready by qubit count and
runs each group in one launch, one CTA per job. Larger jobs run concurrently on
the workers' streams.

Each job's result is the same alone and in the mix: the final state is bit-identical
and the shot outcomes are identical. Alone means submitted by itself, and also run
through the per-pass state API. The results are also within tolerance of the oracle:
complex128 ≤ 1e-12 per amplitude and outcomes identical; complex64 ≤ 2e-5 per amplitude.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stream(seed, count=36, cap=16):
    """Test-sized stream with the serving mix's shape: n = 8 + Geometric(0.15), capped;
    nine jobs in ten want shots, the tenth a Pauli-string expectation."""
    from qclojure_gb300 import workloads

    rng = np.random.default_rng(seed)
    jobs = []
    for i in range(count):
        n = int(min(8 + rng.geometric(0.15) - 1, cap))
        c = workloads.layered_circuit(n, int(rng.integers(2, 10)), seed=seed * 1000 + i)
        if i % 10 == 9:
            pauli = "".join("IXYZ"[k] for k in rng.integers(0, 4, n))
            spec = {"hamiltonian": [{"coefficient": 1.0, "pauli-string": pauli}], "state-vector": True}
        else:
            spec = SHOT_SPEC
        jobs.append((c, {"result-specs": spec}))
    return jobs


SHOT_SPEC = {"measurements": {"shots": 700}, "state-vector": True}


def _sv(r):
    return np.asarray(r["results"]["final-state"]["state-vector"])


@pytest.mark.parametrize("precision,arith,tol", [("c64", "exact", 2e-5), ("c128", "double-float", 1e-12),
                                                 ("c128", "exact", 0.0)])
def test_mix_equals_alone_and_oracle(oracle, precision, arith, tol):
    from qclojure_gb300.backend import create_simulator
    from qclojure_gb300.state import Context

    jobs = _stream(3)
    sim = create_simulator({"precision": precision, "fusion": "tiled", "workers": 4, "seed": 9,
                            "arithmetic": arith})
    ctx = Context(seed=9, arithmetic=arith)
    try:
        # the mix: shot jobs arrive together (one batch submission), the others right after
        shot = [k for k, (c, o) in enumerate(jobs) if o["result-specs"] is SHOT_SPEC]
        bid = sim.batch_submit([jobs[k][0] for k in shot], {"result-specs": SHOT_SPEC})
        ids = [None] * len(jobs)
        for k, jid in zip(shot, sim.batch_status(bid)["job-statuses"]):
            ids[k] = jid
        for k, (c, o) in enumerate(jobs):
            if ids[k] is None:
                ids[k] = sim.submit_circuit(c, o)
        for j in ids:
            assert sim.wait(j, 300_000) == "completed"
        mix = [sim.job_result(j) for j in ids]
        assert max(r["batched-with"] for r in mix) > 1, "no small jobs shared a launch"
        for (c, o), r in zip(jobs, mix):
            a_id = sim.submit_circuit(c, o)  # alone
            assert sim.wait(a_id, 300_000) == "completed"
            a = sim.job_result(a_id)
            assert np.array_equal(_sv(r), _sv(a))
            with ctx.state(c["num-qubits"], precision) as st:  # alone, per-pass kernels
                st.apply(c, fusion="tiled")
                assert np.array_equal(_sv(r), st.download())
            res, ares = r["results"], a["results"]
            ref = oracle.run(c)
            assert np.max(np.abs(_sv(r) - ref)) <= tol
            if "measurement-results" in res:
                assert res["measurement-results"]["measurement-outcomes"] == \
                    ares["measurement-results"]["measurement-outcomes"]
                if precision == "c128":
                    shots = len(res["measurement-results"]["measurement-outcomes"])
                    assert np.array_equal(np.array(res["measurement-results"]["measurement-outcomes"], np.uint64),
                                          oracle.sample(ref, shots, 9))
            else:
                e = res["hamiltonian-result"]["energy-expectation"]
                assert e == ares["hamiltonian-result"]["energy-expectation"]
                p = o["result-specs"]["hamiltonian"][0]["pauli-string"]
                assert abs(e - oracle.pauli_expectation(ref, p)) <= max(tol, 1e-12) * 10
            sim.free_job(r["job-id"])
            sim.free_job(a_id)
    finally:
        ctx.close()
        sim.close()


def test_served_c64_stream_tvd_against_oracle(oracle):
    """The served complex64 contract on a mixed stream that reaches 22 qubits: jobs of
    n = 8 + Geometric(0.15) qubits plus four of 20-22 qubits, nine in ten asking for shots
    and the tenth for a Pauli-string expectation, all submitted while earlier ones run.
    Every served job's outcome distribution is within TVD 1e-5 of the FP64 oracle's, its
    expectation within 1e-5, and its result equals the same job run alone."""
    from qclojure_gb300 import workloads
    from qclojure_gb300.backend import create_simulator

    jobs = _stream(5, count=26, cap=18)
    rng = np.random.default_rng(77)
    for i, n in enumerate((20, 21, 22, 20)):
        c = workloads.layered_circuit(n, int(rng.integers(3, 8)), seed=9000 + i)
        if i == 3:
            pauli = "".join("IXYZ"[k] for k in rng.integers(0, 4, n))
            spec = {"hamiltonian": [{"coefficient": 1.0, "pauli-string": pauli}], "state-vector": True}
        else:
            spec = SHOT_SPEC
        jobs.insert(3 + 6 * i, (c, {"result-specs": spec}))
    assert max(c["num-qubits"] for c, _ in jobs) >= 20
    sim = create_simulator({"precision": "c64", "fusion": "tiled", "workers": 4, "seed": 9})
    try:
        ids = [sim.submit_circuit(c, o) for c, o in jobs]
        for j in ids:
            assert sim.wait(j, 600_000) == "completed"
        for (c, o), jid in zip(jobs, ids):
            r = sim.job_result(jid)
            ref = oracle.run(c)
            sv = _sv(r)
            tvd = 0.5 * float(np.abs(np.abs(sv) ** 2 - np.abs(ref) ** 2).sum())
            assert tvd <= 1e-5, (c["num-qubits"], tvd)
            res = r["results"]
            if "hamiltonian-result" in res:
                p = o["result-specs"]["hamiltonian"][0]["pauli-string"]
                assert abs(res["hamiltonian-result"]["energy-expectation"] - oracle.pauli_expectation(ref, p)) <= 1e-5
            a_id = sim.submit_circuit(c, o)  # alone
            assert sim.wait(a_id, 600_000) == "completed"
            a = sim.job_result(a_id)
            assert np.array_equal(sv, _sv(a))
            if "measurement-results" in res:
                assert res["measurement-results"]["measurement-outcomes"] == \
                    a["results"]["measurement-results"]["measurement-outcomes"]
            sim.free_job(jid)
            sim.free_job(a_id)
    finally:
        sim.close()


def test_resident_loop_idles_out_and_restarts():
    """Small jobs run in a device-resident loop per qubit count. Its only waits are polls of
    the job ring, bounded by an idle budget: with nothing published (the tail word nothing
    raises) every loop kernel returns by itself within milliseconds, and the next job
    starts the loop again. The host reads the loops' state through qg_job_loop_info."""
    import ctypes as C
    import time

    from qclojure_gb300 import _abi as A
    from qclojure_gb300 import workloads
    from qclojure_gb300.backend import create_simulator

    sim = create_simulator({"precision": "c64", "fusion": "tiled", "workers": 2, "seed": 2,
                            "small-job-loop": "on"})

    def info():
        i = A.QgLoopInfo()
        assert sim._lib.qg_job_loop_info(sim._ctx, C.byref(i)) == 0
        return i

    try:
        ids = [sim.submit_circuit(workloads.layered_circuit(n, 4, seed=n), {}) for n in (8, 8, 10, 10, 10)]
        for j in ids:
            assert sim.wait(j, 60_000) == "completed"
        first = info()
        assert first.loops == 2 and first.launches >= 2 and first.jobs == 5
        deadline = time.time() + 2.0
        while info().running and time.time() < deadline:
            time.sleep(0.01)
        assert info().running == 0, "a loop kernel did not leave after its idle budget"
        j = sim.submit_circuit(workloads.layered_circuit(10, 3, seed=99), {})
        assert sim.wait(j, 60_000) == "completed"
        after = info()
        assert after.launches > first.launches and after.jobs == 6
    finally:
        sim.close()


@pytest.mark.parametrize("precision,arith", [("c64", "exact"), ("c128", "double-float"), ("c128", "exact")])
def test_resident_loop_equals_batcher(precision, arith):
    """The resident loop and the host batcher run the same op records per job: identical
    final states and shot outcomes."""
    from qclojure_gb300.backend import create_simulator

    jobs = [(c, o) for c, o in _stream(7, count=24, cap=12) if c["num-qubits"] <= 12]
    out = {}
    for mode in ("on", "off"):
        sim = create_simulator({"precision": precision, "fusion": "tiled", "workers": 2, "seed": 3,
                                "arithmetic": arith, "small-job-loop": mode})
        try:
            ids = [sim.submit_circuit(c, o) for c, o in jobs]
            res = []
            for j in ids:
                assert sim.wait(j, 120_000) == "completed"
                r = sim.job_result(j)
                res.append((_sv(r), r["results"].get("measurement-results", {}).get("measurement-outcomes")))
            out[mode] = res
        finally:
            sim.close()
    for (a, sa), (b, sb) in zip(out["on"], out["off"]):
        assert np.array_equal(a, b) and sa == sb


def test_cancel_small_job_waiting_in_queue():
    """A queued small job can be cancelled; the rest of its batch completes."""
    from qclojure_gb300 import workloads
    from qclojure_gb300.backend import create_simulator

    sim = create_simulator({"precision": "c64", "fusion": "tiled", "workers": 1, "seed": 1})
    try:
        big = sim.submit_circuit(workloads.layered_circuit(24, 30, seed=1), {})
        small = [sim.submit_circuit(workloads.layered_circuit(10, 5, seed=s), {}) for s in range(6)]
        assert sim.cancel_job(small[3]) in ("cancelled", "cannot-cancel")
        assert sim.wait(big, 300_000) == "completed"
        for k, j in enumerate(small):
            s = sim.wait(j, 300_000)
            assert s == "completed" or (k == 3 and s == "cancelled")
    finally:
        sim.close()
