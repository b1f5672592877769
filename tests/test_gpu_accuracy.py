"""Per-result accuracy (result spec "accuracy"): the job's final state against the same
circuit run again in complex128 with exact FP64 arithmetic in the reference's gate order
(the path that equals the oracle bit for bit). The reported max amplitude error,
1 - fidelity and probability TVD must be the distances of the returned state from the
oracle's, computed here on the host.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,arith", [("c64", "exact"), ("c128", "double-float"), ("c128", "exact")])
@pytest.mark.parametrize("n", [9, 16])
def test_accuracy_result_matches_oracle_distance(oracle, precision, arith, n):
    from qclojure_gb300 import workloads
    from qclojure_gb300.backend import create_simulator

    c = workloads.layered_circuit(n, 12, seed=40 + n)
    sim = create_simulator({"precision": precision, "fusion": "tiled", "workers": 2, "seed": 3, "arithmetic": arith})
    try:
        jid = sim.submit_circuit(c, {"result-specs": {"accuracy": True, "state-vector": True}})
        assert sim.wait(jid, 120_000) == "completed"
        r = sim.job_result(jid)
        acc = r["results"]["accuracy-results"]
        sv = np.asarray(r["results"]["final-state"]["state-vector"])
        ref = oracle.run(c)
        d = np.max(np.abs(sv - ref))
        tvd = 0.5 * np.abs(np.abs(sv) ** 2 - np.abs(ref) ** 2).sum()
        assert abs(acc["max-amplitude-error"] - d) <= 1e-15 + 1e-9 * d, (acc, d)
        assert abs(acc["probability-tvd"] - tvd) <= 1e-14 + 1e-6 * tvd, (acc, tvd)
        assert 0.0 <= acc["one-minus-fidelity"] <= 1e-8
        if precision == "c128" and arith == "exact":
            assert acc["max-amplitude-error"] == 0.0 and acc["probability-tvd"] == 0.0
        elif precision == "c128":
            assert acc["max-amplitude-error"] <= 1e-12
        else:
            assert acc["probability-tvd"] <= 1e-5
    finally:
        sim.close()
