"""The optimised CPU state-vector baseline (oracle/cpu_sv.c) computes the oracle's states:
it is only a benchmark figure, but the figure must be for the same computation."""
import numpy as np
import pytest


def test_cpu_sv_matches_oracle(oracle):
    from qclojure_gb300 import workloads

    if oracle.cpu_sv_lib() is None:
        pytest.skip("the CPU baseline could not be built here")
    for c in (workloads.large_circuit(8, 6, seed=3), workloads.layered_circuit(11, 10, seed=4),
              workloads.qft_circuit(9)):
        assert np.max(np.abs(oracle.cpu_sv_run(c) - oracle.run(c))) <= 1e-12
    with pytest.raises(ValueError):
        oracle.cpu_sv_run({"num-qubits": 3, "operations": [
            {"operation-type": "toffoli", "operation-params": {"control1": 0, "control2": 1, "target": 2}}]})
