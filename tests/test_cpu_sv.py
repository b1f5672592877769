"""The optimised CPU state-vector baseline (oracle/cpu_sv.c) computes the oracle's states
bit for bit: it is a benchmark figure and the 30-qubit spot check of the GPU's result in
bench.py, so it must be the same computation, rounding for rounding."""
import math

import numpy as np
import pytest

# every gate cpu_sv implements, with the operand names of the reference's op maps
ONE_Q = ("x", "y", "z", "h", "s", "s-dag", "t", "t-dag")
ONE_Q_ANGLE = ("rx", "ry", "rz", "phase")
CONTROLLED = ("cnot", "cz")  # :cy is refused like the reference refuses it
CONTROLLED_ANGLE = ("crx", "cry", "crz")


def _random_circuit(n: int, count: int, seed: int) -> dict:
    rng = np.random.default_rng(seed)
    ops = []
    kinds = ONE_Q + ONE_Q_ANGLE + CONTROLLED + CONTROLLED_ANGLE + ("rydberg-cz", "rydberg-cphase", "swap")
    for _ in range(count):
        g = kinds[rng.integers(len(kinds))]
        a, b = (int(x) for x in rng.choice(n, 2, replace=False))
        ang = float(rng.uniform(0, 2 * math.pi))
        if g in ONE_Q:
            p = {"target": a}
        elif g in ONE_Q_ANGLE:
            p = {"target": a, "angle": ang}
        elif g in CONTROLLED or g == "rydberg-cz":
            p = {"control": a, "target": b}
        elif g == "swap":
            p = {"qubit1": a, "qubit2": b}
        else:
            p = {"control": a, "target": b, "angle": ang}
        ops.append({"operation-type": g, "operation-params": p})
    return {"num-qubits": n, "operations": ops}


def test_cpu_sv_bit_identical_to_oracle(oracle):
    from qclojure_gb300 import workloads

    if oracle.cpu_sv_lib() is None:
        pytest.skip("the CPU baseline could not be built here")
    cases = [workloads.large_circuit(8, 6, seed=3), workloads.layered_circuit(11, 10, seed=4),
             workloads.qft_circuit(9)] + [_random_circuit(n, 400, seed=n) for n in (3, 7, 12)]
    for c in cases:
        got, want = oracle.cpu_sv_run(c), oracle.run(c)
        assert np.array_equal(got, want), (c.get("name"), float(np.max(np.abs(got - want))))


def test_cpu_sv_refuses_what_it_lacks(oracle):
    if oracle.cpu_sv_lib() is None:
        pytest.skip("the CPU baseline could not be built here")
    with pytest.raises(ValueError):
        oracle.cpu_sv_run({"num-qubits": 3, "operations": [
            {"operation-type": "toffoli", "operation-params": {"control1": 0, "control2": 1, "target": 2}}]})
