"""The variational client (batched objective, parameter-shift gradients, Adam and
gradient descent) against the same loops driven by the oracle's energies."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


class OracleObjective:
    """energies() from the oracle, one circuit at a time (the reference's evaluation)."""

    def __init__(self, oracle, hamiltonian, circuit_fn):
        self.oracle, self.h, self.f = oracle, hamiltonian, circuit_fn
        self.evaluations = 0

    def energies(self, params_list):
        out = []
        for p in params_list:
            s = self.oracle.run(self.f(list(p)))
            out.append(self.oracle.hamiltonian_expectation(s, self.h))
            self.evaluations += 1
        return np.array(out)


def _hea(n, layers):
    """Hardware-efficient ansatz: RY, RZ on every qubit, then a CNOT ladder, per layer."""
    def f(p):
        ops, k = [], 0
        for _ in range(layers):
            for q in range(n):
                ops.append({"operation-type": "ry", "operation-params": {"target": q, "angle": p[k]}})
                ops.append({"operation-type": "rz", "operation-params": {"target": q, "angle": p[k + 1]}})
                k += 2
            for q in range(n - 1):
                ops.append({"operation-type": "cnot", "operation-params": {"control": q, "target": q + 1}})
        return {"num-qubits": n, "operations": ops}
    return f


def _ham(n, seed):
    rng = np.random.default_rng(seed)
    terms = []
    for _ in range(8):
        s = "".join("IXYZ"[k] for k in rng.integers(0, 4, n))
        terms.append({"coefficient": float(rng.normal()), "pauli-string": s})
    terms.append({"coefficient": 0.7, "pauli-string": "Z" * n})
    return terms


@pytest.fixture(scope="module")
def vctx(built):
    from qclojure_gb300.state import Context

    c = Context(seed=1)
    yield c
    c.close()


@pytest.mark.parametrize("precision,arith,tol", [("c128", "double-float", 1e-10), ("c128", "exact", 1e-10),
                                                 ("c64", "exact", 2e-4)])
def test_parameter_shift_gradient(vctx, oracle, precision, arith, tol):
    from qclojure_gb300.variational import BatchedObjective, parameter_shift_gradient

    n, layers = 8, 2
    f, h = _hea(n, layers), _ham(n, 3)
    p = list(np.random.default_rng(4).uniform(-math.pi, math.pi, 2 * n * layers))
    gpu = BatchedObjective(vctx, h, f, precision, arith)
    try:
        g = parameter_shift_gradient(gpu, p)
        r = parameter_shift_gradient(OracleObjective(oracle, h, f), p)
        assert np.max(np.abs(g - r)) <= tol * max(1.0, np.max(np.abs(r)))
        # pi/2 shift: exact derivative of rotation gates; check against central differences
        g2 = parameter_shift_gradient(gpu, p, math.pi / 2)
        e0 = OracleObjective(oracle, h, f)
        fd = []
        for i in range(3):
            a, b = list(p), list(p)
            a[i] += 1e-5
            b[i] -= 1e-5
            ea, eb = e0.energies([a, b])
            fd.append((ea - eb) / 2e-5)
        assert np.allclose(g2[:3], fd, atol=max(1e-6, 50 * tol))
    finally:
        gpu.close()


def _qaoa(n, p, seed):
    from qclojure_gb300 import workloads
    from qclojure_gb300.variational import qaoa_maxcut_circuit

    w = workloads.qaoa_maxcut(n, p, seed)
    return (lambda prm: qaoa_maxcut_circuit(n, w["edges"], prm)), w["hamiltonian"], \
        [x for pair in zip(w["gammas"], w["betas"]) for x in pair]


@pytest.mark.parametrize("method", ["adam", "gradient-descent"])
def test_optimizer_matches_oracle_driven_loop(vctx, oracle, method):
    from qclojure_gb300 import variational as V

    f, h, p0 = _qaoa(8, 2, 5)
    opts = {"learning-rate": 0.05, "max-iterations": 12, "tolerance": 1e-9}
    run = V.adam_optimization if method == "adam" else V.gradient_descent_optimization
    gpu = V.BatchedObjective(vctx, h, f)
    try:
        a = run(gpu, p0, opts)
        b = run(OracleObjective(oracle, h, f), p0, opts)
        assert a["iterations"] == b["iterations"] and a["reason"] == b["reason"]
        # gradient descent is linear in the gradient: the loops agree to rounding. Adam's
        # first step is lr * g / (|g| + 1e-8) per component, so gradient differences of
        # 1e-13 move a component whose gradient is near zero by far more: 1e-5 / 1e-6.
        ptol, etol = (1e-9, 1e-10) if method == "gradient-descent" else (1e-5, 1e-6)
        assert np.max(np.abs(np.array(a["optimal-parameters"]) - b["optimal-parameters"])) <= ptol
        assert np.max(np.abs(np.array(a["convergence-history"]) - b["convergence-history"])) <= etol
        assert a["convergence-history"][-1] < a["convergence-history"][0]  # it descends
        assert gpu.batches == len(a["convergence-history"])  # one sweep per step
    finally:
        gpu.close()


def test_finite_difference_option(vctx, oracle):
    from qclojure_gb300 import variational as V

    f, h, p0 = _qaoa(6, 1, 9)
    gpu = V.BatchedObjective(vctx, h, f)
    try:
        e, g = V._energy_and_gradient(gpu, p0, {"gradient-method": "finite-difference", "gradient-step-size": 1e-4})
        e2, g2 = V._energy_and_gradient(OracleObjective(oracle, h, f), p0,
                                        {"gradient-method": "finite-difference", "gradient-step-size": 1e-4})
        assert abs(e - e2) <= 1e-11 and np.max(np.abs(g - g2)) <= 1e-7
    finally:
        gpu.close()


def test_adaptive_shift_gradient_and_spsa(vctx, oracle):
    """The adaptive-shift gradients and the SPSA loop on the device against the same
    calls on the oracle's energies (same seeded perturbations); 30 iterations stay below
    SPSA's 50-iteration convergence floor, so both runs take the same exit."""
    from qclojure_gb300.variational import (BatchedObjective, adaptive_parameter_shift_gradient,
                                            adaptive_shift_gradient, spsa_optimization)

    n, layers = 6, 1
    f, h = _hea(n, layers), _ham(n, 11)
    p = list(np.random.default_rng(6).uniform(-math.pi, math.pi, 2 * n * layers))
    gpu = BatchedObjective(vctx, h, f)
    ref = OracleObjective(oracle, h, f)
    try:
        g, r = adaptive_shift_gradient(gpu, p), adaptive_shift_gradient(ref, p)
        assert np.max(np.abs(g - r)) <= 1e-10 * max(1.0, np.max(np.abs(r)))
        types = ["rotation", "amplitude"] * n
        g, r = adaptive_parameter_shift_gradient(gpu, p, types), adaptive_parameter_shift_gradient(ref, p, types)
        assert np.max(np.abs(g - r)) <= 1e-10 * max(1.0, np.max(np.abs(r)))
        opts = {"max-iterations": 30, "seed": 2, "blocking-size": 3}
        a, b = spsa_optimization(gpu, p, opts), spsa_optimization(ref, p, opts)
        assert a["iterations"] == b["iterations"] == 30 and not a["success"] and not b["success"]
        assert np.max(np.abs(np.array(a["optimal-parameters"]) - b["optimal-parameters"])) <= 1e-8
        assert np.max(np.abs(np.array(a["convergence-history"]) - b["convergence-history"])) <= 1e-9
    finally:
        gpu.close()
