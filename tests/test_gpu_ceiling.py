"""Memory ceiling: 33-qubit complex128 and 34-qubit complex64 states (128 GiB each),
gates in place, then 10^6 shots. Beyond the oracle's reach, so the checks are
properties: a circuit followed by its inverse returns |0...0>, a GHZ state
samples only its two basis states in equal proportion.

Tolerances: complex128 (double-float) |<Z...Z> - 1| <= 1e-10; complex64 <= 1e-4.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inverse(circuit):
    inv = {"s": "s-dag", "s-dag": "s", "t": "t-dag", "t-dag": "t"}
    ops = []
    for op in reversed(circuit["operations"]):
        t = op["operation-type"]
        p = dict(op.get("operation-params") or {})
        if t in ("rx", "ry", "rz", "phase", "rydberg-cphase", "crz", "crx", "cry", "rzz"):
            p["angle"] = -p["angle"]
        ops.append({"operation-type": inv.get(t, t), "operation-params": p})
    return {"num-qubits": circuit["num-qubits"], "operations": ops}


def _ghz(n):
    ops = [{"operation-type": "h", "operation-params": {"target": 0}}]
    ops += [{"operation-type": "cnot", "operation-params": {"control": q, "target": q + 1}} for q in range(n - 1)]
    return {"num-qubits": n, "operations": ops}


@pytest.mark.parametrize("n,precision,tol", [(33, "c128", 1e-10), (34, "c64", 1e-4)])
def test_ceiling_circuit_then_inverse(gpu_ctx_df, n, precision, tol):
    from qclojure_gb300 import workloads

    c = workloads.ceiling_circuit(n, 2, seed=n)
    with gpu_ctx_df.state(n, precision) as st:
        st.apply(c, fusion="tiled")
        st.apply(_inverse(c), fusion="tiled")
        assert abs(st.pauli_expectation("Z" * n) - 1.0) <= tol
        assert np.all(st.sample(1000, 5) == 0)


@pytest.mark.parametrize("n,precision", [(33, "c128"), (34, "c64")])
def test_ceiling_ghz_million_shots(gpu_ctx_df, n, precision):
    with gpu_ctx_df.state(n, precision) as st:
        st.apply(_ghz(n), fusion="tiled")
        shots = st.sample(1_000_000, 11)
        top = (1 << n) - 1
        assert np.all((shots == 0) | (shots == top))
        frac = float(np.mean(shots == top))
        assert abs(frac - 0.5) <= 0.005  # binomial sigma 5e-4
