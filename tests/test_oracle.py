"""CPU tests of the oracle: pinned against the reference's known answers and
cross-checked with an independent dense Kronecker formulation."""
import math

import numpy as np
import pytest

from _kat import KAT, basis_state, check_case


class OracleEngine:
    def __init__(self, O):
        self.O = O

    def state(self, circuit, init, seed):
        return self.O.run(circuit, basis_state(circuit["num-qubits"], init), seed)

    def pauli(self, circuit, init, seed, p):
        return self.O.pauli_expectation(self.state(circuit, init, seed), p)

    def hamiltonian(self, circuit, init, seed, terms):
        return self.O.hamiltonian_expectation(self.state(circuit, init, seed),
                                              [{"coefficient": c, "pauli-string": s} for c, s in terms])

    def expectation(self, circuit, init, seed, obs, t):
        return self.O.expectation_1q(self.state(circuit, init, seed), obs, t)

    def variance(self, circuit, init, seed, obs, t):
        s = self.state(circuit, init, seed)
        o = np.array(obs)
        e = self.O.expectation_1q(s, obs, t)
        return self.O.expectation_1q(s, (o @ o).tolist(), t) - e * e

    def counts(self, circuit, init, seed, shots):
        out = self.O.sample(self.state(circuit, init, seed), shots, seed)
        vals, cnt = np.unique(out, return_counts=True)
        return {int(v): int(c) for v, c in zip(vals, cnt)}


@pytest.mark.parametrize("case", KAT, ids=[c["name"] for c in KAT])
def test_oracle_reference_kat(oracle, case):
    check_case(case, OracleEngine(oracle))


def test_philox_published_vectors(oracle):
    # Random123 known-answer vectors for philox4x32-10
    assert oracle.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert oracle.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert oracle.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def _kron_gate(n, q, g):
    m = np.array([[1.0]], dtype=np.complex128)
    for k in range(n):
        m = np.kron(m, g if k == q else np.eye(2))
    return m


@pytest.mark.parametrize("seed", range(4))
def test_oracle_matches_dense_kronecker(oracle, seed):
    """The reference's own algorithm (gate.clj:346-395) in numpy agrees to rounding."""
    from qclojure_gb300 import workloads

    n = 5
    c = workloads.layered_circuit(n, 6, seed)
    s = np.zeros(1 << n, np.complex128)
    s[0] = 1
    for op in c["operations"]:
        p = op["operation-params"]
        t = op["operation-type"]
        if t == "cnot":
            ctl, tgt = p["control"], p["target"]
            new = s.copy()
            for i in range(1 << n):
                if (i >> (n - 1 - ctl)) & 1:
                    new[i] = s[i ^ (1 << (n - 1 - tgt))]
            s = new
            continue
        a = p.get("angle", 0.0)
        mats = {
            "h": np.array([[1, 1], [1, -1]]) / math.sqrt(2), "x": np.array([[0, 1], [1, 0]]),
            "y": np.array([[0, -1j], [1j, 0]]), "z": np.diag([1, -1]), "s": np.diag([1, 1j]),
            "t": np.diag([1, np.exp(1j * math.pi / 4)]),
            "rx": np.array([[math.cos(a / 2), -1j * math.sin(a / 2)], [-1j * math.sin(a / 2), math.cos(a / 2)]]),
            "ry": np.array([[math.cos(a / 2), -math.sin(a / 2)], [math.sin(a / 2), math.cos(a / 2)]]),
            "rz": np.diag([np.exp(-0.5j * a), np.exp(0.5j * a)]),
        }
        s = _kron_gate(n, p["target"], mats[t].astype(np.complex128)) @ s
    assert np.max(np.abs(oracle.run(c) - s)) < 1e-13


def test_refalgo_rows_match_gate(oracle):
    rng = np.random.default_rng(0)
    n = 6
    x = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    g = [[0.3 + 0.1j, -0.2], [0.5j, 0.9]]
    y = oracle.refalgo_rows(x, g, 2, 0, 1 << n)
    assert np.allclose(y, _kron_gate(n, 2, np.array(g)) @ x, atol=1e-13)


def test_refalgo_circuit_is_the_oracle_bit_for_bit(oracle):
    """The whole-circuit reference algorithm (dense Kronecker row sums, zeros included)
    leaves the oracle's final state exactly: the row adds exact zeros around the two
    non-zero products in ascending column order (gate.clj:384-395). Its shots follow the
    probabilities (state.clj:897-911)."""
    from qclojure_gb300 import workloads

    for n, depth, seed in ((6, 10, 1), (8, 4, 2)):
        c = workloads.layered_circuit(n, depth, seed)
        s, shots = oracle.refalgo_circuit(c, 2000, seed=5)
        assert np.array_equal(s, oracle.run(c))
        counts = np.bincount(shots.astype(np.int64), minlength=1 << n) / 2000.0
        assert 0.5 * np.abs(counts - oracle.probabilities(s)).sum() < 0.12


def test_controlled_gate_transpose_quirk(oracle):
    """gate.clj:473-483 applies G^T: controlled RY(t) acts as RY(-t) on the target."""
    th = 0.7
    c = {"num-qubits": 2, "operations": [
        {"operation-type": "x", "operation-params": {"target": 0}},
        {"operation-type": "cry", "operation-params": {"control": 0, "target": 1, "angle": th}}]}
    s = oracle.run(c)
    assert abs(s[2] - math.cos(th / 2)) < 1e-15 and abs(s[3] - (-math.sin(th / 2))) < 1e-15


def test_swap_uses_lsb_positions(oracle):
    """gate.clj:768-778: SWAP qubit indices are bit positions from the LSB."""
    c = {"num-qubits": 3, "operations": [
        {"operation-type": "x", "operation-params": {"target": 0}},          # |100> = index 4
        {"operation-type": "swap", "operation-params": {"qubit1": 0, "qubit2": 2}}]}
    s = oracle.run(c)
    assert s[1] == 1  # bits 0 and 2 exchanged: 100 -> 001


def test_unknown_and_identity_fail_like_reference(oracle):
    from qclojure_gb300.circuit import CircuitError

    for t in ("i", "cy", "bogus"):
        with pytest.raises((CircuitError, ValueError)):
            oracle.run({"num-qubits": 2, "operations": [{"operation-type": t, "operation-params": {"target": 0,
                                                                                                 "control": 1}}]})


def test_sampling_rule_first_cumulative_above_draw(oracle):
    s = np.zeros(4, np.complex128)
    s[1] = math.sqrt(0.25)
    s[3] = math.sqrt(0.75)
    out = oracle.sample(s, 2000, 5)
    assert set(np.unique(out)) <= {1, 3}
    assert 0.2 < np.mean(out == 1) < 0.3


def test_sampling_rejects_unnormalized(oracle):
    s = np.zeros(2, np.complex128)
    s[0] = 0.9
    with pytest.raises(ValueError):
        oracle.sample(s, 10, 1)
