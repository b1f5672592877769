"""GPU parity: the sm_103a kernels against the CPU oracle, through the C ABI.

Tolerances (stated per test):
  complex128 plain and tiled executors  bit-exact amplitudes (same rounded products as the oracle)
  complex128 dense fused blocks         max |d amp| <= 1e-12 (FMA inside the block product)
  complex64                             max |d amp| <= 2e-5, probability TVD <= 1e-5
  reductions (Pauli, observables)       |d| <= 1e-12
  sampled outcomes                      identical to the oracle's for the same seed
"""
import math

import numpy as np
import pytest

from _kat import KAT, basis_state, check_case

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


def every_gate_circuit(n, seed):
    rng = np.random.default_rng(seed)
    ops = []

    def q(k=1):
        return [int(x) for x in rng.choice(n, size=k, replace=False)]

    def a():
        return float(rng.uniform(-2 * math.pi, 2 * math.pi))

    for rep in range(3):
        for g in ("h", "x", "y", "z", "s", "s-dag", "t", "t-dag"):
            ops.append({"operation-type": g, "operation-params": {"target": q()[0]}})
        for g in ("rx", "ry", "rz", "phase"):
            ops.append({"operation-type": g, "operation-params": {"target": q()[0], "angle": a()}})
        for g in ("cnot", "cz"):
            c, t = q(2)
            ops.append({"operation-type": g, "operation-params": {"control": c, "target": t}})
        for g in ("crx", "cry", "crz", "rydberg-cphase"):
            c, t = q(2)
            ops.append({"operation-type": g, "operation-params": {"control": c, "target": t, "angle": a()}})
        c, t = q(2)
        ops.append({"operation-type": "rydberg-cz", "operation-params": {"control": c, "target": t}})
        c, t = q(2)
        ops.append({"operation-type": "controlled",
                    "operation-params": {"control-qubits": [c], "target-gate": "y", "target-qubits": [t]}})
        for g in ("swap", "iswap"):
            a1, b1 = q(2)
            ops.append({"operation-type": g, "operation-params": {"qubit1": a1, "qubit2": b1}})
        c1, c2, t = q(3)
        ops.append({"operation-type": "toffoli", "operation-params": {"control1": c1, "control2": c2, "target": t}})
        c, t1, t2 = q(3)
        ops.append({"operation-type": "fredkin", "operation-params": {"control": c, "target1": t1, "target2": t2}})
        ops.append({"operation-type": "rydberg-blockade",
                    "operation-params": {"qubit-indices": q(min(n, 4)), "angle": a()}})
        a1, b1 = q(2)
        ops.append({"operation-type": "rzz", "operation-params": {"qubit1": a1, "qubit2": b1, "angle": a()}})
        ops.append({"operation-type": ("global-rx", "global-ry", "global-rz", "global-h")[rep % 4],
                    "operation-params": {"angle": a()}})
        ops.append({"operation-type": ("global-x", "global-y", "global-z")[rep % 3]})
    return {"num-qubits": n, "operations": ops}


@pytest.fixture(scope="module")
def states(gpu_ctx):
    cache = {}

    def get(n, precision="c128"):
        key = (n, precision)
        if key not in cache:
            cache[key] = gpu_ctx.state(n, precision)
        return cache[key]

    yield get
    for s in cache.values():
        s.close()


def run_gpu(states, circuit, fusion, precision="c128", initial=None, seed=0):
    st = states(circuit["num-qubits"], precision)
    if initial is None:
        st.set_basis(0)
    else:
        st.upload(initial)
    st.apply(circuit, fusion=fusion, seed=seed)
    return st


# ---------------------------------------------------------------------------
@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 10, 12, 13, 14, 17, 20])
@pytest.mark.parametrize("fusion", ["plain", "tiled"])
def test_layered_c128_bit_exact(states, oracle, n, fusion):
    from qclojure_gb300 import workloads

    c = workloads.layered_circuit(n, 20 if n <= 14 else 8, seed=n)
    ref = oracle.run(c)
    got = run_gpu(states, c, fusion).download()
    assert np.array_equal(got, ref), f"max |d| = {np.max(np.abs(got - ref))}"


@pytest.mark.parametrize("n", [3, 9, 14, 16])
@pytest.mark.parametrize("fusion", ["plain", "tiled"])
def test_every_gate_c128_bit_exact(states, oracle, n, fusion):
    c = every_gate_circuit(n, seed=100 + n)
    ref = oracle.run(c)
    got = run_gpu(states, c, fusion).download()
    assert np.array_equal(got, ref), f"max |d| = {np.max(np.abs(got - ref))}"


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("n", [6, 15])
def test_dense_fusion_c128(states, oracle, gpu_ctx, n, k):
    from qclojure_gb300 import workloads
    from qclojure_gb300.state import Context

    c = workloads.layered_circuit(n, 10, seed=k)
    ref = oracle.run(c)
    with Context(fusion="dense", fusion_width=k) as ctx:
        with ctx.state(n) as st:
            st.apply(c, fusion="dense")
            got = st.download()
    assert np.max(np.abs(got - ref)) <= 1e-12  # tolerance: FMA inside the 2^k x 2^k block product


@pytest.mark.parametrize("k", [1, 3, 5])
@pytest.mark.parametrize("n", [6, 15])
def test_dense_fusion_c64(states, oracle, n, k):
    """complex64 dense blocks multiply in FP32 (entries stored as float pairs)."""
    from qclojure_gb300 import workloads
    from qclojure_gb300.state import Context

    c = workloads.layered_circuit(n, 10, seed=20 + k)
    ref = oracle.run(c)
    with Context(fusion="dense", fusion_width=k) as ctx:
        with ctx.state(n, "c64") as st:
            st.apply(c, fusion="dense")
            got = st.download()
    assert np.max(np.abs(got - ref)) <= 2e-5  # FP32 rounding of the block entries and sums


@pytest.mark.parametrize("n", [4, 12, 16])
@pytest.mark.parametrize("fusion", ["plain", "tiled"])
def test_layered_c64(states, oracle, n, fusion):
    from qclojure_gb300 import workloads

    c = workloads.layered_circuit(n, 20, seed=7 + n)
    ref = oracle.run(c)
    st = run_gpu(states, c, fusion, "c64")
    got = st.download()
    assert np.max(np.abs(got - ref)) <= 2e-5
    p = st.probabilities()
    assert 0.5 * np.sum(np.abs(p - oracle.probabilities(ref))) <= 1e-5  # TVD


@pytest.mark.parametrize("n", [20, 21, 22])
def test_layered_c64_interpreted_tile_pairs(oracle, n):
    """Interpreted complex64 passes take two tiles per op dispatch; at these sizes a CTA
    holds several tiles of the state, odd counts included (its last tile runs alone), and
    the QFT's controlled phases test conditions on tile-index bits per tile."""
    from qclojure_gb300 import workloads
    from qclojure_gb300.state import Context

    c = workloads.large_circuit(n, 4, seed=30 + n)
    ref = oracle.run(c)
    with Context(pass_kernels="off") as ctx:
        with ctx.state(n, "c64") as st:
            st.apply(c)
            got = st.download()
    assert np.max(np.abs(got - ref)) <= 2e-5
    assert 0.5 * np.sum(np.abs(np.abs(got) ** 2 - np.abs(ref) ** 2)) <= 1e-5  # TVD


def test_initial_state_upload(states, oracle):
    from qclojure_gb300 import workloads

    rng = np.random.default_rng(3)
    n = 11
    init = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    init /= np.linalg.norm(init)
    c = workloads.layered_circuit(n, 5, seed=1)
    got = run_gpu(states, c, "tiled", initial=init).download()
    assert np.array_equal(got, oracle.run(c, init))


# ---------------------------------------------------------------------------
@pytest.mark.parametrize("n", [1, 5, 12, 18])
def test_probabilities_bit_exact(states, oracle, n):
    from qclojure_gb300 import workloads

    c = workloads.layered_circuit(n, 6, seed=n)
    st = run_gpu(states, c, "tiled")
    assert np.array_equal(st.probabilities(), oracle.probabilities(oracle.run(c)))


@pytest.mark.parametrize("n,shots", [(1, 100), (4, 1000), (10, 1024), (15, 5000), (20, 20000)])
def test_sampling_identical_to_oracle(states, oracle, n, shots):
    from qclojure_gb300 import workloads

    c = workloads.layered_circuit(n, 10, seed=2 * n)
    ref = oracle.run(c)
    st = run_gpu(states, c, "tiled")
    for seed in (1, 99):
        assert np.array_equal(st.sample(shots, seed), oracle.sample(ref, shots, seed))


def test_sampling_plain_equals_tiled(states):
    from qclojure_gb300 import workloads

    c = workloads.layered_circuit(16, 12, seed=5)
    a = run_gpu(states, c, "plain").sample(4096, 7)
    b = run_gpu(states, c, "tiled").sample(4096, 7)
    assert np.array_equal(a, b)


def test_sampling_sparse_state(states):
    """GHZ on 20 qubits: every shot lands on 0 or 2^20-1 (edge: empty blocks)."""
    from qclojure_gb300 import circuit as qc

    st = run_gpu(states, qc.ghz_state_circuit(20), "tiled")
    out = st.sample(10000, 3)
    assert set(np.unique(out).tolist()) <= {0, (1 << 20) - 1}
    assert 0.45 < np.mean(out == 0) < 0.55


def test_sampling_rejects_unnormalized(states):
    from qclojure_gb300 import _abi as A

    st = states(6)
    v = np.zeros(64, np.complex128)
    v[0] = 0.9
    st.upload(v)
    with pytest.raises(A.QgError) as e:
        st.sample(10, 1)
    assert e.value.code == A.QG_ERR_NOT_NORMALIZED


@pytest.mark.parametrize("n", [1, 3, 9, 14])
def test_pauli_expectations(states, oracle, n):
    from qclojure_gb300 import workloads

    rng = np.random.default_rng(n)
    c = workloads.layered_circuit(n, 8, seed=n + 1)
    ref = oracle.run(c)
    st = run_gpu(states, c, "tiled")
    for _ in range(12):
        p = "".join("IXYZ"[k] for k in rng.integers(0, 4, n))
        assert abs(st.pauli_expectation(p) - oracle.pauli_expectation(ref, p)) <= 1e-12
    terms = [(float(rng.normal()), "".join("IXYZ"[k] for k in rng.integers(0, 4, n))) for _ in range(5)]
    exp = oracle.hamiltonian_expectation(ref, [{"coefficient": a, "pauli-string": b} for a, b in terms])
    assert abs(st.hamiltonian(terms) - exp) <= 1e-12


def test_observable_expectations(states, oracle):
    from qclojure_gb300 import workloads

    n = 10
    c = workloads.layered_circuit(n, 6, seed=4)
    ref = oracle.run(c)
    st = run_gpu(states, c, "tiled")
    obs = [[0.3, 0.2 - 0.1j], [0.2 + 0.1j, -0.7]]
    for t in (0, 4, 9):
        assert abs(st.expectation_1q(obs, t) - oracle.expectation_1q(ref, obs, t)) <= 1e-12


def test_norm_and_inner(states, gpu_ctx, oracle):
    from qclojure_gb300 import workloads

    n = 13
    c1 = workloads.layered_circuit(n, 5, seed=1)
    c2 = workloads.layered_circuit(n, 5, seed=2)
    r1, r2 = oracle.run(c1), oracle.run(c2)
    with gpu_ctx.state(n) as a, gpu_ctx.state(n) as b:
        a.apply(c1)
        b.apply(c2)
        assert abs(a.norm2() - 1.0) <= 1e-13
        assert abs(a.inner(b) - oracle.inner(r1, r2)) <= 1e-12


def _compare_numpy(a, r):
    d = a.astype(np.complex128) - r
    na, nr = np.vdot(a, a).real, np.vdot(r, r).real
    z = np.vdot(r, d)
    return {"max_abs_diff": np.max(np.abs(d)),
            "one_minus_fidelity": (nr * np.vdot(d, d).real - abs(z) ** 2) / (na * nr),
            "tvd": 0.5 * np.sum(np.abs(np.abs(a.astype(np.complex128)) ** 2 - np.abs(r) ** 2))}


def test_state_compare(gpu_ctx, gpu_ctx_df, oracle):
    """qg_state_compare against numpy on the downloaded states: two unrelated states, a
    double-float and a complex64 run against the exact run of one circuit, identical states."""
    from qclojure_gb300 import workloads

    n = 13
    c1 = workloads.layered_circuit(n, 12, seed=5)
    c2 = workloads.layered_circuit(n, 12, seed=6)
    with gpu_ctx.state(n) as x1, gpu_ctx.state(n) as x2, gpu_ctx_df.state(n) as f1, \
            gpu_ctx.state(n, "c64") as s1:
        x1.apply(c1)
        x2.apply(c2)
        f1.apply(c1)
        s1.apply(c1)
        r1 = x1.download()
        assert np.array_equal(r1, oracle.run(c1))
        far = x2.compare(x1)
        want = _compare_numpy(x2.download(), r1)
        assert want["one_minus_fidelity"] > 0.5
        assert far["max_abs_diff"] == pytest.approx(want["max_abs_diff"], rel=1e-12)
        assert far["one_minus_fidelity"] == pytest.approx(1 - abs(oracle.inner(r1, x2.download())) ** 2, rel=1e-10)
        assert far["tvd"] == pytest.approx(want["tvd"], rel=1e-10)
        for st, lo, hi in ((f1, 1e-17, 1e-12), (s1, 1e-9, 1e-4)):
            got = st.compare(x1)
            want = _compare_numpy(st.download(), r1)
            assert lo <= got["max_abs_diff"] <= hi
            assert got["max_abs_diff"] == pytest.approx(want["max_abs_diff"], rel=1e-12)
            assert got["tvd"] == pytest.approx(want["tvd"], rel=1e-8)
            assert got["one_minus_fidelity"] == pytest.approx(want["one_minus_fidelity"], rel=1e-6, abs=1e-28)
            assert 0 <= got["one_minus_fidelity"] <= got["max_abs_diff"] ** 2 * 2 ** n
        same = x1.compare(x1)
        assert same == {"max_abs_diff": 0.0, "one_minus_fidelity": 0.0, "tvd": 0.0}
        with pytest.raises(Exception):
            x1.compare(s1)


@pytest.mark.parametrize("fusion", ["plain", "tiled"])
def test_mid_circuit_measurement(states, oracle, fusion):
    from qclojure_gb300 import workloads

    n = 12
    c = workloads.layered_circuit(n, 6, seed=8)
    c["operations"] = c["operations"] + [{"operation-type": "measure",
                                          "operation-params": {"measurement-qubits": [3, 0, 7]}}] + \
        workloads.layered_circuit(n, 3, seed=9)["operations"] + \
        [{"operation-type": "measure", "operation-params": {"measurement-qubits": [11]}}]
    for seed in (1, 2, 3):
        ref = oracle.run(c, seed=seed)
        got = run_gpu(states, c, fusion, seed=seed).download()
        assert np.max(np.abs(got - ref)) <= 1e-12


def test_state_measure_api(states, oracle):
    from qclojure_gb300 import workloads

    n = 9
    c = workloads.layered_circuit(n, 5, seed=12)
    ref = oracle.run(c)
    st = run_gpu(states, c, "tiled")
    o, p = st.measure([2, 5], seed=4)
    ref_s, ref_o, ref_p = oracle.measure(ref, [2, 5], 4, 0)
    assert o == ref_o and abs(p - ref_p) <= 1e-13
    assert np.max(np.abs(st.download() - ref_s)) <= 1e-12


# ---------------------------------------------------------------------------
# size-independent properties at sizes the oracle does not reach quickly
@pytest.mark.parametrize("n,precision,tol", [(26, "c128", 1e-12), (27, "c64", 1e-4)])
def test_circuit_then_inverse_returns_zero_state(gpu_ctx, n, precision, tol):
    from qclojure_gb300 import workloads

    c = workloads.layered_circuit(n, 6, seed=21)
    with gpu_ctx.state(n, precision) as st:
        st.apply(c, fusion="tiled")
        assert abs(st.norm2() - 1.0) <= (1e-12 if precision == "c128" else 1e-5)
        st.apply(_inverse(c), fusion="tiled")
        out = st.sample(1000, 5)
        assert np.all(out == 0)
        assert abs(st.pauli_expectation("Z" * n) - 1.0) <= tol


def test_qft_of_basis_state(gpu_ctx):
    """QFT|j> has |amp| = 2^{-n/2} everywhere (checked on 22 qubits)."""
    from qclojure_gb300 import workloads

    n = 22
    with gpu_ctx.state(n) as st:
        st.set_basis(12345)
        st.apply(workloads.qft_circuit(n), fusion="tiled")
        p = st.probabilities()
        assert np.max(np.abs(p - 2.0 ** -n)) <= 1e-18


def test_plain_equals_tiled_at_24_qubits(gpu_ctx):
    from qclojure_gb300 import workloads

    n = 24
    c = workloads.large_circuit(n, 3, seed=2)
    with gpu_ctx.state(n) as a, gpu_ctx.state(n) as b:
        a.apply(c, fusion="plain")
        b.apply(c, fusion="tiled")
        assert np.array_equal(a.download(), b.download())


# ---------------------------------------------------------------------------
# complex128 in double-float arithmetic (float pairs on the FP32 pipes):
# tolerance max |d amp| <= 1e-12 against the FP64 oracle
@pytest.mark.parametrize("n", [5, 8, 12, 13, 14, 17, 20])
def test_layered_c128_double_float(gpu_ctx_df, oracle, n):
    from qclojure_gb300 import workloads

    c = workloads.layered_circuit(n, 20 if n <= 14 else 8, seed=n)
    ref = oracle.run(c)
    with gpu_ctx_df.state(n) as st:
        st.apply(c, fusion="tiled")
        got = st.download()
        assert np.max(np.abs(got - ref)) <= 1e-12
        assert np.array_equal(st.sample(2000, 3), oracle.sample(ref, 2000, 3))


@pytest.mark.parametrize("n", [9, 16])
def test_every_gate_c128_double_float(gpu_ctx_df, oracle, n):
    c = every_gate_circuit(n, seed=200 + n)
    ref = oracle.run(c)
    with gpu_ctx_df.state(n) as st:
        st.apply(c, fusion="tiled")
        assert np.max(np.abs(st.download() - ref)) <= 1e-12


def test_double_float_mid_circuit_measurement(gpu_ctx_df, oracle):
    """Measurements split the runs of double-float passes: the state is handed over
    as float pairs inside a run and converted back to doubles at each measurement."""
    from qclojure_gb300 import workloads

    n = 16
    c = workloads.layered_circuit(n, 8, seed=18)
    c["operations"] = c["operations"] + [{"operation-type": "measure",
                                          "operation-params": {"measurement-qubits": [3, 0, 15]}}] + \
        workloads.layered_circuit(n, 6, seed=19)["operations"] + \
        [{"operation-type": "measure", "operation-params": {"measurement-qubits": [11]}}] + \
        workloads.layered_circuit(n, 2, seed=20)["operations"]
    with gpu_ctx_df.state(n) as st:
        for seed in (1, 2):
            ref = oracle.run(c, seed=seed)
            st.set_basis(0)
            st.apply(c, fusion="tiled", seed=seed)
            assert np.max(np.abs(st.download() - ref)) <= 1e-12


def test_double_float_deep_circuit_error(gpu_ctx_df, oracle):
    """300 layers (4500 gates) on 10 qubits: accumulated error stays below 1e-12."""
    from qclojure_gb300 import workloads

    c = workloads.layered_circuit(10, 300, seed=77)
    ref = oracle.run(c)
    with gpu_ctx_df.state(10) as st:
        st.apply(c, fusion="tiled")
        err = np.max(np.abs(st.download() - ref))
    assert err <= 1e-12, err


def test_double_float_inverse_at_26_qubits(gpu_ctx_df):
    from qclojure_gb300 import workloads

    n = 26
    c = workloads.large_circuit(n, 6, seed=3)
    with gpu_ctx_df.state(n) as st:
        st.apply(c, fusion="tiled")
        st.apply(_inverse(c), fusion="tiled")
        assert abs(st.pauli_expectation("Z" * n) - 1.0) <= 1e-12
        assert np.all(st.sample(500, 1) == 0)


# ---------------------------------------------------------------------------
class GpuEngine:
    def __init__(self, sim):
        self.sim = sim

    def _run(self, circuit, init, seed, specs):
        from qclojure_gb300.backend import execute_circuit

        n = circuit["num-qubits"]
        r = execute_circuit(self.sim, circuit, {"initial-state": {"state-vector": basis_state(n, init),
                                                                  "num-qubits": n},
                                                "result-specs": specs, "seed": seed})
        assert r["job-status"] == "completed", r
        return r["results"]

    def state(self, circuit, init, seed):
        return np.asarray(self._run(circuit, init, seed, {})["final-state"]["state-vector"])

    def pauli(self, circuit, init, seed, p):
        return self.hamiltonian(circuit, init, seed, [[1.0, p]])

    def hamiltonian(self, circuit, init, seed, terms):
        r = self._run(circuit, init, seed,
                      {"hamiltonian": [{"coefficient": c, "pauli-string": s} for c, s in terms]})
        return r["hamiltonian-result"]["energy-expectation"]

    def expectation(self, circuit, init, seed, obs, t):
        r = self._run(circuit, init, seed, {"expectation": {"observables": [obs], "targets": [t]}})
        return r["expectation-results"][0]["expectation-value"]

    def variance(self, circuit, init, seed, obs, t):
        r = self._run(circuit, init, seed, {"variance": {"observables": [obs], "targets": [t]}})
        return r["variance-results"][0]["variance-value"]

    def counts(self, circuit, init, seed, shots):
        r = self._run(circuit, init, seed, {"measurements": {"shots": shots}})
        return r["measurement-results"]["frequencies"]


@pytest.mark.parametrize("case", KAT, ids=[c["name"] for c in KAT])
def test_gpu_reference_kat(sim, case):
    check_case(case, GpuEngine(sim))
