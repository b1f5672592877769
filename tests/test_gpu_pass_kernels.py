"""Specialised pass kernels (one generated, NVRTC-compiled kernel per tiled pass)
against the CPU oracle, through the C ABI.

The contexts here force the specialised kernels for every state size
(pass_kernels="always"), so small states that the oracle finishes in seconds
exercise the same generated code the large states run. Tolerances:
  complex128 double-float   max |d amp| <= 1e-12 against the FP64 oracle
  complex64                 max |d amp| <= 2e-5, probability TVD <= 1e-5
  sampled outcomes          identical to the oracle's for the same seed (c128)
"""
import numpy as np
import pytest

from test_gpu_parity import _inverse, every_gate_circuit

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx_df(built):
    from qclojure_gb300.state import Context

    ctx = Context(seed=1, arithmetic="double-float", pass_kernels="always")
    yield ctx
    ctx.close()


@pytest.fixture(scope="module")
def ctx_off(built):
    from qclojure_gb300.state import Context

    ctx = Context(seed=1, arithmetic="double-float", pass_kernels="off")
    yield ctx
    ctx.close()


def _run(ctx, circuit, precision, seed=0):
    st = ctx.state(circuit["num-qubits"], precision)
    st.set_basis(0)
    ms, kinds = st.profile(circuit, fusion="tiled", seed=seed)
    return st, kinds


@pytest.mark.parametrize("n", [12, 14, 17, 20])
def test_layered_c128_df_specialised(ctx_df, oracle, n):
    from qclojure_gb300 import workloads

    c = workloads.layered_circuit(n, 20 if n <= 14 else 8, seed=300 + n)
    ref = oracle.run(c)
    st, kinds = _run(ctx_df, c, "c128")
    with st:
        assert np.count_nonzero(kinds == 3) > 0 and np.count_nonzero(kinds == 1) == 0, kinds
        got = st.download()
        assert np.max(np.abs(got - ref)) <= 1e-12, np.max(np.abs(got - ref))
        assert np.array_equal(st.sample(2000, 5), oracle.sample(ref, 2000, 5))


@pytest.mark.parametrize("n", [13, 16])
def test_every_gate_c128_df_specialised(ctx_df, oracle, n):
    c = every_gate_circuit(n, seed=400 + n)
    ref = oracle.run(c)
    st, kinds = _run(ctx_df, c, "c128")
    with st:
        assert np.count_nonzero(kinds == 3) > 0
        err = np.max(np.abs(st.download() - ref))
        assert err <= 1e-12, err


def test_qft_c128_df_specialised(ctx_df, oracle):
    """The QFT passes (long runs of controlled phases on thread and tile bits)."""
    from qclojure_gb300 import workloads

    n = 16
    c = workloads.large_circuit(n, 3, seed=9)
    ref = oracle.run(c)
    st, kinds = _run(ctx_df, c, "c128")
    with st:
        err = np.max(np.abs(st.download() - ref))
        assert err <= 1e-12, err


def test_df_mid_circuit_measurement_specialised(ctx_df, oracle):
    """Measurements split runs of passes: pair/double hand-over at every boundary."""
    from qclojure_gb300 import workloads

    n = 15
    c = workloads.layered_circuit(n, 6, seed=31)
    c["operations"] = c["operations"] + [{"operation-type": "measure",
                                          "operation-params": {"measurement-qubits": [2, 14]}}] + \
        workloads.layered_circuit(n, 5, seed=32)["operations"]
    for seed in (1, 2):
        ref = oracle.run(c, seed=seed)
        st, kinds = _run(ctx_df, c, "c128", seed=seed)
        with st:
            assert np.count_nonzero(kinds == 2) == 1
            assert np.max(np.abs(st.download() - ref)) <= 1e-12


@pytest.mark.parametrize("n", [12, 16, 20])
def test_layered_c64_specialised(ctx_df, oracle, n):
    from qclojure_gb300 import workloads

    c = workloads.layered_circuit(n, 12, seed=500 + n)
    ref = oracle.run(c)
    st, kinds = _run(ctx_df, c, "c64")
    with st:
        assert np.count_nonzero(kinds == 3) > 0
        got = st.download()
        assert np.max(np.abs(got - ref)) <= 2e-5
        tvd = 0.5 * np.sum(np.abs(np.abs(got) ** 2 - np.abs(ref) ** 2))
        assert tvd <= 1e-5, tvd


def test_every_gate_c64_specialised(ctx_df, oracle):
    c = every_gate_circuit(14, seed=614)
    ref = oracle.run(c)
    st, kinds = _run(ctx_df, c, "c64")
    with st:
        assert np.max(np.abs(st.download() - ref)) <= 2e-5


@pytest.mark.parametrize("precision,tol", [("c128", 1e-12), ("c64", 2e-5)])
def test_qaoa_parity_runs_specialised(ctx_df, oracle, precision, tol):
    """QAOA MaxCut: each cost layer's RZZ gates (one angle) run as a parity-count
    table per register instead of one complex product per gate."""
    from qclojure_gb300 import workloads

    for n, seed in ((14, 3), (18, 4)):
        c = workloads.qaoa_maxcut(n, 3, seed)
        ref = oracle.run(c)
        st, kinds = _run(ctx_df, c, precision)
        with st:
            assert np.count_nonzero(kinds == 3) > 0
            assert np.max(np.abs(st.download() - ref)) <= tol


def test_specialised_matches_interpreted(ctx_df, ctx_off):
    """The same program through both executors: equal within the double-float bound."""
    from qclojure_gb300 import workloads

    c = workloads.large_circuit(18, 4, seed=5)
    a, ka = _run(ctx_df, c, "c128")
    b, kb = _run(ctx_off, c, "c128")
    with a, b:
        assert np.all(ka != 1) and np.all(kb != 3)
        assert np.max(np.abs(a.download() - b.download())) <= 1e-12


def test_inverse_at_24_qubits_specialised(ctx_df):
    from qclojure_gb300 import workloads

    n = 24
    c = workloads.large_circuit(n, 4, seed=11)
    st = ctx_df.state(n, "c128")
    with st:
        st.set_basis(0)
        st.apply(c)
        st.apply(_inverse(c))
        assert abs(st.pauli_expectation("Z" * n) - 1.0) <= 1e-12
        assert np.all(st.sample(300, 2) == 0)


def _rotations_at_special_angles(n):
    import math

    ops = [{"operation-type": "h", "operation-params": {"target": q}} for q in range(n)]
    angles = [0.0, math.pi / 2, math.pi, 3 * math.pi / 2, 2 * math.pi, math.pi - 1e-9, 1e-9, -math.pi / 4, 5.0]
    for k, a in enumerate(angles):
        for g in ("rx", "ry", "rz"):
            ops.append({"operation-type": g, "operation-params": {"target": (k + len(g)) % n, "angle": a}})
        ops.append({"operation-type": "cnot", "operation-params": {"control": k % n, "target": (k + 1) % n}})
    return {"num-qubits": n, "operations": ops}


@pytest.mark.parametrize("precision,tol", [("c128", 1e-12), ("c64", 2e-5)])
def test_rotation_factoring_special_angles(ctx_df, oracle, precision, tol):
    """Rotations become unit-diagonal forms plus a global scalar, with an X when the
    off-diagonal entry dominates; angles where an entry vanishes or both are equal
    must keep the reference's results."""
    c = _rotations_at_special_angles(13)
    ref = oracle.run(c)
    st, kinds = _run(ctx_df, c, precision)
    with st:
        assert np.max(np.abs(st.download() - ref)) <= tol


def test_deep_hadamard_chain_rescaling(ctx_df, oracle):
    """2400 Hadamards: their 1/sqrt2 factors are collected with exact 2^-20
    rescales, so the unscaled amplitudes never leave the float range."""
    n = 12
    ops = []
    for layer in range(200):
        ops += [{"operation-type": "h", "operation-params": {"target": q}} for q in range(n)]
        ops.append({"operation-type": "t", "operation-params": {"target": layer % n}})
    c = {"num-qubits": n, "operations": ops}
    ref = oracle.run(c)
    st, _ = _run(ctx_df, c, "c128")
    with st:
        assert np.max(np.abs(st.download() - ref)) <= 1e-12


@pytest.mark.parametrize("precision,tol", [("c128", 1e-12), ("c64", 2e-5)])
def test_parity_runs_with_mixed_angles(ctx_df, oracle, precision, tol):
    """RZZ layers whose angles alternate split into several runs; a run of one angle
    uses one parity-count table."""
    import math

    n = 14
    rng = np.random.default_rng(3)
    ops = [{"operation-type": "h", "operation-params": {"target": q}} for q in range(n)]
    for layer in range(3):
        for e in range(20):
            a, b = (int(x) for x in rng.choice(n, 2, replace=False))
            ang = 0.7 if (e // 3) % 2 == 0 else 1.9 + layer
            ops.append({"operation-type": "rzz", "operation-params": {"qubit1": a, "qubit2": b, "angle": ang}})
        ops += [{"operation-type": "rx", "operation-params": {"target": q, "angle": 0.3 + q / 7}} for q in range(n)]
    c = {"num-qubits": n, "operations": ops}
    ref = oracle.run(c)
    st, _ = _run(ctx_df, c, precision)
    with st:
        assert np.max(np.abs(st.download() - ref)) <= tol


def test_compiled_programs_are_cached(ctx_df):
    """A second run of the same program reuses its compiled modules (cache hit);
    a circuit with other angles compiles anew."""
    import ctypes as C

    from qclojure_gb300 import workloads

    lib = ctx_df.lib

    def info():
        a, h, m = C.c_int32(), C.c_uint64(), C.c_uint64()
        lib.qg_pass_kernels_info(C.byref(a), C.byref(h), C.byref(m))
        return a.value, h.value, m.value

    c = workloads.layered_circuit(14, 6, seed=808)
    with ctx_df.state(14, "c128") as st:
        st.apply(c)
        _, h0, m0 = info()
        st.apply(c)
        avail, h1, m1 = info()
        assert avail == 1 and h1 == h0 + 1 and m1 == m0
        st.apply(workloads.layered_circuit(14, 6, seed=809))
        _, h2, m2 = info()
        assert m2 == m1 + 1
