"""complex64 dense fused blocks on the tensor cores (dense_tc.cu) against the oracle.

With fusion "dense", runs of gates on at most k qubits become one 2^k x 2^k block; a
complex64 state of at least 12 qubits applies each block in one HBM pass with
tcgen05.mma (split-TF32: hi*hi + lo*hi + hi*lo, FP32 accumulate). Blocks of 1-3 qubits
are widened to 4 with the identity. Tolerance: the complex64 contract, probability TVD
<= 1e-5 against the FP64 oracle, and <= 2e-5 per amplitude.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TC_PASS = 4  # profile kind of a tensor-core block pass


def _on_qubits(n, qubits, count, seed):
    """Random one- and two-qubit gates confined to `qubits` (one dense block of them)."""
    import math

    rng = np.random.default_rng(seed)
    ops = []
    one = ("h", "x", "y", "z", "s", "t", "rx", "ry", "rz")
    for _ in range(count):
        if len(qubits) > 1 and rng.integers(3) == 0:
            a, b = (int(x) for x in rng.choice(qubits, 2, replace=False))
            ops.append({"operation-type": "cnot", "operation-params": {"control": a, "target": b}})
        else:
            g = one[rng.integers(len(one))]
            p = {"target": int(rng.choice(qubits))}
            if g in ("rx", "ry", "rz"):
                p["angle"] = float(rng.uniform(0, 2 * math.pi))
            ops.append({"operation-type": g, "operation-params": p})
    return ops


def _check(oracle, c, k, expect_tc=True):
    from qclojure_gb300.state import Context

    n = c["num-qubits"]
    ref = oracle.run(c)
    with Context(fusion="dense", fusion_width=k) as ctx:
        with ctx.state(n, "c64") as st:
            st.set_basis(0)
            ms, kinds = st.profile(c, fusion="dense")
            got = st.download()
    err = float(np.max(np.abs(got - ref)))
    tvd = 0.5 * float(np.abs(np.abs(got) ** 2 - np.abs(ref) ** 2).sum())
    assert err <= 2e-5 and tvd <= 1e-5, (n, k, err, tvd)
    if expect_tc:
        assert (kinds == TC_PASS).any(), kinds
    return kinds


@pytest.mark.parametrize("k", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("n", [12, 13, 17])
def test_layered_blocks(oracle, n, k):
    from qclojure_gb300 import workloads

    kinds = _check(oracle, workloads.layered_circuit(n, 6, seed=40 + k + n), k)
    assert (kinds == TC_PASS).sum() >= 1


@pytest.mark.parametrize("qubits", [
    [0, 1, 2, 3, 4],            # the five highest index bits
    [15, 16, 17, 18, 19],       # the five lowest index bits (bit 0 is a target)
    [0, 7, 12, 18, 19],         # spread, with bits 0 and 1 targets
    [3, 9, 10, 11],             # four qubits in the middle
    [19],                       # one qubit on bit 0, widened to four
    [2, 17],                    # two qubits, widened
])
def test_block_positions(oracle, qubits):
    n = 20
    c = {"num-qubits": n, "operations": _on_qubits(n, qubits, 24, seed=sum(qubits))}
    pre = [{"operation-type": "h", "operation-params": {"target": q}} for q in range(n)]
    c["operations"] = pre + c["operations"]
    _check(oracle, c, 5)


def test_two_calls_and_small_states(oracle):
    """Repeated blocks reuse the same operands; states below 12 qubits keep the CUDA-core path."""
    from qclojure_gb300 import workloads

    c = workloads.layered_circuit(14, 3, seed=5)
    _check(oracle, c, 5)
    _check(oracle, c, 5)
    small = workloads.layered_circuit(9, 4, seed=6)
    kinds = _check(oracle, small, 5, expect_tc=False)
    assert not (kinds == TC_PASS).any()


def test_bounded_wait_gives_up_and_the_context_survives(oracle):
    """Failure path without a GPU fault: with the diagnostic switch on, the kernel's MMA
    thread issues nothing, so the epilogue's bounded wait for the first tile runs out
    (about a second); the kernel drains its bulk copies, frees its tensor memory and
    returns, the run fails with a device error naming the wait, and the same context
    then applies the block correctly."""
    from qclojure_gb300 import _abi as A
    from qclojure_gb300.state import Context

    lib = A.load_library()
    n = 14
    c = {"num-qubits": n, "operations": _on_qubits(n, [3, 9, 10, 11], 16, seed=77)}
    ref = oracle.run(c)
    with Context(fusion="dense", fusion_width=4) as ctx:
        with ctx.state(n, "c64") as st:
            st.set_basis(0)
            _, kinds = st.profile(c, fusion="dense")
            assert 1 <= (kinds == TC_PASS).sum() <= 2, kinds  # one block: about a second per stalled pass
            st.set_basis(0)
            assert lib.qg_diag_dense_tc_stall(1) == 0
            try:
                with pytest.raises(A.QgError, match="bounded wait") as ei:
                    st.apply(c, fusion="dense")
                assert ei.value.code == A.QG_ERR_DEVICE
            finally:
                lib.qg_diag_dense_tc_stall(0)
            st.set_basis(0)
            st.apply(c, fusion="dense")
            got = st.download()
    tvd = 0.5 * float(np.abs(np.abs(got) ** 2 - np.abs(ref) ** 2).sum())
    assert float(np.max(np.abs(got - ref))) <= 2e-5 and tvd <= 1e-5
