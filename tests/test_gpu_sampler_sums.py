"""The sampler's quantised probability sums against the oracle, bit for bit.

measure-state (state.clj:869-913) draws from the cumulative distribution; the sampler
keeps it as integer prefix sums of floor(p 2^62) per amplitude (p = re^2 + im^2 in
FP64). A single quantisation off by one unit would move every later prefix by one and
still leave almost every drawn outcome unchanged, so outcome comparisons cannot see it:
these tests compare every chunk sum and the total with the oracle's. The states cover
the fixed-point fast path (parts below 2^-10: states of 20 and more qubits), its
FP64 fallback (large parts, mixed with small ones in one warp), zero amplitudes, the
partial-block geometry of small states and both precisions.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check(oracle, st):
    got, total = st.sample_sums()
    ref, ref_total = oracle.chunk_sums(st.download().astype(np.complex128))
    assert total == ref_total
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("precision", ["c128", "c64"])
@pytest.mark.parametrize("n", [3, 5, 12, 13, 16, 20, 22])
def test_sample_sums_layered(gpu_ctx, oracle, n, precision):
    from qclojure_gb300 import workloads

    with gpu_ctx.state(n, precision) as st:
        st.apply(workloads.layered_circuit(n, 6, seed=n + 40), fusion="tiled")
        _check(oracle, st)


@pytest.mark.parametrize("precision", ["c128", "c64"])
def test_sample_sums_concentrated_and_sparse(gpu_ctx, oracle, precision):
    """22 qubits with only the 7 lowest-order qubits entangled: 128 large amplitudes
    (the FP64 fallback) among zeros, then a GHZ state (two amplitudes of 1/sqrt 2)."""
    from qclojure_gb300 import circuit as qc
    from qclojure_gb300 import workloads

    n = 22
    c = workloads.layered_circuit(7, 8, seed=3)
    ops = [dict(op) for op in c["operations"]]
    for op in ops:  # move the 7-qubit circuit onto qubits n-7 .. n-1 (index bits 0..6)
        p = dict(op["operation-params"])
        for k in ("target", "control"):
            if k in p:
                p[k] = p[k] + n - 7
        op["operation-params"] = p
    with gpu_ctx.state(n, precision) as st:
        st.apply({"num-qubits": n, "operations": ops}, fusion="tiled")
        _check(oracle, st)
    with gpu_ctx.state(n, precision) as st:
        st.apply(qc.ghz_state_circuit(n), fusion="tiled")
        _check(oracle, st)


@pytest.mark.parametrize("precision", ["c128", "c64"])
def test_sample_sums_crafted_amplitudes(gpu_ctx, oracle, precision):
    """Uploaded (unnormalised) amplitudes: parts of every magnitude from 2^-45 to 2^-8,
    zeros, and sums placed on grid points of 2^-62 (the fast path's guard)."""
    rng = np.random.default_rng(11)
    n = 16
    N = 1 << n
    mag = np.exp2(rng.uniform(-45, -8, size=(N, 2))) * rng.choice([-1.0, 1.0], size=(N, 2))
    v = mag[:, 0] + 1j * mag[:, 1]
    k = N // 4  # a quarter on grid points: re^2 + im^2 within rounding of Q 2^-62
    Q = np.floor(np.exp2(rng.integers(10, 51, size=k)) * (1 + rng.random(k)))
    pt = np.ldexp(Q, -62)
    re = np.sqrt(pt) * rng.random(k)
    im = np.sqrt(pt - re * re)
    im = np.where(rng.random(k) < 0.3, np.nextafter(im, 1.0), im)
    v[:k] = re + 1j * im
    v[k:k + 64] = 0
    v[k + 64:k + 96] = 2.0 ** -10 + 1j * 2.0 ** -11
    with gpu_ctx.state(n, precision) as st:
        st.upload(v)
        _check(oracle, st)


def test_sample_sums_rejects_a_wrong_count(gpu_ctx):
    from qclojure_gb300 import _abi as A

    with gpu_ctx.state(10) as st:
        out = np.zeros(8, np.uint64)
        import ctypes as C

        total = C.c_uint64()
        rc = st.lib.qg_diag_sample_sums(st.h, out.ctypes.data_as(A.U64P), C.c_uint64(8), C.byref(total))
        assert rc == A.QG_ERR_INVALID_ARG
