"""Error-corrected circuits on the device against the oracle: the syndrome round trips of
the bit-flip and Shor codes (encode -> error -> syndrome measurement -> correction ->
decode) and the pipeline's encoded circuit with its mid-circuit syndrome measurements."""
import numpy as np
import pytest

from qclojure_gb300 import circuit as C
from qclojure_gb300 import error_correction as E
from test_error_correction import SIZES, _fidelity_on_qubit0, ec_round_trip

pytestmark = pytest.mark.gpu

CASES = [("bit-flip", None, 0), ("bit-flip", "x", 1), ("bit-flip", "x", 2),
         ("shor", None, 0), ("shor", "x", 4), ("shor", "z", 0), ("shor", "y", 8), ("shor", "z", 5)]


@pytest.mark.parametrize("key,error,qubit", CASES)
def test_round_trip_matches_oracle(gpu_ctx, oracle, key, error, qubit):
    v = np.array([0.6, 0.8j * np.exp(0.3j)])
    n = sum(SIZES[key])
    with gpu_ctx.state(n) as st:
        def run(c, s0):
            st.upload(s0)
            st.apply(c, fusion="tiled")
            return st.download()

        def measure(s, anc):
            st.upload(s)
            o, p = st.measure(anc, seed=7)
            return st.download(), o, p

        bits, p, s = ec_round_trip(run, measure, key, error, qubit, v)
    rbits, rp, rs = ec_round_trip(lambda c, s0: oracle.run(c, s0), lambda s_, anc: oracle.measure(s_, anc, 7, 0),
                                  key, error, qubit, v)
    assert bits == rbits and abs(p - rp) <= 1e-13
    assert np.max(np.abs(s - rs)) <= 1e-12
    assert abs(_fidelity_on_qubit0(s, v) - 1) < 1e-12


@pytest.mark.parametrize("fusion", ["plain", "tiled"])
def test_encoded_pipeline_circuit_matches_oracle(states_ec, oracle, fusion):
    """The bit-flip encoding of a Bell circuit (10 qubits, two syndrome measurements inside
    the circuit) runs on the device as on the oracle, for several collapse seeds."""
    c = C.cnot_gate(C.h_gate(C.create_circuit(2), 0), 0, 1)
    enc = E.apply_error_correction({"circuit": c, "options": {"apply-error-correction?": True}})["circuit"]
    st = states_ec(enc["num-qubits"])
    for seed in (1, 2, 3):
        st.set_basis(0)
        st.apply(enc, fusion=fusion, seed=seed)
        assert np.max(np.abs(st.download() - oracle.run(enc, seed=seed))) <= 1e-12


@pytest.fixture(scope="module")
def states_ec(gpu_ctx):
    cache = {}

    def get(n):
        if n not in cache:
            cache[n] = gpu_ctx.state(n)
        return cache[n]

    yield get
    for st in cache.values():
        st.close()
