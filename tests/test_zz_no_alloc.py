"""qg_state_sample_noalloc against qg_state_sample.

Both entry points run the same sampler kernels on the same state with the same
seed, so the outcomes must be identical (integer work: tolerance zero), here
for two calls in a row on one state. The file sorts last so it also runs after
every other GPU test in one process.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHOTS = 4096


@pytest.mark.parametrize("n,precision", [(5, "c128"), (16, "c64"), (24, "c128")])
def test_noalloc_sampler_matches_allocating_sampler(gpu_ctx, n, precision):
    import torch

    from qclojure_gb300 import workloads

    seeds = (20261204, 7)
    with gpu_ctx.state(n, precision) as st:
        st.apply(workloads.layered_circuit(n, 3, seed=n), fusion="tiled")
        ref = [st.sample(SHOTS, s) for s in seeds]
        bufs = [torch.full((SHOTS,), -1, dtype=torch.int64, device="cuda:0") for _ in seeds]
        torch.cuda.synchronize()
        for s, b in zip(seeds, bufs):  # two calls in a row on the same scratch
            st.sample_noalloc(SHOTS, s, b.data_ptr())
        for r, b in zip(ref, bufs):
            got = b.cpu().numpy().view(np.uint64)
            assert np.array_equal(got, r)
        assert not np.array_equal(ref[0], ref[1])
        st.sample_noalloc(0, seeds[0], 0)  # zero shots: no buffer needed


def test_noalloc_sampler_rejects_states_beyond_its_scratch(gpu_ctx):
    import torch

    from qclojure_gb300._abi import QG_ERR_INVALID_ARG, QgError

    buf = torch.empty(16, dtype=torch.int64, device="cuda:0")
    with gpu_ctx.state(25, "c64") as st:
        with pytest.raises(QgError) as ei:
            st.sample_noalloc(16, 1, buf.data_ptr())
        assert ei.value.code == QG_ERR_INVALID_ARG
        assert "24 qubits" in str(ei.value)


def test_noalloc_sampler_rejects_host_outcome_buffers(gpu_ctx):
    """The outcome buffer must be device memory of the state's device: a pageable host
    array (numpy) is refused before any kernel runs."""
    from qclojure_gb300 import workloads
    from qclojure_gb300._abi import QG_ERR_INVALID_ARG, QgError

    host = np.zeros(64, np.uint64)
    with gpu_ctx.state(8, "c128") as st:
        st.apply(workloads.layered_circuit(8, 2, seed=1), fusion="tiled")
        with pytest.raises(QgError) as ei:
            st.sample_noalloc(64, 1, host.ctypes.data)
        assert ei.value.code == QG_ERR_INVALID_ARG
        assert "device memory" in str(ei.value)
    assert not host.any()
