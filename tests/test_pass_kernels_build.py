"""Specialised pass kernels on the CPU: every circuit shape the GPU tests use must
generate kernels that NVRTC compiles for sm_103a (no device is needed for the
compile), and the exact complex128 policy must stay with the interpreter."""
import ctypes as C

import pytest

from test_gpu_parity import every_gate_circuit


def _build(lib, circuit, precision, arithmetic):
    from qclojure_gb300.circuit import encode

    enc = encode(circuit)
    k, ms = C.c_int32(), C.c_double()
    buf = C.create_string_buffer(4096)
    rc = lib.qg_pass_kernels_build(enc.ref(), precision, arithmetic, C.byref(k), C.byref(ms), buf, 4096)
    return rc, k.value, buf.value.decode()


@pytest.fixture(scope="module")
def lib(built):
    from qclojure_gb300 import _abi as A

    lib = A.load_library()
    avail = C.c_int32()
    lib.qg_pass_kernels_info(C.byref(avail), None, None)
    if not avail.value:
        pytest.skip("NVRTC is not available on this host")
    return lib


@pytest.mark.parametrize("precision,arithmetic", [(0, 1), (1, 0)], ids=["c128-double-float", "c64"])
def test_every_gate_pass_kernels_compile(lib, precision, arithmetic):
    c = every_gate_circuit(14, seed=7)
    rc, kernels, err = _build(lib, c, precision, arithmetic)
    assert rc == 0, err
    assert kernels > 0


def test_qft_and_measurement_pass_kernels_compile(lib):
    from qclojure_gb300 import workloads

    c = workloads.large_circuit(13, 2, seed=3)
    c["operations"].insert(20, {"operation-type": "measure", "operation-params": {"measurement-qubits": [1, 5]}})
    rc, kernels, err = _build(lib, c, 0, 1)
    assert rc == 0, err
    assert kernels > 0


def test_exact_arithmetic_is_not_specialised(lib):
    from qclojure_gb300 import workloads

    rc, kernels, _ = _build(lib, workloads.layered_circuit(12, 3, seed=1), 0, 0)
    assert rc == 0 and kernels == 0


@pytest.mark.parametrize("precision,arithmetic", [(0, 1), (1, 0)], ids=["c128-double-float", "c64"])
def test_qaoa_parity_runs_compile(lib, precision, arithmetic):
    """QAOA cost layers: runs of RZZ with one angle become parity-count tables."""
    from qclojure_gb300 import workloads

    rc, kernels, err = _build(lib, workloads.qaoa_maxcut(16, 3, seed=4), precision, arithmetic)
    assert rc == 0, err
    assert kernels > 0


@pytest.mark.parametrize("precision,arithmetic", [(0, 1), (1, 0)], ids=["c128-double-float", "c64"])
def test_table_form_sweep_kernels_compile(lib, precision, arithmetic):
    """The table-form kernels a parameter sweep compiles (QG_PASS_BUILD_TABLE): QAOA cost
    layers of 36 edges (counts in six bit planes, read out as bytes) and one run of 300
    RZZ of a single angle (nine planes: the read-out bit by bit)."""
    import numpy as np

    from qclojure_gb300 import _abi as A
    from qclojure_gb300 import workloads

    rc, kernels, err = _build(lib, workloads.qaoa_maxcut(24, 3, seed=4), precision, arithmetic | A.QG_PASS_BUILD_TABLE)
    assert rc == 0, err
    assert kernels > 0
    rng = np.random.default_rng(3)
    ops = [{"operation-type": "h", "operation-params": {"target": q}} for q in range(14)]
    for _ in range(300):
        a, b = (int(x) for x in rng.choice(14, 2, replace=False))
        ops.append({"operation-type": "rzz", "operation-params": {"qubit1": a, "qubit2": b, "angle": 0.375}})
    rc, kernels, err = _build(lib, {"num-qubits": 14, "operations": ops}, precision,
                              arithmetic | A.QG_PASS_BUILD_TABLE)
    assert rc == 0, err
    assert kernels > 0
