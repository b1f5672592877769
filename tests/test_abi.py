"""CPU tests of the C ABI library and the host logic (no GPU compute)."""
import ctypes as C
import subprocess

import numpy as np
import pytest


def test_library_exports_every_declared_symbol(built):
    from qclojure_gb300 import _abi as A

    declared = A.declared_symbols()
    assert len(declared) >= 40
    out = subprocess.run(["nm", "-D", "--defined-only", str(A.LIB_PATH)], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    assert set(declared) == set(A.SIGNATURES), "ctypes signatures and header differ"
    lib = A.load_library()
    assert lib.qg_abi_version() == 1


def test_struct_layouts_match_header(built):
    """Sizes the C side expects (checked against a compile of the header)."""
    from qclojure_gb300 import _abi as A

    assert C.sizeof(A.QgOp) == 4 + 4 + 40 + 8 + 64
    assert C.sizeof(A.QgCircuit) == 16
    assert C.sizeof(A.QgConfig) == 6 * 4 + 2 * 8 + 4 * 4
    src = r'''
#include <stdio.h>
#include "qgpu.h"
int main(void){printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(qg_op), sizeof(qg_circuit), sizeof(qg_result_spec),
 sizeof(qg_options), sizeof(qg_config), sizeof(qg_queue_info), sizeof(qg_job_info));return 0;}
'''
    import tempfile
    from pathlib import Path

    with tempfile.TemporaryDirectory() as d:
        p = Path(d) / "s.c"
        p.write_text(src)
        exe = Path(d) / "s"
        subprocess.run(["gcc", "-I", str(A.HEADER.parent), str(p), "-o", str(exe)], check=True)
        sizes = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    assert sizes == [C.sizeof(A.QgOp), C.sizeof(A.QgCircuit), C.sizeof(A.QgResultSpec), C.sizeof(A.QgOptions),
                     C.sizeof(A.QgConfig), C.sizeof(A.QgQueueInfo), C.sizeof(A.QgJobInfo)]


def test_no_device_is_reported_not_faked(built):
    """Without a GPU the context refuses to start; nothing falls back to the CPU."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from qclojure_gb300 import _abi as A

    lib = A.load_library()
    n = C.c_int32(-1)
    assert lib.qg_device_count(C.byref(n)) == 0 and n.value == 0
    ctx = C.c_void_p()
    assert lib.qg_ctx_create(None, C.byref(ctx)) == A.QG_ERR_NO_DEVICE
    from qclojure_gb300.backend import create_simulator

    with pytest.raises(A.QgError):
        create_simulator()


def test_null_arguments_are_rejected(built):
    from qclojure_gb300 import _abi as A

    lib = A.load_library()
    assert lib.qg_ctx_create(None, None) == A.QG_ERR_INVALID_ARG
    assert lib.qg_job_status(None, 1, None) == A.QG_ERR_INVALID_ARG
    assert lib.qg_state_destroy(None) == A.QG_ERR_INVALID_ARG
    assert lib.qg_submit(None, None, None, None) == A.QG_ERR_INVALID_ARG


def test_missing_library_fails_loudly(tmp_path):
    from qclojure_gb300 import _abi as A

    with pytest.raises(RuntimeError):
        A.load_library(tmp_path / "libqgpu.so")


def test_tuning_pick_rule(built):
    """qg_tuning_pick: the fastest valid candidate, unless the default is within the tie
    fraction of it; invalid or unmeasured entries never win (fake timings, no GPU)."""
    from qclojure_gb300 import _abi as A

    lib = A.load_library()

    def pick(ms, valid, default=0, tie=0.01):
        n = len(ms)
        return lib.qg_tuning_pick((C.c_double * n)(*ms), (C.c_int32 * n)(*valid), n, default, tie)

    assert pick([10.0, 8.0, 9.0], [1, 1, 1]) == 1
    assert pick([10.0, 9.95, 9.0], [1, 1, 0]) == 0          # within 1 %: keep the default
    assert pick([10.0, 9.0, 9.5], [1, 1, 1], tie=0.2) == 0  # a wider tie band keeps it too
    assert pick([10.0, 4.0, 9.0], [1, 0, 1]) == 2           # the fastest one did not compile
    assert pick([0.0, 7.0], [1, 1]) == 1                    # no measurement is no candidate
    assert pick([5.0, 7.0], [0, 0]) == -1
    assert pick([12.0, 11.0], [1, 1], default=-1) == 1

