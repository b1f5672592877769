"""The pass-kernel autotuner (qg_autotune) on the device.

It times candidate tile sizes and launch shapes of the specialised pass kernels on a
calibration circuit, keeps the fastest for the context, and programs of that size
then compile with that shape. Checked here: the chosen shape is no slower than the
default on the same calibration (the rule keeps the default unless another shape wins
by more than 1 %), a circuit run with the tuned shape still matches the oracle, and
qg_tuning_set refuses shapes the kernels cannot take.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tol", [("c128", 1e-12), ("c64", 2e-5)])
def test_autotune_picks_no_slower_shape_and_stays_exact(oracle, precision, tol):
    from qclojure_gb300 import workloads
    from qclojure_gb300.state import Context

    n = 20
    with Context(pass_kernels="always", arithmetic="double-float") as ctx:
        res = ctx.autotune(n, precision)
        cands = res["candidates"]
        default = cands[0]
        assert default["tile_bits"] == 12 and default["ms"] > 0
        chosen = res["chosen"]
        assert chosen["ms"] <= default["ms"] * 1.0000001
        assert ctx.tuning(n, precision)["tile_bits"] == chosen["tile_bits"]
        c = workloads.layered_circuit(n, 8, seed=3)
        c = {"num-qubits": n, "operations": c["operations"] + workloads.qft_ops(n)}
        for t in cands:  # every candidate shape computes the same state
            ctx.set_tuning(n, precision, t["tile_bits"], t["reg_bits"], t["buffers"], t["ctas_per_sm"])
            with ctx.state(n, precision) as st:
                st.apply(c)
                got = st.download()
            assert np.max(np.abs(got - oracle.run(c))) <= tol, t


def test_tuning_set_refuses_impossible_shapes():
    from qclojure_gb300._abi import QG_ERR_INVALID_ARG, QgError
    from qclojure_gb300.state import Context

    with Context(pass_kernels="always") as ctx:
        for bad in ((14, 3, 2, 1), (12, 5, 2, 1), (13, 3, 2, 2), (12, 3, 3, 1), (10, 3, 2, 1)):
            with pytest.raises(QgError) as ei:
                ctx.set_tuning(20, "c128", *bad)
            assert ei.value.code == QG_ERR_INVALID_ARG
        ctx.set_tuning(20, "c128", 11, 3, 2, 2)
        assert ctx.tuning(20, "c128")["tile_bits"] == 11
        ctx.set_tuning(20, "c128", 0)
        assert ctx.tuning(20, "c128")["tile_bits"] == 12
