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


@pytest.mark.parametrize("shape", [(12, 4, 2, 1), (11, 4, 2, 2), (12, 4, 1, 1), (10, 3, 3, 4)])
def test_every_accepted_double_float_shape_is_exact(oracle, shape):
    """Shapes qg_tuning_set accepts beyond the autotuner's candidates (16 amplitudes per
    thread in double-float, three tile buffers) compute the state within 1e-12."""
    from qclojure_gb300 import workloads
    from qclojure_gb300.state import Context

    n = 16
    c = workloads.layered_circuit(n, 10, seed=9)
    c = {"num-qubits": n, "operations": c["operations"] + workloads.qft_ops(n)}
    with Context(pass_kernels="always", arithmetic="double-float") as ctx:
        ctx.set_tuning(n, "c128", *shape)
        with ctx.state(n, "c128") as st:
            st.apply(c)
            got = st.download()
    assert np.max(np.abs(got - oracle.run(c))) <= 1e-12


def test_tuning_set_refuses_impossible_shapes():
    from qclojure_gb300._abi import QG_ERR_INVALID_ARG, QgError
    from qclojure_gb300.state import Context

    with Context(pass_kernels="always") as ctx:
        for bad in ((14, 3, 2, 1), (12, 5, 2, 1), (13, 3, 2, 2), (12, 3, 4, 1), (9, 3, 2, 1)):
            with pytest.raises(QgError) as ei:
                ctx.set_tuning(20, "c128", *bad)
            assert ei.value.code == QG_ERR_INVALID_ARG
        ctx.set_tuning(20, "c128", 11, 3, 2, 2)
        assert ctx.tuning(20, "c128")["tile_bits"] == 11
        ctx.set_tuning(20, "c128", 0)
        assert ctx.tuning(20, "c128")["tile_bits"] == 12


def test_crossover_sets_the_specialisation_size(oracle):
    """qg_autotune_crossover measures interpreted vs compile + specialised time per size and
    the context then specialises from the crossover on; results stay within tolerance."""
    import ctypes as C

    from qclojure_gb300 import _abi as A
    from qclojure_gb300 import workloads
    from qclojure_gb300.backend import create_simulator

    sim = create_simulator({"precision": "c64", "fusion": "tiled", "workers": 2, "seed": 1})
    try:
        res = sim.autotune_crossover("c64", 30)
        rows = res["rows"]
        assert [r["qubits"] for r in rows] == [20, 22, 24, 26, 28, 30]
        assert all(r["interpreted_ms"] > 0 and r["specialised_ms"] > 0 and r["compile_ms"] > 0 for r in rows)
        m = res["min_qubits"]
        assert 20 <= m <= 31
        gains = [r["compile_ms"] + r["specialised_ms"] < r["interpreted_ms"] for r in rows]
        assert all(g for r, g in zip(rows, gains) if r["qubits"] >= m)
        n = 20 if m > 20 else m  # a job below (or at) the crossover
        c = workloads.layered_circuit(n, 4, seed=2)
        jid = sim.submit_circuit(c, {"result-specs": {"state-vector": True}})
        assert sim.wait(jid, 300_000) == "completed"
        info = A.QgJobInfo()
        sim._lib.qg_job_details(sim._ctx, C.c_uint64(sim._jid(jid)), C.byref(info))
        assert (info.specialised_passes > 0) == (n >= m)
        sv = np.asarray(sim.job_result(jid)["results"]["final-state"]["state-vector"])
        assert np.max(np.abs(sv - oracle.run(c))) <= 2e-5
    finally:
        sim.close()
