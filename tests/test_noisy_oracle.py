"""The oracle's restatement of the noisy shot loop, pinned to the reference's channel and
noise tests (test/org/soulspace/qclojure/domain/channel_test.clj, noise_test.clj) and
to the channel semantics they describe. CPU only."""
import math

import numpy as np
import pytest


def _max_sq(m):
    return max(abs(z) ** 2 for z in np.asarray(m).ravel())


def test_depolarizing_coefficients(oracle):
    # channel_test.clj:44-70: four operators; identity 1 - p, Paulis p/3; sum 1
    ops = oracle.kraus_channel({"noise-type": "depolarizing", "noise-strength": 0.0})
    assert len(ops) == 4 and _max_sq(ops[0]) == pytest.approx(1.0)
    assert all(_max_sq(m) == pytest.approx(0.0) for m in ops[1:])
    ops = oracle.kraus_channel({"noise-type": "depolarizing", "noise-strength": 0.1})
    assert _max_sq(ops[0]) == pytest.approx(0.9, abs=1e-10)
    assert _max_sq(ops[1]) == pytest.approx(0.1 / 3, abs=1e-10)
    ops = oracle.kraus_channel({"noise-type": "depolarizing", "noise-strength": 0.2})
    assert sum(_max_sq(m) for m in ops) == pytest.approx(1.0, abs=1e-10)
    with pytest.raises(ValueError):
        oracle.kraus_channel({"noise-type": "depolarizing", "noise-strength": 0.8})


def test_damping_coefficients(oracle):
    # channel_test.clj:72-131
    k0, k1 = oracle.kraus_channel({"noise-type": "amplitude-damping", "noise-strength": 0.0})
    assert abs(k0[0, 0]) ** 2 == pytest.approx(1) and abs(k0[1, 1]) ** 2 == pytest.approx(1)
    assert np.all(k1 == 0)
    k0, k1 = oracle.kraus_channel({"noise-type": "amplitude-damping", "noise-strength": 1.0})
    assert abs(k0[1, 1]) ** 2 == pytest.approx(0) and abs(k1[0, 1]) ** 2 == pytest.approx(1)
    k0, k1 = oracle.kraus_channel({"noise-type": "amplitude-damping", "noise-strength": 0.3})
    assert abs(k0[1, 1]) ** 2 == pytest.approx(0.7) and abs(k1[0, 1]) ** 2 == pytest.approx(0.3)
    k0, k1 = oracle.kraus_channel({"noise-type": "phase-damping", "noise-strength": 0.3})
    assert abs(k0[1, 1]) ** 2 == pytest.approx(0.7) and abs(k1[1, 1]) ** 2 == pytest.approx(0.3)
    # decoherence parameters (channel.clj:234-250): gamma = 1 - exp(-(gate_ns / 1000) / T)
    k0, _ = oracle.kraus_channel({"noise-type": "amplitude-damping", "t1-time": 100.0, "gate-time": 50.0})
    assert 1 - abs(k0[1, 1]) ** 2 == pytest.approx(1 - math.exp(-0.05 / 100.0))
    with pytest.raises(ValueError):  # (pos? gate-time)
        oracle.kraus_channel({"noise-type": "phase-damping", "t2-time": 150.0, "gate-time": 0.0})


def test_coherent_operator(oracle):
    # channel_test.clj:133-151: X rotation diagonal cos(t/2); Z "rotation" cos(t), cos(-t)
    (m,) = oracle.kraus_channel({"noise-type": "coherent",
                                 "coherent-error": {"rotation-angle": math.pi / 4, "rotation-axis": "x"}})
    assert m[0, 0].real == pytest.approx(math.cos(math.pi / 8)) and m[1, 1].real == pytest.approx(math.cos(math.pi / 8))
    (m,) = oracle.kraus_channel({"noise-type": "coherent",
                                 "coherent-error": {"rotation-angle": math.pi / 6, "rotation-axis": "z"}})
    assert m[0, 0].real == pytest.approx(math.cos(math.pi / 6)) and m[1, 1].real == pytest.approx(math.cos(math.pi / 6))
    assert oracle.kraus_channel({"noise-type": "unknown"}) is None


def test_channel_choice_rule(oracle):
    # zero noise always keeps the identity (channel_test.clj:236-243); damping channels'
    # first operator has max |K|^2 = 1, so the draw (< 1) always selects it
    ops = oracle.kraus_channel({"noise-type": "depolarizing", "noise-strength": 0.0})
    assert all(oracle.choose_kraus(ops, u) == 0 for u in np.linspace(0, 1, 101, endpoint=False))
    ops = oracle.kraus_channel({"noise-type": "amplitude-damping", "noise-strength": 0.9})
    assert all(oracle.choose_kraus(ops, u) == 0 for u in np.linspace(0, 1, 101, endpoint=False))
    ops = oracle.kraus_channel({"noise-type": "depolarizing", "noise-strength": 0.6})
    assert [oracle.choose_kraus(ops, u) for u in (0.1, 0.39, 0.41, 0.61, 0.81, 0.999)] == [0, 0, 1, 2, 3, 3]


def test_depolarizing_average_fidelity(oracle):
    # channel_test.clj:245-255: p = 0.6 on |0>, mean |<0|psi>| within [0.45, 0.65]
    c = {"num-qubits": 1, "operations": [{"operation-type": "x", "operation-params": {"target": 0}}]}
    nm = {"gate-noise": {"x": {"noise-type": "depolarizing", "noise-strength": 0.6}}}
    _, states = oracle.noisy_shots(c, nm, 400, seed=3)
    fid = np.mean(np.abs(states[:, 1]))  # overlap with the clean result X|0> = |1>
    assert 0.45 < fid < 0.65


def test_readout_noise(oracle):
    # noise_test.clj:87-106
    assert oracle.readout_noise(0b10, 2, None, 1, 0) == 0b10
    ro0 = {"prob-0-to-1": 0.0, "prob-1-to-0": 0.0}
    assert all(oracle.readout_noise(0b10, 2, ro0, 1, s) == 0b10 for s in range(50))
    ro1 = {"prob-0-to-1": 1.0, "prob-1-to-0": 1.0}
    assert all(oracle.readout_noise(0b10, 2, ro1, 1, s) == 0b01 for s in range(50))
    # a factor > 1 from an earlier flipped qubit raises the later qubit's flip rate;
    # correlations from out-of-range or later qubits have no effect (noise_test.clj:108-196)
    base = {"prob-0-to-1": 0.3, "prob-1-to-0": 0.3}
    corr = dict(base, **{"correlated-errors": {0: {1: 3.0}, 1: {0: 100.0}, 7: {1: 0.0}}})
    flips = lambda ro: sum(((oracle.readout_noise(0, 2, ro, 9, s) >> 0) & 1) for s in range(2000))
    assert flips(corr) > 1.5 * flips(base)


def test_noisy_shots_without_noise_are_ideal(oracle):
    from qclojure_gb300 import workloads

    c = workloads.layered_circuit(5, 4, seed=2)
    outs, states = oracle.noisy_shots(c, {}, 20, seed=4)
    ref = oracle.run(c)
    assert np.all(np.abs(states - ref) <= 1e-15)
    assert [int(o) for o in outs] == [int(oracle.lib().or_sample_one(
        oracle._dp(ref), 5, 4, s, 2)) for s in range(20)]


def test_shot_statistics_match_the_channel_mixture(oracle):
    """Over many shots the oracle's outcome frequency matches the mixture its channel
    defines: sum_k p_k |<0|K_k psi>|^2 / ||K_k psi||^2, then readout flips."""
    th = 0.7
    c = {"num-qubits": 1, "operations": [{"operation-type": "ry", "operation-params": {"target": 0, "angle": th}}]}
    p, p01, p10 = 0.3, 0.05, 0.1
    nm = {"gate-noise": {"ry": {"noise-type": "depolarizing", "noise-strength": p}},
          "readout-error": {"prob-0-to-1": p01, "prob-1-to-0": p10}}
    psi = np.array([math.cos(th / 2), math.sin(th / 2)], complex)
    probs = [1 - p, p / 3, p / 3, p / 3]
    mats = [np.eye(2), np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]]), np.diag([1, -1])]
    p0 = sum(w * abs((m @ psi)[0]) ** 2 / np.vdot(m @ psi, m @ psi).real for w, m in zip(probs, mats))
    want = p0 * (1 - p01) + (1 - p0) * p10
    shots = 20000
    outs, _ = oracle.noisy_shots(c, nm, shots, seed=17)
    got = float(np.mean(outs == 0))
    assert abs(got - want) <= 4 * math.sqrt(want * (1 - want) / shots)
