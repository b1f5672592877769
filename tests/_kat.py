"""Shared checker for the reference known-answer cases (tests/golden/reference_kat.json).

An `Engine` supplies: final state for (n, initial basis index, operations, seed),
plus Pauli / Hamiltonian / observable expectations and seeded shot sampling on
that state. The oracle and the GPU backend are both checked through it.
"""
import json
from pathlib import Path

import numpy as np

KAT = json.loads((Path(__file__).parent / "golden" / "reference_kat.json").read_text())["cases"]


def cplx(v):
    return complex(v[0], v[1])


def matrix(m):
    return [[cplx(z) for z in row] for row in m]


def check_case(case, engine, seed=1234):
    n = case["num-qubits"]
    circuit = {"num-qubits": n, "operations": case["operations"]}
    state = engine.state(circuit, case["initial-basis"], seed)
    for chk in case["checks"]:
        k = chk["kind"]
        where = f"{case['name']} ({case['source']}) {k}"
        if k == "state_exact":
            exp = np.array([cplx(z) for z in chk["expected"]])
            assert np.array_equal(state, exp), where
        elif k == "state_close":
            exp = np.array([cplx(z) for z in chk["expected"]])
            assert np.max(np.abs(state - exp)) < chk["tol"], where
        elif k == "amp_close":
            d = abs(state[chk["index"]] - cplx(chk["value"]))
            assert (d == 0) if chk["tol"] == 0 else (d < chk["tol"]), where
        elif k == "amp_abs_close":
            assert abs(abs(state[chk["index"]]) - chk["value"]) < chk["tol"], where
        elif k == "amp_abs_lt":
            assert abs(state[chk["index"]]) < chk["value"], where
        elif k == "amp_abs_gt":
            assert abs(state[chk["index"]]) > chk["value"], where
        elif k == "amp_im_eq":
            assert state[chk["index"]].imag == chk["value"], where
        elif k == "norm_close":
            assert abs(np.sum(np.abs(state) ** 2) - 1.0) < chk["tol"], where
        elif k == "nonzero_count":
            assert int(np.sum(np.abs(state) > 1e-10)) == chk["value"], where
        elif k == "max_abs_close":
            assert abs(np.max(np.abs(state)) - chk["value"]) < chk["tol"], where
        elif k == "pauli_eq":
            v = engine.pauli(circuit, case["initial-basis"], seed, chk["pauli"])
            assert (v == chk["value"]) if chk["tol"] == 0 else abs(v - chk["value"]) < chk["tol"], where
        elif k == "ham_eq":
            v = engine.hamiltonian(circuit, case["initial-basis"], seed, chk["terms"])
            assert (v == chk["value"]) if chk["tol"] == 0 else abs(v - chk["value"]) < chk["tol"], where
        elif k == "obs_close":
            v = engine.expectation(circuit, case["initial-basis"], seed, matrix(chk["observable"]), chk["target"])
            assert abs(v - chk["value"]) < chk["tol"], where
        elif k == "var_close":
            v = engine.variance(circuit, case["initial-basis"], seed, matrix(chk["observable"]), chk["target"])
            assert abs(v - chk["value"]) < chk["tol"], where
        elif k == "counts_exact":
            counts = engine.counts(circuit, case["initial-basis"], seed, chk["shots"])
            assert counts == {int(o): c for o, c in chk["counts"].items()}, where
        elif k == "counts_ratio":
            counts = engine.counts(circuit, case["initial-basis"], seed, chk["shots"])
            assert set(counts) <= set(chk["allowed"]), where
            ratio = counts.get(chk["first"], 0) / chk["shots"]
            assert chk["lo"] < ratio < chk["hi"], where
        else:
            raise AssertionError(f"unknown check {k}")


def basis_state(n, idx):
    s = np.zeros(1 << n, np.complex128)
    s[idx] = 1
    return s
