"""Seeded synthetic workloads of the benchmark shapes.

  layered_circuit   n qubits, depth d: every layer puts one gate drawn uniformly
                    from {H,X,Y,Z,S,T,RX,RY,RZ} (angles U[0, 2pi)) on each qubit,
                    then CNOTs on a random perfect matching with random
                    control/target order (10 qubits x 20 layers is the CPU case).
  qft_circuit       H plus controlled phase pi/2^k (:rydberg-cphase in the
                    reference gate set) and the final SWAPs.
  large_circuit     layered(30, 40) followed by qft(30).
  qaoa_maxcut       p-layer QAOA on a random 3-regular graph: H^n, then per layer
                    RZZ(2 gamma) on every edge and RX(2 beta) on every qubit, with
                    H_C = sum_edges (1 - Z_a Z_b) / 2.
  serving_trace     Poisson arrivals of layered jobs with n = 8 + Geometric(0.15)
                    (failures before the first success) capped at 28, depth
                    U{10..200}; 90 % request U{1k..100k} shots, 10 % the
                    expectation of a random Pauli string.
  ceiling_circuit   layers of {H,S,T,RZ} on every qubit then CZ on a random matching.
All generators take a seed and return circuits in the reference's map form.
"""
from __future__ import annotations

import math

import numpy as np

from . import circuit as qc

LAYER_GATES = ("h", "x", "y", "z", "s", "t", "rx", "ry", "rz")
CEILING_GATES = ("h", "s", "t", "rz")


def _layer(ops: list, n: int, rng: np.random.Generator, gates=LAYER_GATES, two_qubit="cnot"):
    for q in range(n):
        g = gates[rng.integers(len(gates))]
        if g in ("rx", "ry", "rz"):
            ops.append({"operation-type": g, "operation-params": {"target": q,
                                                                  "angle": float(rng.uniform(0, 2 * math.pi))}})
        else:
            ops.append({"operation-type": g, "operation-params": {"target": q}})
    perm = rng.permutation(n)
    for k in range(0, n - 1, 2):
        a, b = int(perm[k]), int(perm[k + 1])
        if rng.integers(2):
            a, b = b, a
        ops.append({"operation-type": two_qubit, "operation-params": {"control": a, "target": b}})


def layered_circuit(n: int, depth: int, seed: int, gates=LAYER_GATES, two_qubit: str = "cnot") -> dict:
    rng = np.random.default_rng(seed)
    ops: list = []
    for _ in range(depth):
        _layer(ops, n, rng, gates, two_qubit)
    return {"num-qubits": n, "operations": ops, "name": f"layered-{n}x{depth}-s{seed}"}


def qft_ops(n: int) -> list:
    ops = []
    for j in range(n):
        ops.append({"operation-type": "h", "operation-params": {"target": j}})
        for k in range(j + 1, n):
            ops.append({"operation-type": "rydberg-cphase",
                        "operation-params": {"control": k, "target": j, "angle": math.pi / (2 ** (k - j))}})
    for i in range(n // 2):
        ops.append({"operation-type": "swap", "operation-params": {"qubit1": i, "qubit2": n - 1 - i}})
    return ops


def qft_circuit(n: int) -> dict:
    return {"num-qubits": n, "operations": qft_ops(n), "name": f"qft-{n}"}


def large_circuit(n: int = 30, depth: int = 40, seed: int = 1) -> dict:
    c = layered_circuit(n, depth, seed)
    c["operations"] = c["operations"] + qft_ops(n)
    c["name"] = f"layered-{n}x{depth}+qft-s{seed}"
    return c


def ceiling_circuit(n: int, depth: int, seed: int) -> dict:
    return layered_circuit(n, depth, seed, gates=CEILING_GATES, two_qubit="cz")


def random_3_regular_graph(n: int, rng: np.random.Generator) -> list[tuple[int, int]]:
    """Pairing model with rejection (no self-loops, no repeated edges)."""
    assert n % 2 == 0 and n >= 4
    for _ in range(10_000):
        stubs = rng.permutation(np.repeat(np.arange(n), 3))
        edges = set()
        ok = True
        for k in range(0, len(stubs), 2):
            a, b = int(stubs[k]), int(stubs[k + 1])
            if a == b or (min(a, b), max(a, b)) in edges:
                ok = False
                break
            edges.add((min(a, b), max(a, b)))
        if ok:
            return sorted(edges)
    raise RuntimeError("no 3-regular graph found")


def qaoa_maxcut(n: int, p: int, seed: int) -> dict:
    rng = np.random.default_rng(seed)
    edges = random_3_regular_graph(n, rng)
    gammas = rng.uniform(0, math.pi, p)
    betas = rng.uniform(0, math.pi / 2, p)
    ops = [{"operation-type": "h", "operation-params": {"target": q}} for q in range(n)]
    for layer in range(p):
        for a, b in edges:
            ops.append({"operation-type": "rzz",
                        "operation-params": {"qubit1": a, "qubit2": b, "angle": float(2 * gammas[layer])}})
        for q in range(n):
            ops.append({"operation-type": "rx", "operation-params": {"target": q, "angle": float(2 * betas[layer])}})
    ham = []
    for a, b in edges:
        ham.append({"coefficient": 0.5, "pauli-string": "I" * n})
        zz = ["I"] * n
        zz[a] = "Z"
        zz[b] = "Z"
        ham.append({"coefficient": -0.5, "pauli-string": "".join(zz)})
    return {"num-qubits": n, "operations": ops, "name": f"qaoa-{n}-p{p}-s{seed}", "edges": edges,
            "gammas": gammas.tolist(), "betas": betas.tolist(), "hamiltonian": ham}


def qaoa_sweep(count: int = 1024, p: int = 3, seed: int = 7, n_choices=(12, 14, 16, 18, 20, 22, 24)) -> list[dict]:
    rng = np.random.default_rng(seed)
    ns = rng.choice(np.array(n_choices), size=count)
    return [qaoa_maxcut(int(n), p, seed * 100003 + i) for i, n in enumerate(ns)]


def serving_trace(num_jobs: int, rate_per_s: float, seed: int, max_qubits: int = 28) -> list[dict]:
    rng = np.random.default_rng(seed)
    t = 0.0
    jobs = []
    for j in range(num_jobs):
        t += float(rng.exponential(1.0 / rate_per_s))
        n = min(max_qubits, 8 + int(rng.geometric(0.15)) - 1)
        depth = int(rng.integers(10, 201))
        circ = layered_circuit(n, depth, seed * 1_000_003 + j)
        if rng.uniform() < 0.9:
            spec = {"measurements": {"shots": int(rng.integers(1000, 100_001))}}
        else:
            ps = "".join("IXYZ"[k] for k in rng.integers(0, 4, n))
            spec = {"hamiltonian": [{"coefficient": 1.0, "pauli-string": ps}]}
        jobs.append({"arrival-s": t, "circuit": circ, "result-specs": spec, "n": n, "depth": depth})
    return jobs
