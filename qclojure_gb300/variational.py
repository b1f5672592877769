"""The variational loop as a client of batched sweeps.

The reference evaluates a variational objective one circuit at a time
(variational-hamiltonian-objective, application/algorithm/variational_algorithm.clj:310-363)
and forms parameter-shift gradients from 2N such evaluations
(parameter-shift-gradient and calculate-parameter-shift-gradient,
application/algorithm/optimization.clj:149-179, :270-298). Here every batch of
parameter vectors a step needs (the new point and its 2N shifted points) is one sweep
of equal-structure circuits (`qg_sweep_*`): one launch per HBM pass over all states,
energies reduced on the device, and new angles only rewrite the op records of the
sweep kept from the previous step.

The optimisers follow optimization.clj's loops (adam-optimization :309-365,
gradient-descent-optimization :367-420, spsa-optimization :463-567) step for step:
same updates, same convergence test, same result maps. The adaptive-shift gradients
(:181-262) evaluate every candidate shift in one batch. The gradient at each new point is computed in
the same batch as the point's energy; when the loop stops there, that gradient is the
`final-gradient`, and the extra evaluations are not counted.
"""
from __future__ import annotations

import math
from typing import Callable, Sequence

import numpy as np

from . import _abi as A
from .sweep import Sweep

DEFAULT_SHIFT = math.pi / 4  # variational_algorithm.clj:410 (:gradient-shift default)


class BatchedObjective:
    """Energies <H> of circuit_fn(params) for many parameter vectors at once."""

    def __init__(self, ctx, hamiltonian: list[dict], circuit_fn: Callable[[Sequence[float]], dict],
                 precision: str = "c128", arithmetic: str = "double-float"):
        self.ctx = ctx
        self.hamiltonian = hamiltonian
        self.circuit_fn = circuit_fn
        self.precision, self.arithmetic = precision, arithmetic
        self._sweeps: dict[int, Sweep] = {}
        self.evaluations = 0
        self.batches = 0
        self.device_ms = 0.0

    def energies(self, params_list: Sequence[Sequence[float]]) -> np.ndarray:
        circuits = [self.circuit_fn(list(p)) for p in params_list]
        k = len(circuits)
        sw = self._sweeps.get(k)
        if sw is not None:
            try:
                sw.update(circuits)
            except A.QgError as e:  # a value-dependent form changed the pass structure
                if e.code != A.QG_ERR_INVALID_ARG:
                    raise
                sw.close()
                sw = None
        if sw is None:
            sw = Sweep(self.ctx, circuits, self.precision, self.arithmetic)
            self._sweeps[k] = sw
        en, st = sw.run([self.hamiltonian] * k)
        self.evaluations += k
        self.batches += 1
        self.device_ms += st["device-ms"] + st["expect-ms"]
        return en

    def __call__(self, params: Sequence[float]) -> float:
        return float(self.energies([params])[0])

    def close(self):
        for sw in self._sweeps.values():
            sw.close()
        self._sweeps.clear()


def shifted_points(params: Sequence[float], shift: float) -> list[list[float]]:
    """θ + s e_i, θ - s e_i for every i (optimization.clj:171-174)."""
    pts = []
    for i in range(len(params)):
        plus, minus = list(params), list(params)
        plus[i] += shift
        minus[i] -= shift
        pts += [plus, minus]
    return pts


def gradient_from_energies(e_shifted: np.ndarray, shift: float) -> np.ndarray:
    """(E+ - E-) / (2 sin s) per parameter (optimization.clj:175-179)."""
    coef = 1.0 / (2.0 * math.sin(shift))
    return coef * (np.asarray(e_shifted[0::2]) - np.asarray(e_shifted[1::2]))


def parameter_shift_gradient(objective, params: Sequence[float], shift: float = DEFAULT_SHIFT) -> np.ndarray:
    """calculate-parameter-shift-gradient with all 2N evaluations in one batch."""
    return gradient_from_energies(objective.energies(shifted_points(params, shift)), shift)


def _energy_and_gradient(objective, params, options):
    """E(θ) and ∇E(θ) from one batch of 2N + 1 circuits: parameter-shift points
    (:gradient-method :parameter-shift, the method variational-optimization passes,
    variational_algorithm.clj:733) or central differences with step h
    (finite-difference-gradient, optimization.clj:125-147)."""
    if options.get("gradient-method", "parameter-shift") == "finite-difference":
        h = options.get("gradient-step-size", 1e-6)
        e = objective.energies([list(params)] + shifted_points(params, h))
        return float(e[0]), (np.asarray(e[1:][0::2]) - np.asarray(e[1:][1::2])) / (2.0 * h)
    shift = options.get("shift", DEFAULT_SHIFT)
    e = objective.energies([list(params)] + shifted_points(params, shift))
    return float(e[0]), gradient_from_energies(e[1:], shift)


def adam_optimization(objective, initial_parameters: Sequence[float], options: dict | None = None) -> dict:
    """adam-optimization (optimization.clj:309-365) with batched parameter-shift gradients."""
    o = options or {}
    lr = o.get("learning-rate", 0.001)
    max_iter = o.get("max-iterations", 500)
    tol = o.get("tolerance", 1e-6)
    b1, b2, eps = o.get("beta1", 0.9), o.get("beta2", 0.999), o.get("epsilon", 1e-8)
    nparam = len(initial_parameters)
    params = np.array(initial_parameters, float)
    m = np.zeros(nparam)
    v = np.zeros(nparam)
    energy, grad = _energy_and_gradient(objective, params, o)
    energies = [energy]
    it = 1
    while True:
        if it >= max_iter:
            return {"success": False, "optimal-parameters": list(params), "optimal-energy": energy,
                    "iterations": it, "function-evaluations": it * nparam * 2, "convergence-history": energies,
                    "reason": "max-iterations-reached"}
        m = b1 * m + (1 - b1) * grad
        v = b2 * v + (1 - b2) * grad * grad
        mc = m / (1 - b1 ** it)
        vc = v / (1 - b2 ** it)
        params = params - lr * (mc / (np.sqrt(vc) + eps))
        used = grad
        new_energy, grad = _energy_and_gradient(objective, params, o)
        diff = abs(energy - new_energy)
        energies.append(new_energy)
        energy = new_energy
        if diff < tol:
            return {"success": True, "optimal-parameters": list(params), "optimal-energy": new_energy,
                    "iterations": it, "function-evaluations": it * nparam * 2, "convergence-history": energies,
                    "final-gradient": list(used), "reason": "converged"}
        it += 1


def gradient_descent_optimization(objective, initial_parameters: Sequence[float], options: dict | None = None) -> dict:
    """gradient-descent-optimization (optimization.clj:367-420): momentum, learning rate
    reduced by 0.8 whenever the energy rises; batched parameter-shift gradients."""
    o = options or {}
    lr = o.get("learning-rate", 0.01)
    max_iter = o.get("max-iterations", 500)
    tol = o.get("tolerance", 1e-6)
    adaptive = o.get("adaptive-learning-rate", True)
    momentum = o.get("momentum", 0.9)
    nparam = len(initial_parameters)
    params = np.array(initial_parameters, float)
    vel = np.zeros(nparam)
    energy, grad = _energy_and_gradient(objective, params, o)
    energies = [energy]
    it = 0
    while True:
        if it >= max_iter:
            return {"success": False, "optimal-parameters": list(params), "optimal-energy": energy,
                    "iterations": it, "function-evaluations": it * nparam * 2, "convergence-history": energies,
                    "reason": "max-iterations-reached"}
        vel = momentum * vel + lr * grad
        params = params - vel
        used = grad
        new_energy, grad = _energy_and_gradient(objective, params, o)
        diff = abs(energy - new_energy)
        if adaptive and new_energy > energy:
            lr *= 0.8
        energies.append(new_energy)
        energy = new_energy
        if diff < tol:
            return {"success": True, "optimal-parameters": list(params), "optimal-energy": new_energy,
                    "iterations": it, "function-evaluations": it * nparam * 2, "convergence-history": energies,
                    "final-gradient": list(used), "reason": "converged"}
        it += 1


ADAPTIVE_SHIFTS = (math.pi / 2, math.pi / 4, math.pi / 8, math.pi / 16)


def adaptive_parameter_shift_gradient(objective, params: Sequence[float], param_types: Sequence[str]) -> np.ndarray:
    """adaptive-parameter-shift-gradient (optimization.clj:181-205): shift π/4 for an
    "amplitude" parameter and π/2 for any other type, all 2N evaluations in one batch.
    Parameters pair with types by position; the shorter list sets the gradient's length."""
    n = min(len(params), len(param_types))
    shifts = [math.pi / 4 if param_types[i] == "amplitude" else math.pi / 2 for i in range(n)]
    pts = []
    for i in range(n):
        plus, minus = list(params), list(params)
        plus[i] += shifts[i]
        minus[i] -= shifts[i]
        pts += [plus, minus]
    e = objective.energies(pts) if pts else np.zeros(0)
    return np.array([(1.0 / (2.0 * math.sin(shifts[i]))) * (e[2 * i] - e[2 * i + 1]) for i in range(n)])


def _max_key_abs(values: Sequence[float]) -> int:
    """Index `(apply max-key #(Math/abs %) values)` picks: of two, the first only when
    strictly larger; after that, a later value whenever it is at least as large."""
    best = 0
    if len(values) > 1:
        best = 0 if abs(values[0]) > abs(values[1]) else 1
        for k in range(2, len(values)):
            if abs(values[k]) >= abs(values[best]):
                best = k
    return best


def adaptive_shift_gradient(objective, params: Sequence[float], options: dict | None = None) -> np.ndarray:
    """calculate-adaptive-shift-gradient with select-best-shift (optimization.clj:207-262):
    per parameter, the parameter-shift gradient at the candidate shift whose gradient is
    largest in magnitude. All 2·N·S evaluations (S candidate shifts, default π/2, π/4,
    π/8, π/16) run as one batch; the gradient at the chosen shift is the one already
    evaluated, as the objective is deterministic."""
    shifts = list((options or {}).get("candidate-shifts", ADAPTIVE_SHIFTS))
    n = len(params)
    if n == 0 or not shifts:
        return np.zeros(0)
    e = objective.energies([pt for sh in shifts for pt in shifted_points(params, sh)])
    per = [gradient_from_energies(e[2 * n * k:2 * n * (k + 1)], sh) for k, sh in enumerate(shifts)]
    return np.array([per[_max_key_abs([g[i] for g in per])][i] for i in range(n)])


def spsa_optimization(objective, initial_parameters: Sequence[float], options: dict | None = None) -> dict:
    """spsa-optimization (optimization.clj:463-567): gains a_k = a / (A + k)^α and
    c_k = c / k^γ, a Bernoulli ±1 perturbation Δ of all parameters, the gradient estimate
    (E(θ + c_k Δ) - E(θ - c_k Δ)) / (2 c_k) · Δ, and the step θ - a_k ĝ; with a blocking
    size above 1 the last iterates are averaged and the average evaluated. Convergence
    needs more than 50 iterations and an energy change below the tolerance. The
    perturbations come from a generator seeded by the "seed" option (the reference draws
    from an unseeded `rand`). Each iteration is one batch: the new point (and its average)
    with the next iteration's two perturbed points, which depend only on the new point and
    the next draws."""
    o = options or {}
    a, c = o.get("a", 0.16), o.get("c", 0.1)
    max_iter = o.get("max-iterations", 1000)
    big_a = o.get("A", 0.1 * max_iter)
    alpha, gamma = o.get("alpha", 0.602), o.get("gamma", 0.101)
    tol = o.get("tolerance", 1e-6)
    block = o.get("blocking-size", 1)
    rng = np.random.default_rng(o.get("seed", 0))
    hyper = {"a": a, "c": c, "A": big_a, "alpha": alpha, "gamma": gamma}

    def probe(params, k):
        ck = c / math.pow(k, gamma)
        delta = [-1.0 if rng.random() < 0.5 else 1.0 for _ in params]
        return ck, delta, [p + ck * d for p, d in zip(params, delta)], [p - ck * d for p, d in zip(params, delta)]

    params = [float(x) for x in initial_parameters]
    nxt = probe(params, 1)
    e = objective.energies([params, nxt[2], nxt[3]])
    prev, ep, em = float(e[0]), float(e[1]), float(e[2])
    energies, blocked = [prev], [params]
    it = 0
    while True:
        if it >= max_iter:
            return {"success": False, "optimal-parameters": params, "optimal-energy": prev, "iterations": it,
                    "function-evaluations": it * 2, "convergence-history": energies,
                    "spsa-hyperparameters": hyper, "reason": "max-iterations-reached"}
        k = it + 1
        ak = a / math.pow(big_a + k, alpha)
        ck, delta = nxt[0], nxt[1]
        coef = (ep - em) / (2.0 * ck)
        new = [p - ak * (coef * d) for p, d in zip(params, delta)]
        blocked.append(new)
        recent = blocked[-block:] if block > 0 else []
        avg = ([sum(col) / len(col) for col in zip(*recent)] if block > 1 else new)
        nxt = probe(new, k + 1)
        batch = [new] + ([avg] if block > 1 else []) + [nxt[2], nxt[3]]
        e = objective.energies(batch)
        new_e = float(e[0])
        avg_e = float(e[1]) if block > 1 else new_e
        ep, em = float(e[-2]), float(e[-1])
        energies.append(new_e)
        if it > 50 and abs(prev - avg_e) < tol:
            return {"success": True, "optimal-parameters": avg, "optimal-energy": avg_e, "iterations": it,
                    "function-evaluations": it * 2 + (1 if block > 1 else 0), "convergence-history": energies,
                    "spsa-hyperparameters": {**hyper, "final-ak": ak, "final-ck": ck}, "reason": "converged"}
        params, prev = new, avg_e
        it += 1


def qaoa_maxcut_circuit(n: int, edges: Sequence[tuple[int, int]], params: Sequence[float]) -> dict:
    """H on every qubit, then per layer RZZ(2γ) on each edge and RX(2β) on each qubit;
    params = [γ_1, β_1, γ_2, β_2, ...]."""
    ops = [{"operation-type": "h", "operation-params": {"target": q}} for q in range(n)]
    for layer in range(len(params) // 2):
        g, b = params[2 * layer], params[2 * layer + 1]
        for a, c in edges:
            ops.append({"operation-type": "rzz", "operation-params": {"qubit1": a, "qubit2": c, "angle": 2.0 * g}})
        for q in range(n):
            ops.append({"operation-type": "rx", "operation-params": {"target": q, "angle": 2.0 * b}})
    return {"num-qubits": n, "operations": ops}
