"""The variational client's host loops against plain restatements of the reference's
sequential loops (optimization.clj:181-262 adaptive shifts, :463-567 SPSA), on a
deterministic classical objective: the batching must not change a single number."""
import math

import numpy as np
import pytest

from qclojure_gb300 import variational as V


class FnObjective:
    def __init__(self, f):
        self.f, self.calls, self.batches = f, 0, 0

    def energies(self, pts):
        self.batches += 1
        self.calls += len(pts)
        return np.array([self.f(list(p)) for p in pts])

    def __call__(self, p):
        return float(self.energies([p])[0])


def landscape(p):
    return sum(math.cos(x + 0.3 * i) * (1 + 0.1 * i) for i, x in enumerate(p)) + 0.2 * math.sin(p[0] - p[-1])


def ps(f, p, i, s):
    a, b = list(p), list(p)
    a[i] += s
    b[i] -= s
    return (1.0 / (2.0 * math.sin(s))) * (f(a) - f(b))


def test_max_key_ties():
    assert V._max_key_abs([1.0]) == 0
    assert V._max_key_abs([2.0, -2.0]) == 1 and V._max_key_abs([3.0, 2.0]) == 0
    assert V._max_key_abs([3.0, 1.0, -3.0, 2.0]) == 2 and V._max_key_abs([1.0, 5.0, 2.0, 5.0]) == 3


def test_adaptive_gradients_match_the_sequential_rules():
    p = [0.4, -1.1, 2.0, 0.05]
    obj = FnObjective(landscape)
    g = V.adaptive_shift_gradient(obj, p)
    assert obj.batches == 1 and obj.calls == 2 * 4 * 4
    for i in range(4):
        cands = [ps(landscape, p, i, s) for s in V.ADAPTIVE_SHIFTS]
        best = V.ADAPTIVE_SHIFTS[V._max_key_abs(cands)]
        assert g[i] == ps(landscape, p, i, best)
    t = V.adaptive_parameter_shift_gradient(obj, p, ["rotation", "amplitude", "phase"])
    assert len(t) == 3 and t[1] == ps(landscape, p, 1, math.pi / 4) and t[2] == ps(landscape, p, 2, math.pi / 2)


def spsa_reference(f, init, o):
    """optimization.clj:463-567 one evaluation at a time, with the same seeded draws."""
    a, c, mi = o.get("a", 0.16), o.get("c", 0.1), o.get("max-iterations", 1000)
    A, al, ga, tol, bs = o.get("A", 0.1 * mi), o.get("alpha", 0.602), o.get("gamma", 0.101), o.get("tolerance", 1e-6), \
        o.get("blocking-size", 1)
    rng = np.random.default_rng(o.get("seed", 0))
    params, it, prev = list(init), 0, f(list(init))
    energies, blocked = [prev], [list(init)]
    while it < mi:
        k = it + 1
        ak, ck = a / math.pow(A + k, al), c / math.pow(k, ga)
        d = [-1.0 if rng.random() < 0.5 else 1.0 for _ in params]
        ep = f([x + ck * y for x, y in zip(params, d)])
        em = f([x - ck * y for x, y in zip(params, d)])
        gc = (ep - em) / (2.0 * ck)
        new = [x - ak * (gc * y) for x, y in zip(params, d)]
        ne = f(new)
        energies.append(ne)
        blocked.append(new)
        avg = [sum(col) / len(col) for col in zip(*blocked[-bs:])] if bs > 1 else new
        ae = f(avg) if bs > 1 else ne
        if it > 50 and abs(prev - ae) < tol:
            return {"success": True, "optimal-parameters": avg, "optimal-energy": ae, "iterations": it,
                    "convergence-history": energies}
        params, prev, it = new, ae, it + 1
    return {"success": False, "optimal-parameters": params, "optimal-energy": prev, "iterations": it,
            "convergence-history": energies}


@pytest.mark.parametrize("opts", [{"max-iterations": 80, "seed": 3},
                                  {"max-iterations": 400, "seed": 5, "tolerance": 1e-4},
                                  {"max-iterations": 300, "seed": 9, "blocking-size": 4, "tolerance": 1e-3}])
def test_spsa_matches_the_sequential_loop(opts):
    init = [0.4, -1.1, 2.0, 0.05, 1.3]
    obj = FnObjective(landscape)
    r = V.spsa_optimization(obj, init, opts)
    ref = spsa_reference(landscape, init, opts)
    for key in ("success", "optimal-parameters", "optimal-energy", "iterations", "convergence-history"):
        assert r[key] == ref[key], key
    assert r["function-evaluations"] == 2 * r["iterations"] + (1 if r["success"] and opts.get("blocking-size", 1) > 1
                                                                else 0)
    # one batch to start, then one per iteration run (the converging one included)
    assert obj.batches == 1 + r["iterations"] + (1 if r["success"] else 0)
