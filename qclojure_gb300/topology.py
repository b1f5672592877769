"""Hardware topologies and topology-aware routing: the pipeline stage of the reference's
domain/topology.clj, restated.

Couplings are adjacency lists (`coupling[q]` = the qubits q connects to). Routing maps
logical qubits to physical ones and, before a two-qubit operation whose qubits are not
adjacent, inserts SWAPs that move the control next to the target. The restatement keeps
the reference's behaviour where it is surprising: the mapping search tries only the n
cyclic offsets for circuits of up to 8 qubits and the identity beyond; after inserting
SWAPs the routing keeps using its initial mapping; a routed two-qubit operation keeps only
its control and target; and when the device has a native SWAP the stage returns the
routing result in place of the pipeline context (topology.clj:723-790).
"""
from __future__ import annotations

import math
from collections import deque

INT_MAX = 2**31 - 1  # Integer/MAX_VALUE: no path
SUPPORTED_TOPOLOGIES = frozenset({"fully-connected", "linear", "ring", "star", "grid", "heavy-hex", "custom"})
_QUBIT_KEYS = ("target", "control", "qubit1", "qubit2", "control1", "control2", "target1", "target2")


class TopologyError(ValueError):
    """Raised where the reference throws from its topology functions."""


# ---------------------------------------------------------------------------
# couplings (topology.clj:27-235)
# ---------------------------------------------------------------------------
def ensure_symmetric_coupling(coupling: list) -> list:
    n = len(coupling)
    out = []
    for i in range(n):
        nb = set(coupling[i]) if i < n else set()
        nb |= {j for j in range(n) if i in coupling[j]}
        out.append(sorted(x for x in nb if x != i))
    return out


def fully_connected_coupling(n: int) -> list:
    return [[j for j in range(n) if j != i] for i in range(n)]


def linear_coupling(n: int) -> list:
    if n < 1:
        return []
    if n == 1:
        return [[]]
    return [[1] if i == 0 else [i - 1] if i == n - 1 else [i - 1, i + 1] for i in range(n)]


def ring_coupling(n: int) -> list:
    if n < 3:
        return linear_coupling(n)
    return [[(i - 1) % n, (i + 1) % n] for i in range(n)]


def octagonal_coupling(n: int) -> list:
    if n != 8:
        raise TopologyError("Assert failed: (= num-qubits 8)")
    return ring_coupling(8)


def star_coupling(n: int) -> list:
    if n < 1:
        return []
    if n == 1:
        return [[]]
    return [list(range(1, n))] + [[0] for _ in range(n - 1)]


def grid_coupling(rows: int, cols: int) -> list:
    out = []
    for i in range(rows * cols):
        r, c = divmod(i, cols)
        nb = []
        if r > 0:
            nb.append(i - cols)
        if r < rows - 1:
            nb.append(i + cols)
        if c > 0:
            nb.append(i - 1)
        if c < cols - 1:
            nb.append(i + 1)
        out.append(nb)
    return out


def heavy_hex_coupling(n: int) -> list:
    """The 7-qubit unit (topology.clj:158-203); other sizes are refused, as there."""
    if n != 7:
        raise TopologyError("Assert failed: (#{7} num-qubits)")
    return ensure_symmetric_coupling([[1], [0, 2, 6], [1, 3], [2, 4], [3, 5], [4, 6], [5, 1]])


def coupling_for_topology(topology: str, n: int) -> list:
    t = str(topology).lstrip(":")
    if t in ("fully-connected", "all-to-all"):
        return fully_connected_coupling(n)
    if t == "linear":
        return linear_coupling(n)
    if t == "ring":
        return ring_coupling(n)
    if t == "octagonal":
        return octagonal_coupling(n)
    if t == "star":
        return star_coupling(n)
    if t == "grid":
        side = int(math.sqrt(n))
        return grid_coupling(side, 0 if side == 0 else int(math.ceil(n / side)))
    if t == "heavy-hex":
        return heavy_hex_coupling(n)
    raise TopologyError("Unsupported topology type")


def validate_coupling(coupling) -> bool:
    """No self-connections; every neighbour exists and lists the qubit back
    (topology.clj:237-262)."""
    if not isinstance(coupling, (list, tuple)) or not all(isinstance(c, (list, tuple)) for c in coupling):
        return False
    n = len(coupling)
    if any(q in coupling[q] for q in range(n)):  # no qubit connects to itself
        return False
    return all(nb < n and q in coupling[nb] for q in range(n) for nb in coupling[q])


# ---------------------------------------------------------------------------
# distances, paths, mapping (topology.clj:264-484)
# ---------------------------------------------------------------------------
def _bfs_path(coupling: list, start, end):
    if start == end:
        return [start]
    q, seen = deque([(start, [start])]), {start}
    while q:
        cur, path = q.popleft()
        if cur == end:
            return path
        nxt = [x for x in (coupling[cur] if isinstance(cur, int) and 0 <= cur < len(coupling) else [])
               if x not in seen]
        for x in nxt:
            q.append((x, path + [x]))
        seen.update(nxt)
    return None


def calculate_distance_matrix(coupling: list) -> list:
    n = len(coupling)
    out = []
    for i in range(n):
        row = []
        for j in range(n):
            p = _bfs_path(coupling, i, j)
            row.append(INT_MAX if p is None else len(p) - 1)
        out.append(row)
    return out


def find_shortest_path(coupling: list, start, end):
    return _bfs_path(coupling, start, end)


def extract_two_qubit_operations(circuit: dict) -> list:
    out = []
    for op in circuit.get("operations") or []:
        p = op.get("operation-params") or {}
        g = op.get("operation-type")
        if p.get("control") is not None and p.get("target") is not None:
            out.append({"control": p["control"], "target": p["target"], "operation-type": g})
        elif p.get("control1") is not None and p.get("target") is not None:
            out.append({"control": p["control1"], "target": p["target"], "operation-type": g})
        elif p.get("target1") is not None and p.get("target2") is not None:
            out.append({"control": p["target1"], "target": p["target2"], "operation-type": g})
        elif p.get("swap1") is not None and p.get("swap2") is not None:
            out.append({"control": p["swap1"], "target": p["swap2"], "operation-type": g})
    return out


def calculate_mapping_cost(ops: list, mapping: dict, dist: list) -> int:
    total = 0
    for op in ops:
        pc, pt = mapping.get(op["control"]), mapping.get(op["target"])
        total = total + dist[pc][pt] if pc is not None and pt is not None else INT_MAX
    return total


def generate_swap_operations(path: list, moved_qubit) -> list:
    if len(path) <= 2:
        return []
    return [{"operation-type": "swap", "operation-params": {"target1": a, "target2": b},
             "routing-info": {"moves-qubit": moved_qubit, "from": a, "to": b}} for a, b in zip(path, path[1:])]


def find_optimal_mapping_for_operations(ops: list, n_logical: int, n_physical: int, dist: list) -> dict:
    if n_logical > n_physical:
        raise TopologyError("Circuit requires more qubits than available in topology")
    if n_logical == 0:
        return {}
    if n_logical <= 8:
        cands = [{q: (q + off) % n_physical for q in range(n_logical)} for off in range(n_physical)]
        return sorted(cands, key=lambda m: calculate_mapping_cost(ops, m, dist))[0]
    return {q: q for q in range(n_logical)}


def find_optimal_mapping(circuit: dict, coupling: list, dist: list) -> dict:
    return find_optimal_mapping_for_operations(extract_two_qubit_operations(circuit), circuit["num-qubits"],
                                               len(coupling), dist)


def update_operation_params(op: dict, fn) -> dict:
    """circuit_composition.clj:16-47: remap every qubit parameter."""
    p = op.get("operation-params")
    if p is None:
        return op
    out = {}
    for k, v in p.items():
        if k in _QUBIT_KEYS:
            out[k] = fn(v)
        elif k == "measurement-qubits":
            out[k] = [fn(x) for x in v]
        else:
            out[k] = v
    return {**op, "operation-params": out}


def _clj_map(m: dict) -> str:
    return "{" + ", ".join(f"{k} {v}" for k, v in m.items()) + "}"


def optimize_for_coupling(circuit: dict, coupling: list, options: dict | None = None) -> dict:
    """optimize-for-coupling (topology.clj:486-623)."""
    o = options or {}
    if not validate_coupling(coupling):
        raise TopologyError("Assert failed: (validate-coupling coupling)")
    dist = calculate_distance_matrix(coupling)
    n = circuit["num-qubits"]
    l2p = find_optimal_mapping(circuit, coupling, dist) if o.get("optimize-mapping?", True) \
        else {q: q for q in range(n)}
    p2l = {p: l for l, p in l2p.items()}
    ops = circuit.get("operations") or []
    if o.get("insert-swaps?", True):
        result, swaps, cur = [], 0, l2p  # the routing never updates its mapping after SWAPs
        for op in ops:
            p = op.get("operation-params") or {}
            if p.get("control") is not None and p.get("target") is not None:
                pc, pt = cur.get(p["control"]), cur.get(p["target"])
                d = dist[pc][pt] if pc is not None and pt is not None else INT_MAX
                if d > 1:
                    path = find_shortest_path(coupling, pc, pt)
                    adj = path[-2] if path and len(path) >= 2 else None
                    sp = find_shortest_path(coupling, pc, adj) if adj is not None else None
                    if sp and len(sp) > 2:
                        sw = generate_swap_operations(sp, p["control"])
                    elif sp and len(sp) == 2:
                        sw = [{"operation-type": "swap", "operation-params": {"target1": sp[0], "target2": sp[1]},
                               "routing-info": {"moves-qubit": p["control"], "from": sp[0], "to": sp[1]}}]
                    else:
                        sw = []
                    swaps += len(sw)
                    result += sw
                    result.append({"operation-type": op.get("operation-type"),
                                   "operation-params": {"control": adj, "target": pt}})
                else:
                    result.append({"operation-type": op.get("operation-type"),
                                   "operation-params": {"control": pc, "target": pt}})
            else:
                result.append(update_operation_params(op, lambda q: cur.get(q, q)))
    else:
        result, swaps = [update_operation_params(op, lambda q: l2p.get(q, q)) for op in ops], 0
    cost = calculate_mapping_cost(extract_two_qubit_operations(circuit), l2p, dist)
    summary = ("Topology optimization summary:\n"
               f"- Hardware qubits: {len(coupling)}\n"
               f"- Logical qubits: {n}\n"
               f"- Qubit mapping: {_clj_map(l2p)}\n"
               f"- SWAP operations added: {swaps}\n"
               f"- Total routing cost: {cost}")
    return {"circuit": {**circuit, "operations": result}, "logical-to-physical": l2p, "physical-to-logical": p2l,
            "swap-count": swaps, "total-cost": cost, "topology-summary": summary}


# ---------------------------------------------------------------------------
# analysis (topology.clj:625-721)
# ---------------------------------------------------------------------------
def analyze_coupling_connectivity(coupling: list) -> dict:
    n = len(coupling)
    if n <= 1:
        return {"num-qubits": n, "total-edges": 0, "avg-degree": 0, "max-degree": 0, "min-degree": 0,
                "diameter": 0, "is-connected": n == 1}
    deg = [len(c) for c in coupling]
    dist = calculate_distance_matrix(coupling)
    alld = [dist[i][j] for i in range(n) for j in range(n) if i != j]
    diameter = INT_MAX if INT_MAX in alld else max(alld)
    total = sum(deg) / 2
    return {"num-qubits": n, "total-edges": int(total) if total == int(total) else total,
            "avg-degree": sum(deg) / float(n), "max-degree": max(deg), "min-degree": min(deg),
            "diameter": diameter, "is-connected": diameter != INT_MAX}


def get_coupling_info(coupling: list, name: str = "Topology") -> str:
    a = analyze_coupling_connectivity(coupling)
    dia = "∞ (disconnected)" if a["diameter"] == INT_MAX else a["diameter"]
    return (f"{name} Analysis:\n- Qubits: {a['num-qubits']}\n- Edges: {a['total-edges']}\n"
            f"- Average degree: {a['avg-degree']:.2f}\n- Degree range: {a['min-degree']}-{a['max-degree']}\n"
            f"- Diameter: {dia}\n- Connected: {'true' if a['is-connected'] else 'false'}")


def compare_couplings(circuit: dict, topologies: dict) -> list:
    rows = []
    for name, coupling in topologies.items():
        r = optimize_for_coupling(circuit, coupling)
        rows.append({"topology-name": name, "total-cost": r["total-cost"], "swap-count": r["swap-count"],
                     "logical-to-physical": r["logical-to-physical"]})
    return sorted(rows, key=lambda x: x["total-cost"])


def topology_aware_transform(ctx: dict) -> dict:
    """topology-aware-transform (topology.clj:723-790)."""
    if not (ctx.get("options") or {}).get("optimize-topology?"):
        return ctx
    circuit, device = ctx["circuit"], ctx.get("device") or {}
    supported = device.get("supported-operations") or frozenset()
    coupling = device.get("coupling") or coupling_for_topology(device.get("topology"), device.get("num-qubits", 0))
    res = optimize_for_coupling(circuit, coupling, ctx.get("options"))
    if "swap" in supported:
        return res  # the routing result takes the context's place
    ops = []
    for op in res["circuit"]["operations"]:
        if op.get("operation-type") == "swap":
            p = op.get("operation-params") or {}
            a, b = p.get("target1"), p.get("target2")
            ops += [{"operation-type": "cnot", "operation-params": {"control": a, "target": b}},
                    {"operation-type": "cnot", "operation-params": {"control": b, "target": a}},
                    {"operation-type": "cnot", "operation-params": {"control": a, "target": b}}]
        else:
            ops.append(op)
    return {**ctx, "circuit": {**res["circuit"], "operations": ops},
            "logical-to-physical": res["logical-to-physical"], "physical-to-logical": res["physical-to-logical"],
            "swap-count": res["swap-count"], "total-cost": res["total-cost"]}
