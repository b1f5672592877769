"""Device maps (domain/device.clj): normalisation and the small queries over them.

A device is the reference's map with string keys ("native-gates", "virtual-gates",
"supported-operations", "coupling", "topology", "noise-model", "performance").
"""
from __future__ import annotations


def supported_operations(device: dict):
    """supported-operations (device.clj:50-55): the device's own set, or the union of its
    native and virtual gates when it has none (nil counts as none)."""
    own = device.get("supported-operations")
    if own is not None:
        return own
    return frozenset(device.get("native-gates") or ()) | frozenset(device.get("virtual-gates") or ())


def validate_device(device: dict) -> dict:
    """validate-device (device.clj:57-68): adds the supported operations and, when the
    device names only a topology, the coupling that topology has for its qubit count."""
    from .topology import coupling_for_topology

    coupling = device.get("coupling")
    if coupling is None and device.get("topology") is not None:
        coupling = coupling_for_topology(device["topology"], device.get("num-qubits"))
    return {**device, "supported-operations": supported_operations(device), "coupling": coupling}


def validate_devices(devices) -> list[dict]:
    """validate-devices (device.clj:70-73)."""
    return [validate_device(d) for d in devices]


def noise_model(device: dict) -> dict:
    """noise-model (device.clj:75-83)."""
    return device.get("noise-model", {})


def gate_fidelity(device: dict):
    """gate-fidelity (device.clj:85-96): the first of the performance map's gate,
    two-qubit and single-qubit fidelities that is set, else None."""
    perf = device.get("performance") or {}
    for key in ("gate-fidelity", "two-qubit-gate-fidelity", "single-qubit-gate-fidelity"):
        v = perf.get(key)
        if v is not None and v is not False:
            return v
    return None


def estimated_fidelity(device: dict, gate_count):
    """estimated-fidelity (device.clj:98-112): fidelity^count for a positive count."""
    f = gate_fidelity(device) if device else None
    if f is None or not device or gate_count is None or gate_count <= 0:
        return None
    return f ** gate_count


def validate_circuit(device: dict, circuit: dict) -> dict:
    """validate-circuit (device.clj:114-135): the circuit's operation types the device's
    "supported-operations" lacks (a device without that key supports nothing)."""
    sup = device.get("supported-operations") or frozenset()
    seen = []
    for op in circuit.get("operations") or []:
        t = op.get("operation-type")
        if t not in seen:
            seen.append(t)
    missing = [t for t in seen if t not in sup]
    return {"all-gates-supported?": not missing, "unsupported-gates": missing}


def compare_gate_support(device1: dict, device2: dict) -> dict:
    """compare-gate-support (device.clj:137-159)."""
    a = frozenset(device1.get("supported-operations") or ())
    b = frozenset(device2.get("supported-operations") or ())
    return {"device1-operations": device1.get("supported-operations"),
            "device2-operations": device2.get("supported-operations"),
            "shared-operations": a & b, "device1-only": a - b, "device2-only": b - a,
            "total-unique-operations": a | b}
