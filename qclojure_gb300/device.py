"""Device normalisation (domain/device.clj:50-73), as the hardware simulator applies it to
a device map it is given (hardware_simulator.clj:409-414).

A device is the reference's map with string keys ("native-gates", "virtual-gates",
"supported-operations", "coupling", "topology", "num-qubits").
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
    device names only a topology, the coupling that topology has for its qubit count.
    A topology without a natural-number "num-qubits" fails, as the coupling builders'
    nat-int? preconditions make the reference fail."""
    from .topology import coupling_for_topology

    coupling = device.get("coupling")
    if coupling is None and device.get("topology") is not None:
        nq = device.get("num-qubits")
        if not isinstance(nq, int) or isinstance(nq, bool) or nq < 0:
            raise ValueError(f"device {device.get('id', device.get('name'))!r} has topology "
                             f"{device['topology']!r} but no natural-number num-qubits ({nq!r})")
        coupling = coupling_for_topology(device["topology"], nq)
    return {**device, "supported-operations": supported_operations(device), "coupling": coupling}


def validate_devices(devices) -> list[dict]:
    """validate-devices (device.clj:70-73)."""
    return [validate_device(d) for d in devices]
