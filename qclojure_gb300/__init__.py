"""GB300-native state-vector simulator backend for QClojure circuits.

The compute path is libqgpu.so (hand-written sm_103a CUDA behind the C ABI in
include/qgpu.h). This package holds the host side above that ABI: the circuit
model and encoder, the QuantumBackend protocol mirror, the device-state API
and the workload generators.
"""
from .circuit import (create_circuit, add_gate, bell_state_circuit, ghz_state_circuit, encode,  # noqa: F401
                      circuit_metadata, circuit_depth)

__all__ = ["create_circuit", "add_gate", "bell_state_circuit", "ghz_state_circuit", "encode",
           "circuit_metadata", "circuit_depth", "create_simulator", "GpuStateVectorSimulator"]


def __getattr__(name):
    if name in ("create_simulator", "GpuStateVectorSimulator", "execute_circuit"):
        from . import backend
        return getattr(backend, name)
    raise AttributeError(name)
