"""Estimates over a noise model, without simulation (application/noise_analysis.clj).

These functions read the same noise-model maps the noisy trajectory runner takes
("gate-noise" per operation type with "noise-strength", "t1-time", ...; "readout-error")
and the circuit maps of `circuit.py`. They restate the reference's arithmetic and its
orders: gate counts and the error sum follow a Clojure map's iteration order (first
appearance for up to eight gate types, the keyword hash trie beyond), the dominant error
sources are a stable descending sort of that order, and the selective-mitigation
suggestion prints its lazy sequence of gate types the way `str` does (class name and hash
code, not the elements).
"""
from __future__ import annotations

import re

from .clj import hash_keyword, lazy_seq_of_keywords_str, map_order


def _check(circuit, noise_model) -> None:
    if not (isinstance(circuit, dict) and isinstance(circuit.get("num-qubits"), int)
            and isinstance(circuit.get("operations"), list)):
        raise ValueError("not a circuit")
    if not isinstance(noise_model, dict):
        raise ValueError("not a noise model")


def _strength(noise_model: dict, gate_type: str) -> float:
    return ((noise_model.get("gate-noise") or {}).get(gate_type) or {}).get("noise-strength", 0.0)


def gate_frequencies(circuit: dict) -> dict:
    """`(frequencies (map :operation-type ops))` in the map's iteration order."""
    counts: dict = {}
    for op in circuit["operations"]:
        t = op.get("operation-type")
        counts[t] = counts.get(t, 0) + 1
    return {k: counts[k] for k in map_order(list(counts), hash_keyword)}


def estimate_circuit_fidelity(circuit: dict, noise_model: dict) -> dict:
    """estimate-circuit-fidelity (noise_analysis.clj:24-56): the error is the sum over gate
    types of count x noise strength (0 for gates without an entry), the fidelity
    max(0, 1 - error)."""
    _check(circuit, noise_model)
    counts = gate_frequencies(circuit)
    total = 0.0
    for t, n in counts.items():
        total = total + n * _strength(noise_model, t)
    sources = sorted(((t, n * _strength(noise_model, t)) for t, n in counts.items()), key=lambda e: -e[1])
    return {"estimated-fidelity": max(0.0, 1.0 - total), "total-estimated-error": total,
            "gate-counts": counts, "dominant-error-sources": sources}


_PLATFORMS = [("ionq", "trapped-ion"), ("rigetti|ibm", "superconducting"), ("xanadu", "photonic"),
              ("quera", "neutral-atom")]


def compare_hardware_platforms(circuit: dict, platform_models: dict) -> dict:
    """compare-hardware-platforms (noise_analysis.clj:58-96): each platform's fidelity
    estimate with the coherence times of its first gate entry, its readout
    probabilities ("N/A" where absent) and a platform type found from its name."""
    if not isinstance(platform_models, dict):
        raise ValueError("platform models must be a map")
    out = {}
    for name, model in platform_models.items():
        data = estimate_circuit_fidelity(circuit, model)
        gn = model.get("gate-noise") or {}
        order = map_order(list(gn), hash_keyword)
        first = (gn[order[0]] if order else None) or {}
        ro = model.get("readout-error") or {}
        kind = next((k for pat, k in _PLATFORMS if re.search(pat, name)), "unknown")
        out[name] = {**data, "coherence-times": {"t1-time": first.get("t1-time", "N/A"),
                                                 "t2-time": first.get("t2-time", "N/A")},
                     "readout-fidelity": {"prob-0-to-1": ro.get("prob-0-to-1", "N/A"),
                                          "prob-1-to-0": ro.get("prob-1-to-0", "N/A")},
                     "platform-type": kind}
    return out


def noise_aware_circuit_depth(circuit: dict, noise_model: dict):
    """noise-aware-circuit-depth (noise_analysis.clj:98-119): the operation count plus
    count x (largest gate noise strength) x 10 when that strength is positive; an integer
    otherwise."""
    _check(circuit, noise_model)
    ops = circuit["operations"]
    strengths = [_strength(noise_model, op.get("operation-type")) for op in ops]
    top = max(strengths) if strengths else 0.0
    base = len(ops)
    return base + base * top * 10 if top > 0 else base


def recommend_error_mitigation(circuit: dict, noise_model: dict, options: dict | None = None) -> list[dict]:
    """recommend-error-mitigation (noise_analysis.clj:121-153): noise reduction below 0.95
    estimated fidelity, circuit cutting above 20 operations, selective mitigation when a
    gate type contributes more than 0.01."""
    _check(circuit, noise_model)
    data = estimate_circuit_fidelity(circuit, noise_model)
    dominant = data["dominant-error-sources"]
    recs = []
    if data["estimated-fidelity"] < 0.95:
        recs.append({"strategy": "noise-reduction", "reason": "Low estimated fidelity",
                     "suggestion": "Consider circuit optimization or shorter depth"})
    if len(circuit["operations"]) > 20:
        recs.append({"strategy": "circuit-cutting", "reason": "Deep circuit",
                     "suggestion": "Consider breaking circuit into smaller pieces"})
    if any(c > 0.01 for _, c in dominant):
        recs.append({"strategy": "selective-mitigation", "reason": "Specific gates dominate errors",
                     "suggestion": "Focus mitigation on: " + lazy_seq_of_keywords_str([t for t, _ in dominant])})
    return recs
