"""Noisy hardware simulation: the reference's hardware simulator with its shot loop run
as batched device trajectories.

The reference (src/org/soulspace/qclojure/adapter/backend/hardware_simulator.clj) runs
every shot as a fresh simulation: gate noise after each operation whose
:operation-type has an entry in the device's noise model (domain/noise.clj:53-102,
domain/channel.clj:40-232), one sampled outcome, readout noise (noise.clj:107-202),
and collects the first :max-trajectories final states into a density matrix
(domain/state.clj:726-791). Here the shots are trajectories of one compiled program on
the GPU (`qg_noisy_run`); this module translates the reference's noise-model maps into
the C structures, and shapes the results as the reference does.

Noise models use the reference's map shape with string keys:

    {"gate-noise": {"h": {"noise-type": "depolarizing", "noise-strength": 0.001},
                    "cnot": {"noise-type": "amplitude-damping", "t1-time": 100.0,
                             "gate-time": 300.0}},
     "readout-error": {"prob-0-to-1": 0.01, "prob-1-to-0": 0.02,
                       "correlated-errors": {0: {1: 2.0}}}}
"""
from __future__ import annotations

import ctypes as C
import itertools
import threading
import time
from collections import Counter
from typing import Any

import numpy as np

from . import _abi as A
from .circuit import circuit_metadata, encode, encode_operation

DEFAULT_STRENGTH = 0.01  # noise.clj:71
DEFAULT_COHERENT = {"rotation-angle": 0.01, "rotation-axis": "z"}  # noise.clj:93
AXES = {"x": 0, "y": 1, "z": 2}
MAX_DENSITY_QUBITS = 10


def _name(k) -> str:
    s = str(k)
    return s[1:] if s.startswith(":") else s


class NoiseSpec:
    """The C view (qg_noise_model) of a noise model for one circuit: one entry per
    gate-noise key, the entry and the noise target of every operation, the readout
    probabilities and the flattened correlation map. Keeps its arrays alive."""

    def __init__(self, circuit: dict, noise_model: dict | None):
        nm = noise_model or {}
        gate_noise = {_name(k): v for k, v in (nm.get("gate-noise") or {}).items()}
        names = list(gate_noise)
        self.entries = (A.QgGateNoise * max(1, len(names)))()
        for i, name in enumerate(names):
            cfg = gate_noise[name] or {}
            e = self.entries[i]
            e.noise_type = A.NOISE_TYPES.get(_name(cfg.get("noise-type")), A.QG_NOISE_NONE)
            e.strength = float(cfg.get("noise-strength", DEFAULT_STRENGTH))
            present = 0
            for key, bit, field in (("t1-time", A.QG_NOISE_HAS_T1, "t1_us"), ("t2-time", A.QG_NOISE_HAS_T2, "t2_us"),
                                    ("gate-time", A.QG_NOISE_HAS_GATE_TIME, "gate_time_ns")):
                if cfg.get(key) is not None:
                    present |= bit
                    setattr(e, field, float(cfg[key]))
            e.present = present
            ce = cfg.get("coherent-error") or DEFAULT_COHERENT
            e.coherent_angle = float(ce.get("rotation-angle", 0.0))
            e.coherent_axis = AXES.get(_name(ce.get("rotation-axis")), 3)
        index = {name: i for i, name in enumerate(names)}
        ops = circuit.get("operations") or []
        op_entry, op_target = [], []
        for op in ops:
            k = len(encode_operation(op)) if names else 1
            e = index.get(_name(op.get("operation-type")), -1)
            tgt = int((op.get("operation-params") or {}).get("target", 0) or 0)
            # noise follows the last encoded op of the operation (the whole operation first)
            op_entry += [-1] * (k - 1) + [e]
            op_target += [0] * (k - 1) + [tgt]
        self.op_entry = (C.c_int32 * max(1, len(op_entry)))(*op_entry)
        self.op_target = (C.c_int32 * max(1, len(op_target)))(*op_target)
        self.sites = sum(1 for e in op_entry if e >= 0)
        ro = nm.get("readout-error")
        corr = []
        if ro:
            for src, row in (ro.get("correlated-errors") or {}).items():
                # a row that is not a map (a bare factor) adjusts nothing: `get` on a
                # number gives nil in noise.clj:134-141
                for dst, f in (row.items() if isinstance(row, dict) else ()):
                    corr.append((int(src), int(dst), float(f)))
        self.corr_source = (C.c_int32 * max(1, len(corr)))(*[c[0] for c in corr])
        self.corr_target = (C.c_int32 * max(1, len(corr)))(*[c[1] for c in corr])
        self.corr_factor = (C.c_double * max(1, len(corr)))(*[c[2] for c in corr])
        m = A.QgNoiseModel()
        m.num_entries = len(names)
        m.entries = self.entries
        m.op_entry = self.op_entry
        m.op_target = self.op_target
        m.has_readout = 1 if ro else 0
        m.prob_0_to_1 = float(ro.get("prob-0-to-1", 0.0)) if ro else 0.0
        m.prob_1_to_0 = float(ro.get("prob-1-to-0", 0.0)) if ro else 0.0
        m.num_correlations = len(corr)
        m.corr_source = self.corr_source
        m.corr_target = self.corr_target
        m.corr_factor = self.corr_factor
        self.model = m


class NoisyRun(dict):
    """outcomes (uint64 basis indices after readout noise), trajectories (complex128,
    one row per collected shot), final-state (the last shot's), stats."""


def run_trajectories(ctx, circuit: dict, noise_model: dict | None, shots: int, seed: int = 0,
                     precision: str = "c128", max_trajectories: int = 100) -> NoisyRun:
    """Run `shots` noisy shots of `circuit` on the context's GPU (qg_noisy_run)."""
    lib = ctx.lib
    n = circuit["num-qubits"]
    enc = encode(circuit)
    spec = NoiseSpec(circuit, noise_model)
    if spec.model.num_entries and len(spec.op_entry) < enc.count:
        raise A.QgError(A.QG_ERR_INVALID_ARG, "noise map does not cover the encoded operations")
    N = 1 << n
    k = min(int(shots), int(max_trajectories))
    out = np.zeros(max(1, shots), np.uint64)
    traj = np.zeros((max(1, k), N), np.complex128)
    final = np.zeros(N, np.complex128)
    stats = A.QgNoisyStats()
    rc = lib.qg_noisy_run(ctx.ctx, enc.ref(), C.byref(spec.model), C.c_uint64(shots), C.c_uint64(seed),
                          A.QG_C64 if precision == "c64" else A.QG_C128, int(max_trajectories),
                          out.ctypes.data_as(A.U64P), traj.ctypes.data_as(A.DP) if k > 0 else None,
                          final.ctypes.data_as(A.DP) if shots > 0 else None, C.byref(stats))
    if rc != A.QG_OK:
        buf = C.create_string_buffer(1024)
        lib.qg_last_error(ctx.ctx, C.c_uint64(0), buf, C.c_int64(len(buf)))
        raise A.QgError(rc, buf.value.decode(errors="replace"))
    return NoisyRun(outcomes=out[:shots], trajectories=traj[:k], final_state=final,
                    stats={"device-ms": stats.device_ms, "total-ms": stats.total_ms, "batches": stats.batches,
                           "batch-size": stats.batch_size, "noise-sites": stats.noise_sites,
                           "passes": stats.passes, "distinct-states": stats.distinct_states})


def basis_string(index: int, n: int) -> str:
    """state.clj basis-string: qubit 0 first."""
    return format(int(index), f"0{n}b") if n else ""


def trajectory_to_density_matrix(trajectories: np.ndarray) -> dict:
    """state.clj:726-791 with equal weights."""
    k = trajectories.shape[0]
    w = np.full(k, 1.0 / k)
    rho = (trajectories.T * w) @ trajectories.conj()
    return {"density-matrix": rho, "trace": float(np.trace(rho).real), "weights": list(w)}


def _pauli_expectation(states: np.ndarray, pauli: str) -> np.ndarray:
    n = len(pauli)
    idx = np.arange(states.shape[1], dtype=np.int64)
    xm = zm = ny = 0
    for q, ch in enumerate(pauli):
        b = 1 << (n - 1 - q)
        if ch in "XY":
            xm |= b
        if ch in "YZ":
            zm |= b
        ny += ch == "Y"
    sign = 1 - 2 * (np.array([bin(z).count("1") & 1 for z in (idx & zm)]))
    ph = (-1j) ** ny
    return np.real(np.sum(states.conj() * (ph * sign * states[:, idx ^ xm]), axis=1))


def _extract(run: NoisyRun, base: dict, specs: dict, circuit: dict, shots: int) -> dict:
    """extract-noisy-results (result.clj:641-790) for the result types computed here."""
    n = circuit["num-qubits"]
    out: dict[str, Any] = {"result-types": set(specs)}
    rho = base.get("density-matrix")
    traj = run["trajectories"]
    for kind, spec in specs.items():
        if kind == "measurements":
            freq = base["measurement-results"]
            total = sum(freq.values())
            emp = {o: c / total for o, c in freq.items()} if total else {}
            out["measurement-results"] = {
                "measurement-outcomes": list(freq), "measurement-probabilities": emp, "empirical-probabilities": emp,
                "shot-count": total, "measurement-qubits": list((spec or {}).get("measurement-qubits") or range(n)),
                "frequencies": freq, "source": "noisy-simulation"}
        elif kind == "hamiltonian":
            terms = spec.get("hamiltonian", spec) if isinstance(spec, dict) else spec
            e = 0.0
            for t in terms:
                e += t["coefficient"] * float(np.mean(_pauli_expectation(traj, t["pauli-string"])))
            out["hamiltonian-result"] = {"energy-expectation": e, "hamiltonian": terms, "source": "density-matrix"}
        elif kind == "probability":
            p = np.mean(np.abs(traj) ** 2, axis=0)
            res = {"probability-outcomes": p}
            ts = (spec or {}).get("target-states")
            if ts:
                res["target-probabilities"] = {s: float(p[int(s, 2) if isinstance(s, str) else int(s)]) for s in ts}
            out["probability-results"] = res
        elif kind == "density-matrix" and spec is True and rho is not None:
            out["density-matrix-result"] = {"density-matrix": rho, "num-qubits": n,
                                            "trace": base["density-matrix-trace"], "from-trajectories": True,
                                            "trajectory-count": base["trajectory-count"]}
        elif kind == "state-vector" and spec is True:
            p = np.mean(np.abs(traj) ** 2, axis=0)
            out["state-vector-result"] = {"num-qubits": n, "state-vector": np.sqrt(p).astype(np.complex128),
                                          "basis-labels": [basis_string(i, n) for i in range(1 << n)]}
        # other result types: not computed for noisy runs (the reference prints a warning)
    return out


def execute_circuit(circuit: dict, device: dict | None = None, options: dict | None = None, ctx=None,
                    seed: int | None = None) -> dict:
    """hardware_simulator.clj:196-241 and execute-circuit-simulation-with-trajectories
    (:102-193): `shots` noisy shots (default 1024), measurement frequencies keyed by
    bitstring, the last shot's final state, the first :max-trajectories (default 100)
    final states and their density matrix (up to 10 qubits here)."""
    from .state import Context

    options = options or {}
    noise_model = (device or {}).get("noise-model") or {}
    shots = int(options.get("shots", 1024))
    max_traj = int(options.get("max-trajectories", 100))
    specs = options.get("result-specs")
    t0 = time.perf_counter()
    own = ctx is None
    ctx = ctx or Context(precision=options.get("precision", "c128"))
    try:
        run = run_trajectories(ctx, circuit, noise_model, shots,
                               seed if seed is not None else int(options.get("seed", time.time_ns() & 0xFFFFFFFF)),
                               options.get("precision", "c128"), max_traj)
    except A.QgError as e:
        return {"job-status": "failed", "error-message": str(e), "exception-type": "QgError"}
    finally:
        if own:
            ctx.close()
    n = circuit["num-qubits"]
    freq = Counter(basis_string(o, n) for o in run["outcomes"])
    base: dict[str, Any] = {"measurement-results": dict(freq),
                            "final-state": {"num-qubits": n, "state-vector": run["final_state"]}}
    traj = run["trajectories"]
    if len(traj):
        base["trajectories"] = [{"num-qubits": n, "state-vector": v} for v in traj]
        base["trajectory-count"] = len(traj)
        if n <= MAX_DENSITY_QUBITS:
            dm = trajectory_to_density_matrix(traj)
            base["density-matrix"] = dm["density-matrix"]
            base["density-matrix-trace"] = dm["trace"]
            base["trajectory-weights"] = dm["weights"]
    results = dict(base)
    if specs:
        results.update(_extract(run, base, specs, circuit, shots))
    return {"job-status": "completed", "circuit": circuit, "circuit-metadata": circuit_metadata(circuit),
            "shots-executed": shots, "execution-time-ms": (time.perf_counter() - t0) * 1e3,
            "results": results, "device-stats": run["stats"]}


class HardwareSimulator:
    """The QuantumBackend protocol of hardware_simulator.clj:262-395: asynchronous jobs on
    a worker thread, job status and results, cancellation of queued jobs, devices."""

    _ids = itertools.count(1)

    def __init__(self, config: dict | None = None, device: dict | None = None, devices: list | None = None):
        from .state import Context

        self.config = config or {"max-qubits": 16}
        self._devices = list(devices or [])
        from .circuit import NATIVE_SIMULATOR_GATE_SET

        noiseless = {"id": "noiseless", "name": "Noiseless device", "noise-model": {},
                     "native-gates": set(NATIVE_SIMULATOR_GATE_SET)}
        if device is not None:
            # create-hardware-simulator normalises a device it is given
            # (hardware_simulator.clj:409-414, device.clj:57-68)
            from .device import validate_device

            device = validate_device(device)
            self._devices.append(device)
        self._current = device or (self._devices[0] if self._devices else noiseless)
        self._ctx = Context(precision=self.config.get("precision", "c128"))
        self._jobs: dict[str, dict] = {}
        self._lock = threading.Lock()
        self._cv = threading.Condition(self._lock)
        self._queue: list[str] = []
        self._worker = threading.Thread(target=self._loop, daemon=True)
        self._stop = False
        self._worker.start()

    def close(self):
        with self._cv:
            self._stop = True
            self._cv.notify_all()
        self._worker.join()
        self._ctx.close()

    def backend_info(self) -> dict:
        return {"backend-type": "hardware-simulator", "backend-name": "Hardware Simulator",
                "devices": self._devices, "device": self._current, "config": self.config,
                "capabilities": {"multi-device"}}

    def device(self) -> dict:
        return self._current

    def available(self) -> bool:
        return True

    def devices(self) -> list:
        return list(self._devices)

    def select_device(self, device) -> dict:
        if isinstance(device, str):
            device = next((d for d in self._devices if d.get("id") == device), None)
        self._current = device
        return self._current

    def submit_circuit(self, circuit: dict, options: dict | None = None) -> str:
        job_id = f"job_{next(self._ids)}_{int(time.time() * 1000)}"
        job = {"id": job_id, "circuit": circuit, "options": dict(options or {}), "device": self._current,
               "status": "queued", "result": None, "created-at": time.time() * 1000, "completed-at": None}
        # submit-circuit runs the hardware optimisation pipeline and executes the original
        # circuit: the pipeline only decides whether the job fails (hardware_simulator.clj:300-330)
        from .optimization import OptimizationError, optimize

        opts = dict(options or {})
        try:
            # the defaults, then every submitted option over them (`merge`)
            optimize(circuit, self._current, {
                "optimize-gates?": opts.get("optimize-gates?", True),
                "optimize-qubits?": opts.get("optimize-qubits?", True),
                "optimize-topology?": opts.get("optimize-topology?", False),
                "transform-operations?": opts.get("transform-operations?", True),
                "max-iterations": opts.get("max-iterations", 100), **opts})
        except OptimizationError as e:
            job.update({"status": "failed", "completed-at": time.time() * 1000,
                        "result": {"job-status": "failed", "error-message": str(e)}})
            with self._lock:
                self._jobs[job_id] = job
            return job_id
        with self._cv:
            self._jobs[job_id] = job
            self._queue.append(job_id)
            self._cv.notify_all()
        return job_id

    def _loop(self):
        while True:
            with self._cv:
                while not self._queue and not self._stop:
                    self._cv.wait()
                if self._stop:
                    return
                jid = self._queue.pop(0)
                job = self._jobs[jid]
                if job["status"] != "queued":
                    continue
                job["status"] = "running"
            try:
                res = execute_circuit(job["circuit"], job["device"], job["options"], ctx=self._ctx)
            except Exception as e:  # a job that raises fails; the worker keeps serving
                res = {"job-status": "failed", "error-message": f"{type(e).__name__}: {e}"}
            with self._cv:
                job["result"] = res
                job["status"] = res["job-status"]
                job["completed-at"] = time.time() * 1000
                self._cv.notify_all()

    def wait(self, job_id: str, timeout_s: float = 60.0) -> str:
        end = time.time() + timeout_s
        with self._cv:
            while job_id in self._jobs and self._jobs[job_id]["status"] in ("queued", "running"):
                left = end - time.time()
                if left <= 0:
                    break
                self._cv.wait(left)
            return self.job_status(job_id)

    def job_status(self, job_id: str) -> str:
        job = self._jobs.get(job_id)
        return job["status"] if job else "not-found"

    def job_result(self, job_id: str) -> dict:
        job = self._jobs.get(job_id)
        if job is None:
            return {"job-id": job_id, "job-status": "not-found", "error-message": "Job not found"}
        if job["status"] == "completed":
            return dict(job["result"], **{"job-id": job_id})
        if job["status"] == "failed":
            return job["result"]
        return {"job-id": job_id, "job-status": job["status"], "error-message": "Job not completed"}

    def cancel_job(self, job_id: str) -> str:
        with self._cv:
            job = self._jobs.get(job_id)
            if job is None:
                return "not-found"
            if job["status"] == "queued":
                job["status"] = "cancelled"
                job["completed-at"] = time.time() * 1000
                return "cancelled"
            return "already-completed"

    def queue_status(self) -> dict:
        with self._lock:
            st = [j["status"] for j in self._jobs.values()]
        return {"total-jobs": len(st), "active-jobs": sum(s in ("queued", "running") for s in st),
                "completed-jobs": sum(s == "completed" for s in st)}


def create_hardware_simulator(config: dict | None = None, device: dict | None = None,
                              devices: list | None = None) -> HardwareSimulator:
    """hardware_simulator.clj:400-418. `devices` is the catalogue the simulator starts with
    (the reference loads its own, simulator-devices.edn, and starts on its first entry:
    hardware_simulator.clj:39-55); `load_devices` reads that file."""
    return HardwareSimulator(config, device, devices)


def load_devices(path: str) -> list[dict]:
    """The device maps of an EDN device catalogue such as the reference's
    resources/simulator-devices.edn, with keyword keys and values as plain strings (the
    spelling this package uses: "native-gates", "gate-noise", "all-to-all") and sets as
    frozensets."""
    from .edn import EdnError, load

    data = load(path)
    if not isinstance(data, list) or not all(isinstance(d, dict) for d in data):
        raise EdnError("a device catalogue is a vector of device maps")
    return data
