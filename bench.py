#!/usr/bin/env python
"""Benchmark: a 30-qubit layered circuit (40 layers of one random gate from
{H,X,Y,Z,S,T,RX,RY,RZ} per qubit plus CNOTs on a random matching) followed by a
30-qubit QFT, on one GB300, through libqgpu.so.

One step = zero-state + the whole circuit (2280 gates) on a device-resident
2^30-amplitude state. value = gate-amplitudes/s = sum_gates 2^n / step time,
summed over ranks (replicas: every rank simulates its own state, no collective).
The state (16 GiB c128 / 8 GiB c64) is larger than L2, so no flush is needed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's algorithm (the dense Kronecker mat-vec
of QClojure's simulator, restated in C in oracle/) on the host cores for the
same workload: a bounded sample of output amplitudes of one gate per step.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "30-qubit layer time & HBM GB/s; serve circuits/s + p50/p99, c64 vs c128"
UNIT = "gate-amplitudes/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--qubits", type=int, default=30)
    ap.add_argument("--depth", type=int, default=40)
    ap.add_argument("--precision", choices=["c128", "c64"], default="c128")
    ap.add_argument("--fusion", choices=["plain", "tiled", "dense"], default="tiled")
    ap.add_argument("--no-extras", action="store_true", help="skip the c64 / e2e / cpu-baseline legs")
    ap.add_argument("--pass-kernels", choices=["auto", "always", "off"], default="auto",
                    help="specialised per-pass kernels (auto: states of 29 qubits and more)")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default pass-kernel shape instead of timing the candidates first")
    ap.add_argument("--shape", default=None,
                    help="pass-kernel shape tile_bits,reg_bits,buffers,ctas_per_sm for the main precision "
                         "(set directly, no autotuning; for profiling a chosen shape)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), float(f[3]), f[5], f[6], f[7], f[8]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        reasons = set()
        for r in rows:
            for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), r[3:]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows), "samples": len(rows), "reasons": sorted(reasons)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
def cpu_reference_rate(n: int, gates_per_step: int, budget_s: float, threads: int | None = None):
    """Reference algorithm on the host: rows of the dense Kronecker mat-vec of one
    1-qubit gate (gate.clj:346-395), each row visiting all 2^n columns. Returns
    (gate-amplitudes/s, description, threads)."""
    import numpy as np

    from oracle import oracle as O

    O.lib()
    threads = threads or os.cpu_count() or 1
    avail_gb = 0.0
    try:
        for line in Path("/proc/meminfo").read_text().splitlines():
            if line.startswith("MemAvailable"):
                avail_gb = int(line.split()[1]) / 2**20
    except OSError:
        pass
    m = n
    while m > 20 and (16 << m) / 2**30 > 0.4 * avail_gb:
        m -= 2
    rng = np.random.default_rng(0)
    x = (rng.standard_normal(1 << m) + 1j * rng.standard_normal(1 << m)) / math.sqrt(2 << m)
    h = [[1 / math.sqrt(2), 1 / math.sqrt(2)], [1 / math.sqrt(2), -1 / math.sqrt(2)]]
    t0 = time.perf_counter()
    O.refalgo_rows(x, h, m // 2, 0, 1)
    one = time.perf_counter() - t0
    rows_per_thread = max(1, int(budget_s / max(one, 1e-6)))
    results = [0] * threads

    def work(k):
        O.refalgo_rows(x, h, m // 2, k * rows_per_thread, rows_per_thread)
        results[k] = rows_per_thread

    ths = [threading.Thread(target=work, args=(k,)) for k in range(threads)]
    t0 = time.perf_counter()
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    dt = time.perf_counter() - t0
    rows = sum(results)
    rate = rows / dt * (2.0 ** (m - n))  # per-row work is 2^m MACs; scale to 2^n columns
    desc = (f"{rows} output amplitudes of one H gate's dense 2^{m}x2^{m} Kronecker mat-vec"
            + (f", scaled by 2^{m - n} to {n} qubits (host memory)" if m != n else "")
            + f", {threads} threads, {dt:.1f} s")
    return rate, desc, threads


# ---------------------------------------------------------------------------
def replay_trace(sim, trace, timeout_s=900.0):
    """Submit each job of `trace` at its arrival time through the job API and wait for all.
    Latency of a job = its submission delay + queue + execution time on the runtime's clock.
    Returns (circuits/s over first arrival .. last completion, latencies in ms, jobs that
    shared a small-job launch, largest such launch)."""
    import ctypes as C

    from qclojure_gb300 import _abi as A

    ids = [None] * len(trace)
    lag = [0.0] * len(trace)
    t0 = time.perf_counter()

    def submitter():
        for k, job in enumerate(trace):
            wait = t0 + job["arrival-s"] - time.perf_counter()
            if wait > 0:
                time.sleep(wait)
            ids[k] = sim.submit_circuit(job["circuit"], {"result-specs": job["result-specs"]})
            lag[k] = time.perf_counter() - (t0 + job["arrival-s"])

    th = threading.Thread(target=submitter)
    th.start()
    th.join()
    lat, batched, max_batch = [], 0, 0
    for k, jid in enumerate(ids):
        s = sim.wait(jid, int(timeout_s * 1e3))
        if s != "completed":
            raise RuntimeError(f"serving job {k} ended {s}")
    t_end = time.perf_counter()
    for k, jid in enumerate(ids):
        info = A.QgJobInfo()
        sim._lib.qg_job_details(sim._ctx, C.c_uint64(sim._jid(jid)), C.byref(info))
        lat.append(lag[k] * 1e3 + info.queue_time_ms + info.execution_time_ms)
        if info.batched_with > 1:
            batched += 1
        max_batch = max(max_batch, info.batched_with)
        sim.free_job(jid)
    return len(trace) / (t_end - t0), lat, batched, max_batch


def serving_leg(num_jobs=250, rates=(5, 20, 100, 5000), seed=11, plain_jobs=100):
    """Serving stream: Poisson arrivals, n = 8 + Geometric(0.15) capped at 28, depth U{10..200}
    of the layered recipe, 90% shot jobs (1k..100k shots) and 10% Pauli-string expectations.
    complex64 served (continuous batching, concurrent worker streams, large jobs specialised
    from the measured crossover on) against plain complex128 per job (one HBM pass per gate,
    one job at a time) on the first `plain_jobs` jobs of the same trace."""
    from qclojure_gb300 import workloads
    from qclojure_gb300.backend import create_simulator

    def pct(v, q):
        s = sorted(v)
        return s[min(len(s) - 1, int(round(q * (len(s) - 1))))]

    out = {"workload": f"{num_jobs} jobs: n = 8 + Geometric(0.15) capped at 28, depth U{{10..200}} layered, "
                       "90% shots U{1k..100k}, 10% Pauli expectation", "c64_served": {}}
    sim = create_simulator({"precision": "c64", "fusion": "tiled", "workers": 16, "seed": 5})
    try:
        # from which size a one-off job of the stream's mean depth gains from compiling its kernels
        try:
            out["specialise_from"] = sim.autotune_crossover("c64", 100)
        except Exception as e:  # the leg still runs with the default crossover
            out["specialise_from"] = {"error": f"{type(e).__name__}: {e}"}
        replay_trace(sim, workloads.serving_trace(24, 1000.0, seed + 99, max_qubits=14))  # warm-up
        for r in rates:
            trace = workloads.serving_trace(num_jobs, float(r), seed)
            cps, lat, nb, mb = replay_trace(sim, trace)
            out["c64_served"][str(r)] = {"circuits_per_s": cps, "p50_ms": pct(lat, 0.5), "p99_ms": pct(lat, 0.99),
                                         "jobs_batched": nb, "largest_batch": mb}
        out["precompiled_jobs"] = sim.queue_status()["precompiled-jobs"]
    finally:
        sim.close()
    trace = workloads.serving_trace(num_jobs, float(rates[-1]), seed)[:plain_jobs]
    plain = create_simulator({"precision": "c128", "fusion": "plain", "workers": 1, "seed": 5,
                              "arithmetic": "exact"})
    try:
        lat = []
        t0 = time.perf_counter()
        for job in trace:
            t1 = time.perf_counter()
            jid = plain.submit_circuit(job["circuit"], {"result-specs": job["result-specs"]})
            if plain.wait(jid, 900_000) != "completed":
                raise RuntimeError("plain job failed")
            lat.append((time.perf_counter() - t1) * 1e3)
            plain.free_job(jid)
        dt = time.perf_counter() - t0
    finally:
        plain.close()
    out["plain_c128_per_job"] = {"circuits_per_s": len(trace) / dt, "p50_ms": pct(lat, 0.5), "p99_ms": pct(lat, 0.99),
                                 "jobs": len(trace),
                                 "note": "the trace's first jobs, one at a time, one HBM pass per gate"}
    top = out["c64_served"][str(rates[-1])]["circuits_per_s"]
    out["served_over_plain"] = top / out["plain_c128_per_job"]["circuits_per_s"]
    return out


# ---------------------------------------------------------------------------
def cpu_statevector_rates(args, rank: int) -> dict:
    """Beside the reference's algorithm, the best CPU figure: an optimised CPU state
    vector (oracle/cpu_sv.c: one in-place pass per gate, OpenMP on all host cores,
    complex128), NOT the reference. Bounded samples of the workload: its first 300 gates
    at 24 qubits and its first 12 gates at 30 qubits, after one gate that touches the
    state's pages."""
    try:
        import numpy as np

        from oracle import oracle as ORC
        from qclojure_gb300 import workloads

        lib = ORC.cpu_sv_lib()
        if lib is None:
            return {"unavailable": "the CPU state-vector library could not be built"}
        out = {"label": "not the reference: optimised CPU state vector, all host cores", "threads": int(lib.sv_threads())}
        for sn, sg in ((24, 300), (30, 12)):
            ops = workloads.large_circuit(sn, args.depth, args.seed + rank)["operations"][:sg + 1]
            sv = np.zeros(1 << sn, np.complex128)
            sv[0] = 1
            ORC.cpu_sv_run({"num-qubits": sn, "operations": ops[:1]}, sv)
            t0 = time.perf_counter()
            ORC.cpu_sv_run({"num-qubits": sn, "operations": ops[1:]}, sv)
            dt = time.perf_counter() - t0
            out[f"n{sn}"] = {"gates": sg, "s": dt, "gate_amps_per_s": sg * 2 ** sn / dt}
            del sv
        return out
    except Exception as e:  # the line must still print
        return {"error": f"{type(e).__name__}: {e}"}


# ---------------------------------------------------------------------------
CONFIG0 = {"qubits": 10, "depth": 20, "shots": 1024, "seed": 0}


def reference_config0(measure_up_to: int = 12, extrapolate_to: int = 16) -> dict:
    """The reference's algorithm on the plain CPU case, single-threaded as the reference runs
    a job (one future per job, ideal_simulator.clj:129): the config-0 circuit (10 qubits,
    depth 20, 300 gates) and 1024 shots, run whole by oracle.refalgo_circuit (a dense
    Kronecker mat-vec per single-qubit gate, a full probability scan per shot). The same
    recipe at 8..measure_up_to qubits is measured whole; beyond that the time is
    extrapolated from the largest measured size by the single-qubit gates' 4^n work and
    labelled so. A lower bound on the reference's JVM time, which cannot run on this machine."""
    from oracle import oracle as O
    from qclojure_gb300 import workloads

    d, shots = CONFIG0["depth"], CONFIG0["shots"]
    out = {"label": "reference algorithm restated in C (oracle/qgo.c or_refalgo_circuit), 1 thread; "
                    "a lower bound on the reference's JVM time", "threads": 1,
           "recipe": f"layered depth {d} + {shots} shots, seed {CONFIG0['seed']}", "by_qubits": {}}
    last = None
    for n in range(8, measure_up_to + 1):
        c = workloads.layered_circuit(n, d, CONFIG0["seed"])
        t0 = time.perf_counter()
        O.refalgo_circuit(c, shots, 1)
        dt = time.perf_counter() - t0
        g1 = sum(1 for op in c["operations"] if op["operation-type"] != "cnot")
        out["by_qubits"][str(n)] = {"gates": len(c["operations"]), "s": dt, "measured": True}
        last = (n, dt, g1)
    n0, t0s, g10 = last
    for n in range(measure_up_to + 1, extrapolate_to + 1):
        g1 = n * d
        est = t0s * (g1 / g10) * 4.0 ** (n - n0)
        out["by_qubits"][str(n)] = {"gates": g1 + (n // 2) * d, "s": est, "measured": False,
                                    "extrapolated_from": n0}
    out["config0_s"] = out["by_qubits"][str(CONFIG0["qubits"])]["s"]
    out["config0_circuits_per_s"] = 1.0 / out["config0_s"]
    return out


def gpu_config0(device: int, runs: int = 50) -> dict:
    """The config-0 job end to end through the job API on the GPU (complex128, final
    state + probabilities + 1024 shots into host buffers), mean over `runs` jobs."""
    from qclojure_gb300 import workloads
    from qclojure_gb300.backend import GpuStateVectorSimulator, execute_circuit

    c = workloads.layered_circuit(CONFIG0["qubits"], CONFIG0["depth"], CONFIG0["seed"])
    opts = {"result-specs": {"measurements": {"shots": CONFIG0["shots"]}, "probabilities": {}}, "seed": 1}
    out = {}
    for arith in ("double-float", "exact"):
        sim = GpuStateVectorSimulator({"precision": "c128", "fusion": "tiled", "workers": 1, "seed": 1,
                                       "arithmetic": arith}, device=device)
        try:
            for _ in range(3):
                r = execute_circuit(sim, c, opts, timeout_ms=60_000)
                sim.free_job(r["job-id"])
            t0 = time.perf_counter()
            for _ in range(runs):
                r = execute_circuit(sim, c, opts, timeout_ms=60_000)
                assert r["job-status"] == "completed", r
                sim.free_job(r["job-id"])
            dt = (time.perf_counter() - t0) / runs
        finally:
            sim.close()
        out[arith.replace("-", "_")] = {"ms_per_job": dt * 1e3, "circuits_per_s": 1.0 / dt}
    out["path"] = "qg_submit -> qg_wait -> final state, probabilities, 1024 shots (host buffers)"
    return out


def oracle_spot_check_30(ctx, n: int, depth: int, seed: int, device: int) -> dict:
    """The large-n oracle check: the 30-qubit recipe at reduced depth (`depth` layers + the
    full QFT) run by the CPU state vector (oracle/cpu_sv.c, bit-identical to the oracle,
    all host cores), uploaded as a complex128 reference, against the device's double-float
    result (the benchmarked path) and its exact FP64 result."""
    import numpy as np

    from oracle import oracle as ORC
    from qclojure_gb300 import workloads

    if ORC.cpu_sv_lib() is None:
        return {"unavailable": "the CPU state-vector library could not be built"}
    c = workloads.layered_circuit(n, depth, seed)
    c = {"num-qubits": n, "operations": c["operations"] + workloads.qft_ops(n)}
    sv = np.zeros(1 << n, np.complex128)
    sv[0] = 1
    t0 = time.perf_counter()
    ORC.cpu_sv_run(c, sv)
    cpu_s = time.perf_counter() - t0
    out = {"workload": f"layered-{n}x{depth}+qft{n} ({len(c['operations'])} gates)",
           "oracle": "oracle/cpu_sv.c on the host (bit-identical to oracle/qgo.c)", "cpu_s": cpu_s}
    from qclojure_gb300.state import Context

    with ctx.state(n, "c128") as ref:
        ref.upload(sv)
        del sv
        with ctx.state(n, "c128") as s:
            s.set_basis(0)
            s.apply(c)
            out["c128_double_float"] = s.compare(ref)
        with Context(device=device, workers=1, seed=7, arithmetic="exact") as cx:
            with cx.state(n, "c128") as s:
                s.set_basis(0)
                s.apply(c)
                out["c128_exact"] = s.compare(ref)
    return out


# ---------------------------------------------------------------------------
def _short(x, digits: int = 4):
    """Floats to `digits` significant digits, recursively (the summary keys at the line's end)."""
    if isinstance(x, float):
        return float(f"{x:.{digits}g}") if math.isfinite(x) else x
    if isinstance(x, dict):
        return {k: _short(v, digits) for k, v in x.items()}
    if isinstance(x, list):
        return [_short(v, digits) for v in x]
    return x


def order_line(line: dict) -> dict:
    """The JSON line's key order: the contract's keys, then the long legs, then the
    headline's evidence (roofline, CPU baselines, end to end, complex64, exact FP64,
    accuracy) so that the end of the line carries it."""
    head = ["metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
            "vs_baseline", "dtype", "data", "gpu_launches", "config", "clocks"]
    tail = ["cpu_baseline", "e2e", "layer_ms", "hbm_passes_per_step", "roofline", "c64", "exact_fp64",
            "oracle_30q", "accuracy"]
    out = {k: line[k] for k in head if k in line}
    out.update({k: v for k, v in line.items() if k not in out and k not in tail})
    for k in tail:
        if k in line:
            out[k] = _short(line[k]) if k in ("c64", "exact_fp64", "oracle_30q", "accuracy") else line[k]
    return out


def max_over_ranks(ms: float, dist=None, device: str = "cpu") -> float:
    """The slowest rank's time: every rank runs its own replica (no data exchange), and
    the job is done when the last one is."""
    if dist is None:
        return ms
    import torch

    t = torch.tensor([ms], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def whole_job_rate(world: int, units_per_rank: float, ms_per_step: float) -> float:
    """Units processed by all replicas per second (weak scaling: fixed work per rank)."""
    return world * units_per_rank / (ms_per_step / 1e3)


# ---------------------------------------------------------------------------
def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from qclojure_gb300 import workloads

    gates = len(workloads.large_circuit(args.qubits, args.depth, args.seed)["operations"])
    vals = []
    desc = ""
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_reference_rate(args.qubits, gates, 0.5)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        v, desc, threads = cpu_reference_rate(args.qubits, gates, 2.5)
        vals.append(v)
    dt = time.perf_counter() - t0
    value = statistics.mean(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"layered-{args.qubits}x{args.depth}+qft{args.qubits}", "n_qubits": args.qubits,
                   "gates": gates, "precision": "c128"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc,
                         "extrapolated": "a sample of one gate's rows scaled to the whole circuit: the "
                                         "dense algorithm cannot run a 30-qubit gate (2^60 entries)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference (Clojure/JVM) cannot run here; this times its algorithm restated in C",
    }
    try:
        line["cpu_baseline"]["config0"] = reference_config0()
    except Exception as e:  # the line must still print
        line["cpu_baseline"]["config0"] = {"error": f"{type(e).__name__}: {e}"}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import __graft_entry__ as g

    g.build()
    import ctypes as C

    import numpy as np

    from qclojure_gb300 import _abi as A
    from qclojure_gb300 import workloads
    from qclojure_gb300.circuit import encode
    from qclojure_gb300.state import Context

    n = args.qubits
    circ = workloads.large_circuit(n, args.depth, args.seed + rank)
    layers_only = workloads.layered_circuit(n, args.depth, args.seed + rank)
    gates = len(circ["operations"])
    N = 1 << n
    lib = A.load_library()
    ctx = Context(device=local, workers=1, seed=7, pass_kernels=args.pass_kernels)
    # the pass kernels' tile size and launch shape, chosen on the device before timing
    tuning = {}
    if args.shape:
        kb, rb, bf, ct = (int(x) for x in args.shape.split(","))
        ctx.set_tuning(n, args.precision, kb, rb, bf, ct)
        tuning[args.precision] = {"chosen": ctx.tuning(n, args.precision), "set": "--shape"}
    elif not args.no_autotune and args.fusion == "tiled":
        for tp in ((args.precision, "c64") if args.precision == "c128" and not args.no_extras else (args.precision,)):
            try:
                tuning[tp] = ctx.autotune(n, tp, circ)  # timed on the workload itself
            except Exception as e:  # nothing to tune (exact arithmetic, interpreted sizes)
                tuning[tp] = {"skipped": f"{type(e).__name__}: {e}"}
    st = ctx.state(n, args.precision)
    dptr, sptr = st.device_ptr()
    stream = torch.cuda.ExternalStream(sptr, device=torch.device("cuda", local))

    def step():
        st.set_basis(0)
        st.apply(circ, fusion=args.fusion)

    # specialised pass kernels: generated and compiled once per program (cached), before timing
    compile_ms, n_spec = st.prepare(circ, fusion=args.fusion)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    l0 = C.c_uint64()
    lib.qg_kernel_launches(C.byref(l0))
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    e1.synchronize()
    l1 = C.c_uint64()
    lib.qg_kernel_launches(C.byref(l1))
    ck = clocks.stop()
    torch.cuda.synchronize()
    elapsed_ms = e0.elapsed_time(e1)
    elapsed_ms = max_over_ranks(elapsed_ms, dist, "cuda")
    ms_per_step = elapsed_ms / args.steps
    value = whole_job_rate(world, gates * N, ms_per_step)

    # per-pass timing (separate, untimed run) for the roofline of the dominant kernel
    enc = encode(circ)
    cap = 8192
    pms = (C.c_float * cap)()
    pkind = (C.c_int32 * cap)()
    npass = C.c_int32()
    st.set_basis(0)
    from qclojure_gb300.backend import FUSIONS

    rc = lib.qg_state_profile(st.h, enc.ref(), FUSIONS[args.fusion], 0, pms, pkind, cap, C.byref(npass))
    pass_ms = [pms[i] for i in range(npass.value)] if rc == 0 else []
    kinds = [pkind[i] for i in range(npass.value)] if rc == 0 else []
    B = 16 if args.precision == "c128" else 8
    pass_bytes = 2 * B * N
    dom_kind = (4 if 4 in kinds else 3 if 3 in kinds else 1) if args.fusion != "plain" else 0
    dom = [t for t, k in zip(pass_ms, kinds) if k == dom_kind]
    peak, peak_src = measured_peaks()
    mean_pass = statistics.mean(dom) if dom else float("nan")
    achieved = pass_bytes / (mean_pass / 1e3) / 1e9 if dom else float("nan")
    # DRAM bytes per tiled pass from an ncu capture of the same kernel on a 26-qubit state
    # (dram__bytes_read.sum + dram__bytes_write.sum = 2.087e9 per c128 launch, 1.012e9 per c64
    # launch), scaled by the amplitudes processed
    traffic, traffic_src = None, None
    if args.fusion == "tiled":
        traffic = (2.087e9 if args.precision == "c128" else 1.012e9) * 2 ** (n - 26)
        traffic_src = "ncu capture at 26 qubits x 2^(n-26)"
    # time of the 40 random layers alone, per layer
    st.prepare(layers_only, fusion=args.fusion)
    st.set_basis(0)
    tl0 = torch.cuda.Event(enable_timing=True)
    tl1 = torch.cuda.Event(enable_timing=True)
    tl0.record(stream)
    st.apply(layers_only, fusion=args.fusion)
    tl1.record(stream)
    tl1.synchronize()
    layer_ms = tl0.elapsed_time(tl1) / args.depth

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32x2 double-float (f64 storage)" if args.precision == "c128" else "f32", "data": "synthetic",
        "config": {"workload": f"layered-{n}x{args.depth}+qft{n}", "n_qubits": n, "depth": args.depth,
                   "gates": gates, "precision": args.precision, "fusion": args.fusion,
                   "parallelism": f"replicas{world}", "l2": "state larger than L2 (no flush needed)",
                   "pass_kernel_shape": {k: (v.get("chosen") or v) for k, v in tuning.items()} or "default"},
        "autotune": tuning,
        "layer_ms": layer_ms,
        "pass_kernels": {"specialised_passes": n_spec, "compile_ms": compile_ms,
                         "note": "NVRTC compile of the per-pass kernels, once per program, before timing"},
        "hbm_passes_per_step": len(pass_ms),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if dom else None, "traffic": traffic,
                     "traffic_source": traffic_src,
                     "kernel": "k_dense_tc (dense block on the tensor cores, complex64)" if dom_kind == 4 else
                     ("qgp_<pass> (specialised tiled pass, " + ("double-float)" if args.precision == "c128"
                                                                 else "complex64)"))
                     if dom_kind == 3 else ("k_tile2<PolDFT>" if args.precision == "c128" else "k_tile2<PolF>"),
                     "peak_source": peak_src, "pass_bytes": pass_bytes, "mean_pass_ms": mean_pass,
                     "passes": len(dom),
                     "note": ("passes are bound by FP32 instruction issue, not HBM: ncu on the same kernel "
                              "and shape (26 qubits) shows 59-68% issue active and 31-32% DRAM throughput "
                              "for double-float complex128")
                     if dom_kind == 3 and args.precision == "c128" else None},
        "gpu_launches": int(l1.value - l0.value),
        "clocks": ck,
    }

    if rank == 0 and not args.no_extras:
        # accuracy against an exact FP64 run of the same circuit: complex128 with every product
        # and sum rounded in the reference's gate order (the path that is bit-identical to the
        # oracle in the parity tests), compared on the device with the benchmarked result
        ctx_x = Context(device=local, workers=1, seed=7, arithmetic="exact")
        sx = ctx_x.state(n, "c128")
        _, sxs = sx.device_ptr()
        xstream = torch.cuda.ExternalStream(sxs, device=torch.device("cuda", local))
        sx.set_basis(0)
        xa = torch.cuda.Event(enable_timing=True)
        xb = torch.cuda.Event(enable_timing=True)
        xa.record(xstream)
        sx.apply(circ, fusion=args.fusion)
        xb.record(xstream)
        xb.synchronize()
        st.set_basis(0)
        st.apply(circ, fusion=args.fusion)
        accuracy = {"reference": "c128 exact FP64 arithmetic, gate order of the reference",
                    "reference_ms": xa.elapsed_time(xb),
                    ("c128_double_float" if args.precision == "c128" else "c64"): st.compare(sx)}
        # complex64 leg (same circuit)
        if args.precision == "c128":
            st64 = ctx.state(n, "c64")
            _, s64 = st64.device_ptr()
            stream64 = torch.cuda.ExternalStream(s64, device=torch.device("cuda", local))
            c64_compile_ms, _ = st64.prepare(circ, fusion=args.fusion)
            for _ in range(2):
                st64.set_basis(0)
                st64.apply(circ, fusion=args.fusion)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream64)
            for _ in range(args.steps):
                st64.set_basis(0)
                st64.apply(circ, fusion=args.fusion)
            b.record(stream64)
            b.synchronize()
            ms64 = a.elapsed_time(b) / args.steps
            st64.set_basis(0)
            p64, k64 = st64.profile(circ, fusion=args.fusion)
            d64 = [t for t, k in zip(p64, k64) if k in (1, 3)]
            m64 = statistics.mean(d64) if d64 else float("nan")
            a64 = 2 * 8 * N / (m64 / 1e3) / 1e9 if d64 else float("nan")
            line["c64"] = {"value": gates * N / (ms64 / 1e3), "ms_per_step": ms64, "compile_ms": c64_compile_ms,
                           "hbm_passes_per_step": len(p64),
                           "roofline": {"bound": "hbm", "achieved": a64, "peak": peak, "unit": "GB/s",
                                        "frac": a64 / peak if d64 else None,
                                        "traffic": 1.012e9 * 2 ** (n - 26), "mean_pass_ms": m64,
                                        "kernel": "qgp_<pass> (specialised tiled pass, complex64)"}}
            accuracy["c64"] = st64.compare(sx)  # the profile run above left the circuit's result
            st64.close()
        sx.close()
        ctx_x.close()
        line["accuracy"] = accuracy
        # the exact FP64 path (every product and sum an IEEE double in the reference's gate
        # order, interpreted tiled passes) on the same circuit, timed once above
        line["exact_fp64"] = {"ms_per_step": accuracy["reference_ms"],
                              "value": gates * N / (accuracy["reference_ms"] / 1e3), "unit": UNIT}
        # the large-n oracle check: 4 layers + QFT at full width on the host's CPU state vector
        try:
            line["oracle_30q"] = oracle_spot_check_30(ctx, n, 4, args.seed + rank, local)
        except Exception as e:  # the line must still print
            line["oracle_30q"] = {"error": f"{type(e).__name__}: {e}"}
        # dense fused blocks of k = 1..5 qubits, per-pass bandwidth on the first two layers of
        # the workload: complex128 blocks compute in FP64 inside tiled passes; complex64 blocks
        # run one HBM pass each on the tensor cores (split-TF32, kind 4 in the profile)
        dense_sample = workloads.layered_circuit(n, 2, args.seed + rank)
        dense = {"sample": f"first 2 layers of layered-{n}x{args.depth} ({len(dense_sample['operations'])} gates)"}
        for dprec in (("c128", "c64") if args.precision == "c128" else ("c64",)):
            rows = {}
            for k in range(1, 6):
                with Context(device=local, workers=1, seed=7, fusion_width=k) as ctx_k:
                    with ctx_k.state(n, dprec) as sk:
                        sk.set_basis(0)
                        sk.apply(dense_sample, fusion="dense")  # warm-up
                        sk.set_basis(0)
                        pk_ms, pk_kind = sk.profile(dense_sample, fusion="dense")
                tiles = [t for t, kk in zip(pk_ms, pk_kind) if kk in (1, 4)]
                ntc = sum(1 for kk in pk_kind if kk == 4)
                bpp = 2 * (16 if dprec == "c128" else 8) * N
                mean_k = statistics.mean(tiles) if tiles else float("nan")
                rows[str(k)] = {"passes": len(pk_ms), "block_passes": len(tiles), "tensor_core_passes": ntc,
                                "total_ms": float(sum(pk_ms)), "mean_block_pass_ms": mean_k,
                                "block_pass_gbs": bpp / (mean_k / 1e3) / 1e9 if tiles else None,
                                "block_pass_frac": bpp / (mean_k / 1e3) / 1e9 / peak if tiles else None}
            dense[dprec] = rows
        line["dense_blocks"] = dense

        # noisy trajectories (the hardware simulator's shot loop): the 10-qubit, 20-layer
        # recipe with depolarizing noise on every gate type and readout errors, as batched
        # device trajectories; shots with equal Kraus choices share one state
        from qclojure_gb300.hardware import run_trajectories

        noisy_c = workloads.layered_circuit(10, 20, args.seed + rank)
        noisy = {"workload": "layered-10x20 (300 gates), depolarizing on every gate, readout 1%/2%"}
        for label, p1, p2 in (("realistic", 0.001, 0.01), ("heavy", 0.02, 0.05)):
            gn = {g: {"noise-type": "depolarizing", "noise-strength": p1} for g in workloads.LAYER_GATES}
            gn["cnot"] = {"noise-type": "depolarizing", "noise-strength": p2}
            nm = {"gate-noise": gn, "readout-error": {"prob-0-to-1": 0.01, "prob-1-to-0": 0.02}}
            shots = 100_000
            run_trajectories(ctx, noisy_c, nm, 1000, seed=1, max_trajectories=0)  # warm-up
            t0 = time.perf_counter()
            run = run_trajectories(ctx, noisy_c, nm, shots, seed=2, max_trajectories=0)
            dt = time.perf_counter() - t0
            noisy[label] = {"depolarizing": [p1, p2], "shots": shots, "shots_per_s": shots / dt, "ms": dt * 1e3,
                            "device_ms": run["stats"]["device-ms"], "distinct_states": run["stats"]["distinct-states"],
                            "noise_sites": run["stats"]["noise-sites"], "batches": run["stats"]["batches"]}
        line["noisy_trajectories"] = noisy

        # variational loop client: Adam with parameter-shift gradients on QAOA MaxCut
        # (20 qubits, p = 3, 6 parameters): each step is one sweep of 13 circuits (the new
        # point and its 12 shifted points); beside it the same step as 13 separate circuits
        try:
            from qclojure_gb300 import variational as V

            vw = workloads.qaoa_maxcut(20, 3, 17)
            vf = lambda prm: V.qaoa_maxcut_circuit(20, vw["edges"], prm)  # noqa: E731
            vp0 = [x for pair in zip(vw["gammas"], vw["betas"]) for x in pair]
            vobj = V.BatchedObjective(ctx, vw["hamiltonian"], vf)
            V.adam_optimization(vobj, vp0, {"learning-rate": 0.02, "max-iterations": 3, "tolerance": 0})  # warm-up
            t0 = time.perf_counter()
            vres = V.adam_optimization(vobj, vp0, {"learning-rate": 0.02, "max-iterations": 21, "tolerance": 0})
            vdt = time.perf_counter() - t0
            vobj.close()
            steps = len(vres["convergence-history"])
            hterms = [(t["coefficient"], t["pauli-string"]) for t in vw["hamiltonian"]]
            t0 = time.perf_counter()
            for prm in [vp0] + V.shifted_points(vp0, V.DEFAULT_SHIFT):
                with ctx.state(20, "c128") as s1:
                    s1.apply(vf(prm))
                    s1.hamiltonian(hterms)
            plain_step = time.perf_counter() - t0
            line["variational"] = {"workload": "Adam, QAOA MaxCut n=20 p=3 (6 parameters), parameter-shift gradients",
                                   "steps": steps, "steps_per_s": steps / vdt, "circuits_per_step": 13,
                                   "energy_first_last": [vres["convergence-history"][0], vres["convergence-history"][-1]],
                                   "plain_step_ms": plain_step * 1e3, "batched_step_ms": vdt / steps * 1e3}
        except Exception as e:  # the line must still print
            line["variational"] = {"error": f"{type(e).__name__}: {e}"}

        # OpenQASM ingestion (host): the 40 random layers of the workload (1800 gates)
        # emitted as OpenQASM 3 and parsed back, then submitted as a job
        from qclojure_gb300 import qasm as Q

        qc = workloads.layered_circuit(n, args.depth, args.seed + rank)
        t0 = time.perf_counter()
        qtext = Q.circuit_to_qasm3(qc)
        t1 = time.perf_counter()
        parsed = Q.qasm3_to_circuit(qtext)
        t2 = time.perf_counter()
        line["qasm"] = {"workload": f"layered-{n}x{args.depth} as OpenQASM 3 ({len(qc['operations'])} gates, "
                                    f"{len(qtext)} bytes)", "emit_ms": (t1 - t0) * 1e3, "parse_ms": (t2 - t1) * 1e3,
                        "gates_per_s": len(qc["operations"]) / (t2 - t1),
                        "round_trip_equal": parsed["operations"] == qc["operations"]}

        # the hardware pipeline's stages (host) on the workload, for a device with the
        # simulator's native gate set
        from qclojure_gb300 import optimization as OPT
        from qclojure_gb300.circuit import NATIVE_SIMULATOR_GATE_SET

        try:
            t0 = time.perf_counter()
            optr = OPT.optimize(circ, {"native-gates": set(NATIVE_SIMULATOR_GATE_SET)})
            line["optimization"] = {"workload": f"layered-{n}x{args.depth}+qft{n} ({gates} gates)",
                                    "ms": (time.perf_counter() - t0) * 1e3,
                                    "gates_after": len(optr["circuit"]["operations"]),
                                    "qubits_after": optr["circuit"]["num-qubits"],
                                    "unsupported_after": optr["final-unsupported-gates"]}
        except Exception as e:  # the line must still print
            line["optimization"] = {"error": f"{type(e).__name__}: {e}"}
        # batched parameter sweep: 1024 QAOA MaxCut circuits (p=3, n uniform over 12..24 even),
        # one launch per pass over all states of a size, replayed from CUDA graphs
        from qclojure_gb300.sweep import Sweep

        st.close()
        qc_list = workloads.qaoa_sweep(1024, 3, seed=7)
        hams = [c["hamiltonian"] for c in qc_list]
        qaoa = {}
        for prec, arith in (("c64", "exact"), ("c128", "double-float")):
            with Sweep(ctx, qc_list, precision=prec, arithmetic=arith) as sw:
                for _ in range(2):
                    sw.run(hams)
                t0 = time.perf_counter()
                reps = 3
                for _ in range(reps):
                    en, sst = sw.run(hams)
                dt = (time.perf_counter() - t0) / reps
                pass_gbs = sst["pass-bytes"] / (sst["device-ms"] / 1e3) / 1e9
                qaoa[prec] = {"circuits_per_s": len(qc_list) / dt, "ms_per_sweep": dt * 1e3,
                              "device_ms": sst["device-ms"], "energy_ms": sst["expect-ms"],
                              "launches": sst["launches"], "graphs": sst["graphs"],
                              "state_gib": sst["state-bytes"] / 2**30,
                              "level_graph_ms": sst["level-graph-ms"], "size_graphs_ms": sst["size-graphs-ms"],
                              "roofline": {"bound": "hbm", "achieved": pass_gbs, "peak": peak, "unit": "GB/s",
                                           "frac": pass_gbs / peak, "pass_bytes": sst["pass-bytes"],
                                           "kernel": "qgl_<level> (sweep level kernels, all sizes per launch)"
                                           if sst["graphs"] == 1 else "qgs_<pass> (table-form pass kernels per size)"}}
        # plain per-circuit complex128 (one HBM pass per gate, one job at a time) on a sample
        sample = qc_list[:48]
        t0 = time.perf_counter()
        for c in sample:
            with ctx.state(c["num-qubits"], "c128") as s1:
                s1.apply(c, fusion="plain")
                s1.hamiltonian([(t["coefficient"], t["pauli-string"]) for t in c["hamiltonian"]])
        dt = time.perf_counter() - t0
        qaoa["plain_c128_per_circuit"] = {"circuits_per_s": len(sample) / dt, "sample": len(sample)}
        qaoa["workload"] = "1024 QAOA MaxCut p=3, random 3-regular graphs, n uniform in {12,...,24}"
        line["qaoa_sweep"] = qaoa

        # end to end through the job API: circuit in, 1024-shot histogram out (host buffers)
        from qclojure_gb300.backend import create_simulator, execute_circuit

        st.close()
        sim = create_simulator({"precision": args.precision, "fusion": args.fusion, "workers": 1, "seed": 5})
        if tuning.get(args.precision, {}).get("chosen"):  # the same kernel shape as the device-timed run
            ch = tuning[args.precision]["chosen"]
            from qclojure_gb300.state import Context as _C
            from qclojure_gb300.backend import _CtxView

            _C.set_tuning(_CtxView(sim._lib, sim._ctx), n, args.precision, ch["tile_bits"], ch["reg_bits"],
                          ch["buffers"], ch["ctas_per_sm"])
        opts = {"result-specs": {"measurements": {"shots": 1024}}}
        execute_circuit(sim, circ, opts, timeout_ms=600_000)
        t0 = time.perf_counter()
        e2e_steps = max(1, min(args.steps, 2))
        for _ in range(e2e_steps):
            r = execute_circuit(sim, circ, opts, timeout_ms=600_000)
            assert r["job-status"] == "completed", r
            sim.free_job(r["job-id"])
        dt = (time.perf_counter() - t0) / e2e_steps
        h2d = enc.count * C.sizeof(A.QgOp)
        line["e2e"] = {"value": gates * N / dt, "unit": UNIT, "h2d_bytes_per_step": h2d,
                       "d2h_bytes_per_step": 1024 * 8 * 2, "ms_per_step": dt * 1e3,
                       "path": "qg_submit -> qg_wait -> qg_result_counts/shots (1024 shots)"}
        sim.close()

        # memory ceiling: 33-qubit complex128 and 34-qubit complex64 (128 GiB each), depth 30 of
        # {H,S,T,RZ} on every qubit + CZ on a random matching, in place, then 10^6 shots
        ceiling = {}
        for cn, cprec in ((33, "c128"), (34, "c64")):
            cc = workloads.ceiling_circuit(cn, 30, seed=args.seed)
            with ctx.state(cn, cprec) as sc:
                cc_compile_ms, _ = sc.prepare(cc, fusion=args.fusion)
                _, scs = sc.device_ptr()
                cstream = torch.cuda.ExternalStream(scs, device=torch.device("cuda", local))
                ca = torch.cuda.Event(enable_timing=True)
                cb = torch.cuda.Event(enable_timing=True)
                ca.record(cstream)
                sc.apply(cc, fusion=args.fusion)
                cb.record(cstream)
                cb.synchronize()
                gms = ca.elapsed_time(cb)
                t0 = time.perf_counter()
                sc.sample(1_000_000, 3)
                sms = (time.perf_counter() - t0) * 1e3
            cg = len(cc["operations"])
            ceiling[cprec] = {"n_qubits": cn, "state_gib": (16 if cprec == "c128" else 8) * 2**cn / 2**30,
                              "gates": cg, "gates_ms": gms, "gate_amps_per_s": cg * 2**cn / (gms / 1e3),
                              "shots": 1_000_000, "shots_ms": sms, "compile_ms": cc_compile_ms}
        ceiling["workload"] = "ceiling: depth 30 of {H,S,T,RZ} + CZ matching, in place, 10^6 shots"
        line["memory_ceiling"] = ceiling
        line["serving"] = serving_leg()
        rate, desc, threads = cpu_reference_rate(n, gates, 8.0)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc}
        line["cpu_baseline"]["optimised_statevector"] = cpu_statevector_rates(args, rank)
        try:
            line["cpu_baseline"]["config0"] = {"reference_algorithm": reference_config0(),
                                               "gpu": gpu_config0(local)}
        except Exception as e:  # the line must still print
            line["cpu_baseline"]["config0"] = {"error": f"{type(e).__name__}: {e}"}
    else:
        st.close()
    ctx.close()
    if rank == 0:
        print(json.dumps(order_line(line)), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
