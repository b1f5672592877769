"""Build the CPU oracle (oracle/qgo.c) into oracle/_build/libqgo.so.

Test infrastructure only: the product library never links it. Compiled with
-ffp-contract=off so every product and sum rounds separately, as the
reference's JVM arithmetic does.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "qgo.c"
OUT = HERE / "_build" / "libqgo.so"


def build_oracle(force: bool = False) -> Path:
    deps = [SRC, HERE.parent / "include" / "qgpu.h", Path(__file__)]
    if not force and OUT.exists() and all(d.stat().st_mtime <= OUT.stat().st_mtime for d in deps):
        return OUT
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    OUT.parent.mkdir(parents=True, exist_ok=True)
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [cc, "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=c11",
           "-D_GNU_SOURCE", str(SRC), "-o", str(tmp), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


SV_SRC = HERE / "cpu_sv.c"
SV_OUT = HERE / "_build" / "libcpusv.so"


def build_cpu_sv(force: bool = False):
    """The optimised CPU state-vector baseline (cpu_sv.c, with qgo.c for the gate
    matrices) as oracle/_build/libcpusv.so, with OpenMP where the compiler has it.
    Returns None when it cannot be built: it only feeds a benchmark figure."""
    deps = [SV_SRC, SRC, HERE.parent / "include" / "qgpu.h", Path(__file__)]
    if not force and SV_OUT.exists() and all(d.stat().st_mtime <= SV_OUT.stat().st_mtime for d in deps):
        return SV_OUT
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    SV_OUT.parent.mkdir(parents=True, exist_ok=True)
    tmp = SV_OUT.with_suffix(".so.tmp")
    for omp in (["-fopenmp"], []):
        cmd = [cc, "-O3", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=c11", "-D_GNU_SOURCE",
               *omp, str(SRC), str(SV_SRC), "-o", str(tmp), "-lm"]
        if subprocess.run(cmd, capture_output=True, text=True).returncode == 0:
            os.replace(tmp, SV_OUT)
            return SV_OUT
    return None


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
