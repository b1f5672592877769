"""Build libqgpu.so (sm_103a) in-tree with nvcc.

The library is compiled from qclojure_gb300/csrc/*.{cu,cpp} into
qclojure_gb300/_lib/libqgpu.so. Translation units compile in parallel; the
build is skipped when the library is newer than every source.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_lib"
LIB = OUT_DIR / "libqgpu.so"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libqgpu.so")


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


EMBEDDED = {"kEmbedPassPrelude": "pass_prelude.cuh", "kEmbedDf64": "df64.cuh"}


def write_embedded(obj_dir: Path) -> Path:
    """The device prelude of the specialised pass kernels, as C strings: NVRTC
    compiles it at run time together with each program's generated passes."""
    out = obj_dir / "embedded_sources.cpp"
    parts = ["// generated by qclojure_gb300/build.py from csrc/*.cuh\nnamespace qg {\n"]
    for sym, name in EMBEDDED.items():
        text = (CSRC / name).read_text()
        assert ")QGEMBED" not in text
        parts.append(f'extern const char {sym}[] = R"QGEMBED({text})QGEMBED";\n')
    parts.append("}  // namespace qg\n")
    body = "".join(parts)
    if not out.exists() or out.read_text() != body:
        out.write_text(body)
    return out


def build_library(force: bool = False, verbose: bool = False) -> Path:
    srcs = sources()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    if not force and not _stale(LIB, srcs + headers + [Path(__file__)]):
        return LIB
    nvcc = nvcc_path()
    obj_dir = OUT_DIR / "obj"
    obj_dir.mkdir(parents=True, exist_ok=True)
    srcs = srcs + [write_embedded(obj_dir)]
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(INCLUDE), "-lineinfo"]

    def compile_one(src: Path) -> Path:
        obj = obj_dir / (src.name + ".o")
        if src.suffix == ".cu":
            cmd = [nvcc, *ARCH, *common, "-Xptxas", "-warn-spills", "-c", str(src), "-o", str(obj)]
        else:
            cmd = [nvcc, *common, "-x", "c++", "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 2))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose=True))
