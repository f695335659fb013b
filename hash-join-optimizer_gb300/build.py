"""Builds libhjgb300.so (CUDA kernels for sm_103a + host runtime + C ABI).

Every translation unit compiles in parallel into _build/; the shared library
lands next to this file.  Run directly (`python build.py [-v]`) or through
`__graft_entry__.build()`.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
LIB = HERE / "libhjgb300.so"

CUDA_SOURCES = ["hj_scan.cu", "hj_decode.cu", "hj_build.cu", "hj_probe.cu",
                "hj_materialize.cu", "hj_transfer.cu", "hj_engine.cu", "hj_noalloc.cu",
                "hj_batch.cu", "hj_serve.cu", "hj_filter.cu"]
CXX_SOURCES = ["hj_pages_host.cpp", "contest.cpp", "hj_cache.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libhjgb300.so")


def _run(cmd: list[str]) -> str:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout + proc.stderr)
    return proc.stdout + proc.stderr


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((HERE.parent / "include").glob("*.h"))
    jobs = []
    for src in CUDA_SOURCES:
        obj = BUILD / (src + ".o")
        if _stale(obj, [CSRC / src] + headers) or ptxas_info:
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-Xcompiler", "-O3", "--expt-relaxed-constexpr", "-c", str(CSRC / src), "-o", str(obj)]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for src in CXX_SOURCES:
        obj = BUILD / (src + ".o")
        if _stale(obj, [CSRC / src] + headers):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-Wall", "-c", str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    objs = [str(BUILD / (s + ".o")) for s in CUDA_SOURCES + CXX_SOURCES]
    if _stale(LIB, [Path(o) for o in objs]):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *objs, "-lpthread"])
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
