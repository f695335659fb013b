"""The UnchainedHash-shaped C++ adapter (include/hj_unchained.h): the
reference's build_insert / finalize_build / probe(key, cb) interface over the
GPU table.  The CPU test compiles and links a user of the header; the GPU test
runs it against a brute-force multimap and UnchainedHash's directory words."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CUDA = Path("/usr/local/cuda")


def _build(hj, tmp_path) -> Path:
    exe = tmp_path / "unchained_adapter"
    lib_dir = hj.LIB_PATH.parent
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", str(ROOT / "include"), "-I", str(CUDA / "include"),
           str(ROOT / "tests" / "unchained_adapter.cpp"), "-L", str(lib_dir), "-lhjgb300", f"-Wl,-rpath,{lib_dir}",
           "-L", str(CUDA / "lib64"), "-lcudart", f"-Wl,-rpath,{CUDA / 'lib64'}", "-o", str(exe)]
    out = subprocess.run(cmd, capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    return exe


def test_adapter_compiles_and_links(hj, tmp_path):
    assert _build(hj, tmp_path).exists()


@pytest.mark.gpu
def test_adapter_matches_unchained_semantics(hj, tmp_path):
    exe = _build(hj, tmp_path)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().endswith("ok")
