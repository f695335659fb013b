"""The C++ drop-in boundary: a harness written against include/plan.h links
libhjgb300.so and runs the reference's unit-test plans through
Contest::build_context / execute / destroy_context."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _build(hj, tmp_path) -> Path:
    exe = tmp_path / "contest_harness"
    lib_dir = hj.LIB_PATH.parent
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"), str(ROOT / "tests" / "contest_harness.cpp"),
                    "-L", str(lib_dir), "-lhjgb300", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], check=True)
    return exe


def test_harness_compiles_against_plan_h(hj, tmp_path):
    assert _build(hj, tmp_path).exists()


@pytest.mark.gpu
def test_contest_execute_runs_reference_unit_tests(hj, tmp_path):
    exe = _build(hj, tmp_path)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().endswith("ok")
